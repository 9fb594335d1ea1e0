"""Failure detection on the GPU without a fault: the staged PCG's bounded waits run out.

Every wait inside the staged PCG kernels (a shared-memory stage's mbarrier, the grid
barrier of the one-launch PCG) polls a bounded number of times.  With the bound set to 0
through symxg_set_wait_poll_limit every such wait gives up at once: the kernels stop their
work, drain their own bulk copies with the default bound, flag the solve, and return, so the
call fails with SYMXG_ERR_RUNTIME.  The test then restores the bound and checks that the same
handle (the same CUDA context) solves the step normally: no trap, no hang, no lost context.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg(lib):
    import symx_gb300

    return symx_gb300


@pytest.mark.parametrize("case", ["tet4_6p", "hex8_3"])
def test_bounded_wait_gives_up_and_context_stays_usable(sg, case):
    from symx_gb300 import problems

    L = sg.load()
    p = problems.step_problem(case)
    s = sg.ElasticSolver(p)
    s.set_settings(cg_rel_tolerance=1e-3, precision="mixed")
    s.set_state(p["x_init"], p["x0"], p["v0"])
    ref = s.solve()
    x_ref = s.get_positions()
    assert ref["solver_return"] == 0
    assert L.symxg_wait_poll_limit() == 1 << 22
    L.symxg_set_wait_poll_limit(0)
    try:
        assert L.symxg_wait_poll_limit() == 0
        s.set_state(p["x_init"], p["x0"], p["v0"])
        with pytest.raises(sg.SymxgError, match="bounded wait"):
            s.solve()
    finally:
        L.symxg_set_wait_poll_limit(-1)
    assert L.symxg_wait_poll_limit() == 1 << 22
    # the same handle, after the failed call: same Newton and CG counts, same positions
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st = s.solve()
    assert st["solver_return"] == 0
    assert st["newton_iterations"] == ref["newton_iterations"]
    assert st["cg_iterations"] == ref["cg_iterations"]
    assert np.array_equal(s.get_positions(), x_ref)
