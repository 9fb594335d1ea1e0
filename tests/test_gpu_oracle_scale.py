"""At-scale parity of the Newton step against the oracle's complete FP64 solve.

tet4_32p is the metric's configuration (seeded 5 % spacing perturbation of the initial
positions, v0 ~ N(0, 0.5^2), E = 1e5, nu = 0.3, clamped x = 0 face) at 32^3 cells:
35,937 vertices, 196,608 tets, small enough for the oracle's complete solve to take seconds.
Tolerances (of the step's displacement |x_oracle - x0|):
  FP64   same Newton iterations, CG within 2 %, positions within 1e-8.
  mixed  converged (max |grad E| < 1e-6), positions within 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_solution():
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.step_problem("tet4_32p")
    P = O.Problem(p, 0)
    P.set_x(p["x_init"])
    st = P.solve(O.default_settings(cg_rel_tolerance=1e-3))
    assert st["solver_return"] == 0
    return p, st, P.get_x()


@pytest.fixture(scope="module")
def sg(lib):
    import symx_gb300

    return symx_gb300


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_step_at_scale_matches_oracle(sg, oracle_solution, precision):
    p, st_o, x_o = oracle_solution
    s = sg.ElasticSolver(p)
    s.set_settings(cg_rel_tolerance=1e-3, precision=precision)
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st = s.solve()
    assert st["solver_return"] == 0
    assert st["final_residual"] < 1e-6
    x = s.get_positions()
    err = np.linalg.norm(x - x_o) / np.linalg.norm(x_o - p["x0"])
    if precision == "fp64":
        assert st["newton_iterations"] == st_o["newton_iterations"]
        assert abs(st["cg_iterations"] - st_o["cg_iterations"]) <= 2 + 0.02 * st_o["cg_iterations"]
        assert err < 1e-8, err
    else:
        assert err < 1e-6, err
