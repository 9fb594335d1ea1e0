"""Stand-alone block-Jacobi PCG (symxg_bcsr_pcg_*) against the oracle's restatement of
bsm::solve_pcg on assembled, projected Hessians of the step problems.

Tolerances: f64  iteration count equal to the oracle's, solution within 1e-9 of max |x|;
            f32  true residual |b - A x| / |b| (computed in float64) below 10 x rel_tol.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg(lib):
    import symx_gb300

    return symx_gb300


def system(case, seed=11):
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.step_problem(case)
    rp, cols, vals, _ = O.Problem(p, 1).assemble(True)
    b = problems.normal(seed, 3 * (rp.size - 1))
    return rp, cols, vals, b


def gpu_solve(sg, rp, cols, vals, b, dtype, **kw):
    import torch

    t = getattr(torch, dtype)
    x = torch.full((b.size,), float("nan"), dtype=t, device="cuda")
    info = sg.bcsr_pcg(torch.tensor(rp, device="cuda"), torch.tensor(cols, device="cuda"),
                       sg.component_major(torch.tensor(vals, dtype=t, device="cuda")),
                       torch.tensor(b, dtype=t, device="cuda"), x, **kw)
    torch.cuda.synchronize()
    return x.double().cpu().numpy(), info


@pytest.mark.parametrize("case", ["tet4_6p", "hex8_3", "tet4_10"])
def test_pcg_f64_matches_oracle(sg, case):
    from oracle import oracle as O

    rp, cols, vals, b = system(case)
    xo, it_o, conv_o = O.bcsr_pcg(rp, cols, vals, b, 1e-12, 1e-8, 2000)
    x, info = gpu_solve(sg, rp, cols, vals, b, "float64", abs_tol=1e-12, rel_tol=1e-8, max_iterations=2000)
    assert conv_o and info["converged"] == 1
    assert info["n_iterations"] == it_o
    assert np.max(np.abs(x - xo)) <= 1e-9 * np.max(np.abs(xo))


@pytest.mark.parametrize("case", ["tet4_6p", "tet4_10"])
def test_pcg_f32_true_residual(sg, case):
    from oracle import oracle as O

    rp, cols, vals, b = system(case)
    A = O.bcsr_to_scipy(rp, cols, vals)
    x, info = gpu_solve(sg, rp, cols, vals, b, "float32", abs_tol=1e-12, rel_tol=1e-5, max_iterations=2000)
    assert info["converged"] == 1 and info["found_indefiniteness"] == 0
    assert np.linalg.norm(b - A @ x) <= 10 * 1e-5 * np.linalg.norm(b)
    _, it_o, _ = O.bcsr_pcg(rp, cols, vals, b, 1e-12, 1e-5, 2000)
    assert abs(info["n_iterations"] - it_o) <= max(2, it_o // 10)


def test_pcg_repeat_is_deterministic(sg):
    rp, cols, vals, b = system("tet4_10")
    x1, i1 = gpu_solve(sg, rp, cols, vals, b, "float32", rel_tol=1e-4)
    x2, i2 = gpu_solve(sg, rp, cols, vals, b, "float32", rel_tol=1e-4)
    assert i1 == i2 and np.array_equal(x1, x2)


def test_pcg_edge_cases(sg):
    import torch

    from symx_gb300.capi import SymxgError

    rp, cols, vals, b = system("tet4_6p")
    # zero right-hand side: x = 0 after no iteration (solve_pcg.h:115-122)
    x, info = gpu_solve(sg, rp, cols, vals, np.zeros_like(b), "float64")
    assert info["converged"] == 1 and info["n_iterations"] == 0 and not np.any(x)
    # iteration cap
    _, info = gpu_solve(sg, rp, cols, vals, b, "float64", rel_tol=1e-12, abs_tol=0.0, max_iterations=1)
    assert info["converged"] == 0 and info["n_iterations"] == 1
    # negative definite: stops on p.Ap <= 0 in the first iteration
    _, info = gpu_solve(sg, rp, cols, -vals, b, "float64")
    assert info["converged"] == 0 and info["found_indefiniteness"] == 1 and info["n_iterations"] == 1
    # a row without its diagonal block is refused
    keep = np.ones(cols.size, dtype=bool)
    keep[np.flatnonzero(cols[rp[0]:rp[1]] == 0)[0] + rp[0]] = False
    rp2 = rp.copy()
    rp2[1:] -= 1
    with pytest.raises(SymxgError, match="diagonal"):
        gpu_solve(sg, rp2, cols[keep], vals[keep], b, "float64")
    # a values stride below the block count is refused before any kernel reads a value
    import ctypes as C

    from symx_gb300 import capi

    L = sg.load()
    d_rp, d_cols = torch.tensor(rp, device="cuda"), torch.tensor(cols, device="cuda")
    d_vals = sg.component_major(torch.tensor(vals, dtype=torch.float64, device="cuda"))
    d_b = torch.tensor(b, device="cuda")
    d_x = torch.zeros_like(d_b)
    pinfo = capi.PcgInfo()
    rc = L.symxg_bcsr_pcg_f64(rp.size - 1, C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_cols.data_ptr()),
                              C.c_void_p(d_vals.data_ptr()), cols.size - 1, C.c_void_p(d_b.data_ptr()),
                              C.c_void_p(d_x.data_ptr()), 1e-10, 1e-6, 100, C.byref(pinfo), None)
    assert rc == 1 and "vals_stride" in L.symxg_last_error().decode()
    # empty system
    t = torch.zeros(0, dtype=torch.float32, device="cuda")
    info = sg.bcsr_pcg(torch.zeros(1, dtype=torch.int32, device="cuda"), torch.zeros(0, dtype=torch.int32, device="cuda"),
                       torch.zeros(9, 0, dtype=torch.float32, device="cuda"), t, t)
    assert info["converged"] == 1 and info["n_iterations"] == 0
