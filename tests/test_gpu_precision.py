"""The FP64 parts of the mixed-precision split, on the GPU.

* FP64-accurate projection (projection_fp64_refinement): an FP32 cyclic Jacobi refined by
  one FP64 Ogita-Aishima step, the clamping applied as an FP64 correction.  On the FP32
  element Hessians of the mixed path its result must equal an FP64 eigen-projection of the
  same FP32 matrices up to the final rounding to float (tolerance 2e-7 of max |H|; the FP32
  Jacobi alone is off by ~1e-6).  In the FP64 path it must match the reference's projected
  Hessians as the pure FP64 Jacobi does (1e-9 of max |H|).
* FP64 residual replacement in the FP32 PCG (cg_residual_replacement): the solve with both
  converges to the reference's positions within 1e-6 of the displacement, with the same
  Newton iterations, and reports its replacements.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg(lib):
    import symx_gb300

    return symx_gb300


def make(sg, case, precision, **kw):
    from symx_gb300 import problems

    p = problems.step_problem(case)
    s = sg.ElasticSolver(p)
    s.set_settings(cg_rel_tolerance=1e-3, precision=precision, **kw)
    s.set_state(p["x_init"], p["x0"], p["v0"])
    return p, s


def helmert_q(nb=4):
    B = np.zeros((nb, nb - 1))
    for m in range(1, nb):
        c = 1.0 / np.sqrt(m * (m + 1))
        B[:m, m - 1] = c
        B[m, m - 1] = -m * c
    return np.kron(B, np.eye(3))


def fp64_deflated_projection(H, eps=1e-10):
    """FP64 eigen-projection of translation-invariant 12 x 12 matrices in the complement of
    the translations, plus the translation eigenvalues 0 -> eps (numpy eigh)."""
    Q = helmert_q()
    out = np.empty_like(H)
    T = (eps / 4.0) * np.kron(np.ones((4, 4)), np.eye(3))
    for e, h in enumerate(H):
        A = Q.T @ h @ Q
        w, V = np.linalg.eigh(A)
        dw = np.where(w < eps, eps - w, 0.0)
        out[e] = h + Q @ ((V * dw) @ V.T) @ Q.T + T
    return out


@pytest.mark.parametrize("case", ["tet4_6p", "tet4_5c"])
def test_refined_projection_is_fp64_accurate_on_fp32_hessians(sg, case):
    p, s = make(sg, case, "mixed")
    _, _, H = s.element_outputs(0, project=False)  # the FP32 element Hessians
    _, _, H32 = s.element_outputs(0, project=True)  # FP32 Jacobi
    s.set_settings(projection_fp64_refinement=1)
    _, _, Hr = s.element_outputs(0, project=True)  # FP32 Jacobi + FP64 refinement
    ref = fp64_deflated_projection(H)
    scale = np.max(np.abs(ref))
    err_refined = np.max(np.abs(Hr - ref)) / scale
    err_fp32 = np.max(np.abs(H32 - ref)) / scale
    print(f"{case}: refined {err_refined:.2e}, FP32 Jacobi {err_fp32:.2e} of max |H|")
    assert err_refined <= 2e-7
    # symmetric to the last bit
    assert np.array_equal(Hr, np.transpose(Hr, (0, 2, 1)))


@pytest.mark.parametrize("case", ["tet4_3", "tet4_6p"])
def test_refined_projection_fp64_matches_reference(sg, golden, case):
    p, s = make(sg, case, "fp64", projection_fp64_refinement=1)
    ev = golden(f"{case}_eval")
    _, _, Hp = s.element_outputs(0, project=True)
    ref = ev["hess_sample_projected"]
    assert np.max(np.abs(Hp[ev["hess_sample_idx"]] - ref)) <= 1e-9 * np.max(np.abs(ref))


@pytest.mark.parametrize("case", ["tet4_6p", "tet4_10", "tet4_5c"])
def test_newton_fp64_refined_projection_matches_reference(sg, golden, case):
    p, s = make(sg, case, "fp64", projection_fp64_refinement=1)
    st = s.solve()
    sol = golden(f"{case}_solve") if case != "tet4_5c" else None
    assert st["solver_return"] == 0 and st["final_residual"] < 1e-6
    if sol is not None:
        assert st["newton_iterations"] == int(sol["newton_iterations_full"])
        assert abs(st["cg_iterations"] - int(sol["cg_iterations_full"])) <= 2 + 0.02 * int(sol["cg_iterations_full"])
        x, xr = s.get_positions(), sol["x_full"]
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr - p["x0"]) < 1e-8


@pytest.mark.parametrize("case", ["tet4_6p", "tet4_10"])
def test_newton_mixed_fp64_split_matches_reference(sg, golden, case):
    """Mixed precision with the FP64-accurate projection, an FP64 residual replacement every 10
    PCG iterations and FP64 sums of the PCG's dot-product partials."""
    p, s = make(sg, case, "mixed", projection_fp64_refinement=1, cg_residual_replacement=10, cg_fp64_partial_sums=1)
    st = s.solve()
    sol = golden(f"{case}_solve")
    assert st["solver_return"] == 0 and st["final_residual"] < 1e-6
    assert st["newton_iterations"] == int(sol["newton_iterations_full"])
    assert st["cg_residual_replacements"] > 0
    assert abs(st["cg_iterations"] - int(sol["cg_iterations_full"])) <= 2 + 0.05 * int(sol["cg_iterations_full"])
    x, xr = s.get_positions(), sol["x_full"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr - p["x0"]) < 1e-6


def test_fp64_partial_sums_are_deterministic(sg):
    p, s = make(sg, "tet4_10", "mixed", cg_fp64_partial_sums=1)
    st1 = s.solve()
    x1 = s.get_positions()
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st2 = s.solve()
    assert st1["cg_iterations"] == st2["cg_iterations"] and np.array_equal(x1, s.get_positions())


def test_residual_replacement_keeps_the_iteration(sg):
    """The replacement only swaps the recursive residual for the true one: CG counts within
    5 % of the solve without it, and the same converged positions to the solve tolerance."""
    p, s = make(sg, "tet4_10", "mixed")
    st0 = s.solve()
    x0 = s.get_positions()
    s.set_settings(cg_residual_replacement=5)
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st1 = s.solve()
    assert st1["solver_return"] == 0 and st1["cg_residual_replacements"] >= st1["cg_iterations"] // 5 - st1["newton_iterations"]
    assert abs(st1["cg_iterations"] - st0["cg_iterations"]) <= 2 + 0.05 * st0["cg_iterations"]
    assert np.linalg.norm(s.get_positions() - x0) / np.linalg.norm(x0 - p["x0"]) < 1e-6
