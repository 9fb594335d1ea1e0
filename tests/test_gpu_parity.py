"""GPU parity of the CUDA solve path against the oracle and the reference's golden outputs.

Every call goes through the C ABI (libsymxg.so).  Tolerances:
  FP64 path   energy 1e-12 rel, gradient 1e-9 of max |g|, element Hessians 1e-10 of max |H|,
              projected Hessians 1e-9 of max |H|, final positions 1e-8 of |x - x0|.
  Mixed path  element Hessians 1e-5 of max |H| (float storage), final positions 1e-6 rel and
              1e-6 of |x - x0|.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = ["tet4_3", "tet4_6p", "hex8_3", "tet4_10", "tet10_2"]


@pytest.fixture(scope="module")
def sg(lib):
    import symx_gb300

    return symx_gb300


def make(sg, case, precision="fp64"):
    from symx_gb300 import problems

    p = problems.step_problem(case)
    s = sg.ElasticSolver(p)
    s.set_settings(cg_rel_tolerance=1e-3, precision=precision)
    s.set_state(p["x_init"], p["x0"], p["v0"])
    return p, s


@pytest.mark.parametrize("case", CASES)
def test_energy_gradient_match_reference(sg, golden, case):
    p, s = make(sg, case)
    ev = golden(f"{case}_eval")
    E, g = s.evaluate()
    assert abs(E - ev["E"]) <= 1e-12 * abs(ev["E"])
    assert np.max(np.abs(g - ev["grad"])) <= 1e-9 * np.max(np.abs(ev["grad"]))
    assert abs(s.evaluate_energy() - ev["E_only"]) <= 1e-12 * abs(ev["E_only"])


@pytest.mark.parametrize("case", ["tet4_3", "hex8_3", "tet4_6p", "tet10_2"])
def test_element_outputs_match_oracle(sg, golden, case):
    from oracle import oracle as O

    p, s = make(sg, case)
    E, g, H = s.element_outputs(0, project=False)
    nodes = p["conn"].shape[1]
    xe = p["x_init"][p["conn"]]
    Xe = p["X"][p["conn"]]
    E_o, g_o, H_o = O.nh_element_batch(xe, Xe, p["mu"], p["lam"])
    # at rest E and g are roundoff around zero: scale them by the element's stiffness
    h = 0.01
    scale_H = np.max(np.abs(H_o))
    assert np.max(np.abs(H - H_o)) <= 1e-10 * scale_H
    assert np.max(np.abs(g - g_o)) <= 1e-10 * max(np.max(np.abs(g_o)), scale_H * h)
    assert np.max(np.abs(E - E_o)) <= 1e-11 * max(np.max(np.abs(E_o)), scale_H * h * h)
    # projected element Hessians against the reference's project_to_PD_inplace
    ev = golden(f"{case}_eval")
    _, _, Hp = s.element_outputs(0, project=True)
    idx = ev["hess_sample_idx"]
    ref = ev["hess_sample_projected"]
    assert np.max(np.abs(Hp[idx] - ref)) <= 1e-9 * np.max(np.abs(ref))
    assert nodes in (4, 8, 10)


@pytest.mark.parametrize("case", CASES)
def test_assembled_hessian_matches_reference(sg, golden, case):
    from oracle import oracle as O

    p, s = make(sg, case)
    ev = golden(f"{case}_eval")
    rp, cols, vals = s.assembled_hessian(project=True)
    A = O.bcsr_to_scipy(rp, cols, vals)
    assert A.nnz == int(ev["nnz"])
    for v, ref in zip(ev["probe_vectors"], ev["probe_products"]):
        y = A @ v
        # the penalty rows dominate the scale; compare the elastic part separately too
        assert np.max(np.abs(y - ref)) <= 1e-10 * np.max(np.abs(ref))
    free = np.setdiff1d(np.arange(p["X"].shape[0]), p["bc_idx"])
    rows = (3 * free[:, None] + np.arange(3)).ravel()
    for v, ref in zip(ev["probe_vectors"], ev["probe_products"]):
        y = A @ v
        assert np.max(np.abs(y[rows] - ref[rows])) <= 1e-9 * np.max(np.abs(ref[rows]))
    if "triplet_idx" in ev.files:
        import scipy.sparse as sp

        ti, tv = ev["triplet_idx"], ev["triplet_val"]
        R = sp.coo_matrix((tv, (ti[:, 0], ti[:, 1])), shape=A.shape).tocsr()
        D = (A - R).tocoo()
        scale = np.max(np.abs(R[rows][:, rows].data))
        dd = (A - R)[rows][:, rows]
        assert np.max(np.abs(dd.data), initial=0.0) <= 1e-9 * scale
        assert np.max(np.abs(D.data), initial=0.0) <= 1e-9 * np.max(np.abs(R.data))


@pytest.mark.parametrize("case", CASES)
def test_newton_fp64_matches_reference(sg, golden, case):
    p, s = make(sg, case)
    st = s.solve()
    sol = golden(f"{case}_solve")
    assert st["solver_return"] == 0
    assert st["final_residual"] < 1e-6
    assert st["newton_iterations"] == int(sol["newton_iterations_full"])
    assert abs(st["cg_iterations"] - int(sol["cg_iterations_full"])) <= 2 + 0.02 * int(sol["cg_iterations_full"])
    x, xr = s.get_positions(), sol["x_full"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr - p["x0"]) < 1e-8
    # a single Newton iteration reproduces the reference's first step too
    s.set_settings(max_iterations=1, max_iterations_as_success=1)
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st1 = s.solve()
    x1, xr1 = s.get_positions(), sol["x_it1"]
    assert st1["solver_return"] == 0
    assert np.linalg.norm(x1 - xr1) / np.linalg.norm(xr1 - p["x0"]) < 1e-8


@pytest.mark.parametrize("case", CASES)
def test_newton_mixed_converges_to_fp64_solution(sg, golden, case):
    p, s = make(sg, case, precision="mixed")
    st = s.solve()
    sol = golden(f"{case}_solve")
    assert st["solver_return"] == 0
    assert st["final_residual"] < 1e-6
    x, xr = s.get_positions(), sol["x_full"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-6
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr - p["x0"]) < 1e-6


MODES = {0: "newton", 1: "projected", 2: "on_demand", 3: "progressive"}


@pytest.mark.parametrize("mode", sorted(MODES))
def test_projection_modes_fp64_match_reference(sg, golden, mode):
    """Every ProjectionToPD mode from an indefinite start (tet4_5c: the Newton guess squeezed
    to half height), FP64, against the reference: the same return code, Newton iterations and
    Hessian / projected-Hessian counts, CG iterations within 3 %, positions within 1e-8 of the
    displacement (plain Newton fails with LinearSystemSolveFailure in its second iteration,
    as the reference does)."""
    p, s = make(sg, "tet4_5c")
    s.set_settings(project_to_pd=mode)
    st = s.solve()
    d, tag = golden("tet4_5c_modes"), MODES[mode]
    assert st["solver_return"] == int(d[f"return_{tag}"])
    for k in ("newton_iterations", "n_hessians", "n_projected_hessians"):
        assert st[k] == int(d[f"{k}_{tag}"]), (k, st[k], int(d[f"{k}_{tag}"]))
    cg = int(d[f"cg_iterations_{tag}"])
    assert abs(st["cg_iterations"] - cg) <= 2 + 0.03 * cg
    x, xr = s.get_positions(), d[f"x_{tag}"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr - p["x0"]) < 1e-8


@pytest.mark.parametrize("mode", [2, 3])
def test_projection_modes_mixed_converge(sg, golden, mode):
    """The adaptive modes in mixed precision: converged, fewer Hessians projected than
    evaluated, positions within 1e-6 relative of the reference's solution in that mode."""
    p, s = make(sg, "tet4_5c", precision="mixed")
    s.set_settings(project_to_pd=mode)
    st = s.solve()
    assert st["solver_return"] == 0 and st["final_residual"] < 1e-6
    assert 0 < st["n_projected_hessians"] < st["n_hessians"]
    x, xr = s.get_positions(), golden("tet4_5c_modes")[f"x_{MODES[mode]}"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-6


def test_unknown_projection_mode_rejected(sg):
    from symx_gb300.capi import SymxgError

    _, s = make(sg, "tet4_3")
    with pytest.raises(SymxgError, match="projection mode"):
        s.set_settings(project_to_pd=4)


@pytest.mark.parametrize("case", ["tet4_6p", "hex8_3", "tet10_2"])
def test_mixed_element_hessians_within_float_tolerance(sg, case):
    """FP32 element Hessians of the mixed path against the FP64 path (Hex8: summed over the
    eight quadrature points by the lanes that evaluate them)."""
    p, s = make(sg, case, precision="mixed")
    _, _, H32 = s.element_outputs(0, project=False)
    s.set_settings(precision="fp64")
    _, _, H64 = s.element_outputs(0, project=False)
    assert np.max(np.abs(H32 - H64)) <= 1e-5 * np.max(np.abs(H64))


@pytest.mark.parametrize("case", ["tet4_6p", "hex8_3"])
def test_mixed_energy_gradient_double_float_accuracy(sg, case):
    """The mixed path evaluates element energies and gradients in double-float (about 48
    significant bits): within 1e-12 of the FP64 path, element by element; the line-search
    energy (its own kernel) likewise."""
    from symx_gb300 import problems

    p, s = make(sg, case, precision="mixed")
    # a deformed state (at rest the element energies are rounding noise around zero)
    x = p["X"] + 5e-4 * problems.normal(26, p["X"].size).reshape(-1, 3)
    s.set_state(x, p["x0"], p["v0"])
    E32, g32, _ = s.element_outputs(0, project=False)
    s.set_settings(precision="fp64")
    E64, g64, _ = s.element_outputs(0, project=False)
    assert np.max(np.abs(E32 - E64)) <= 1e-12 * np.max(np.abs(E64))
    assert np.max(np.abs(g32 - g64)) <= 1e-12 * np.max(np.abs(g64))
    # whole solves: the mixed solve still lands on the FP64 solution
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st64 = s.solve()
    x64 = s.get_positions()
    s.set_settings(precision="mixed")
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st32 = s.solve()
    assert st32["solver_return"] == 0 and st64["solver_return"] == 0
    assert np.max(np.abs(s.get_positions() - x64)) <= 1e-6 * np.max(np.abs(x64 - p["x0"]))


@pytest.mark.parametrize("dtype,tol", [("float64", 1e-9), ("float32", 1e-4)])
def test_project_pd_kernel_matches_reference(sg, golden, dtype, tol):
    import torch

    for name in ("project12", "project24"):
        d = golden(name)
        H = torch.tensor(d["inputs"], dtype=getattr(torch, dtype), device="cuda")
        nc = sg.project_pd(H)
        out = H.double().cpu().numpy()
        for i in range(out.shape[0]):
            scale = np.max(np.abs(d["inputs"][i]))
            assert np.max(np.abs(out[i] - d["outputs"][i])) <= tol * scale, (name, i)
        assert not nc


def test_project_pd_edge_cases(sg):
    import torch

    # already positive definite: untouched; zero matrix: all eigenvalues clamped to eps
    A = torch.eye(12, dtype=torch.float64, device="cuda").repeat(3, 1, 1)
    A[1] *= 5.0
    A[2].zero_()
    ref = A.clone()
    sg.project_pd(A)
    assert torch.equal(A[0], ref[0]) and torch.equal(A[1], ref[1])
    assert torch.allclose(A[2], 1e-10 * torch.eye(12, dtype=torch.float64, device="cuda"))
    # empty batch
    E = torch.zeros((0, 12, 12), dtype=torch.float32, device="cuda")
    sg.project_pd(E)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_bcsr_spmv_kernel(sg, dtype):
    import torch

    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.step_problem("tet4_6p")
    ref = O.Problem(p, 1)
    rp, cols, vals, _ = ref.assemble(True)
    A = O.bcsr_to_scipy(rp, cols, vals)
    x = problems.normal(5, A.shape[0])
    t = getattr(torch, dtype)
    y = torch.zeros(A.shape[0], dtype=t, device="cuda")
    sg.bcsr_spmv(torch.tensor(rp, device="cuda"), torch.tensor(cols, device="cuda"),
                 sg.component_major(torch.tensor(vals, dtype=t, device="cuda")), torch.tensor(x, dtype=t, device="cuda"), y)
    tol = 1e-12 if dtype == "float64" else 1e-5
    yr = A @ x
    assert np.max(np.abs(y.double().cpu().numpy() - yr)) <= tol * np.max(np.abs(yr))


def test_deterministic_repeat(sg):
    p, s = make(sg, "tet4_6p", precision="mixed")
    s.solve()
    x1 = s.get_positions()
    s.set_state(p["x_init"], p["x0"], p["v0"])
    s.solve()
    assert np.array_equal(x1, s.get_positions())


def test_failure_modes_return_codes(sg):
    # PCG capped at one iteration cannot reach the forcing tolerance: linear-solve failure
    p, s = make(sg, "tet4_10")
    s.set_settings(cg_max_iterations=1)
    st = s.solve()
    assert st["solver_return_name"] == "LinearSystemSolveFailure"
    # an unreachable Armijo condition exhausts the backtracking budget
    p, s = make(sg, "tet4_3")
    s.set_settings(line_search_armijo_beta=1e6, max_backtracking_armijo_iterations=3)
    st = s.solve()
    assert st["solver_return_name"] == "TooManyArmijoIterations"
    # max_iterations without success flag
    p, s = make(sg, "tet4_3")
    s.set_settings(max_iterations=1)
    st = s.solve()
    assert st["solver_return_name"] == "TooManyIterations"


def test_inverted_initial_element_is_rejected_by_line_search(sg):
    # an inverted element makes E = +inf (log guard): the first evaluation is not finite and
    # the solver reports failure instead of returning garbage
    p, s = make(sg, "tet4_3")
    x = p["x_init"].copy()
    t = p["conn"][5]
    x[t[0]], x[t[1]] = x[t[1]].copy(), x[t[0]].copy()
    s.set_state(x, p["x0"], p["v0"])
    E, _ = s.evaluate()
    assert np.isinf(E) and E > 0
    st = s.solve()
    assert st["solver_return"] != 0


def test_fp32_tet4_hessians_take_the_deflated_projection(sg):
    """The mixed path projects 12x12 element Hessians in the complement of the rigid
    translations when their translation residual is below 1e-5 of max |H|; the FP32
    Neo-Hookean Hessians from the generated kernels should (nearly) all qualify."""
    p, s = make(sg, "tet4_10", precision="mixed")
    _, _, H = s.element_outputs(0, project=False)
    res = np.abs(H.reshape(-1, 12, 4, 3).sum(axis=2)).max(axis=(1, 2))
    hmax = np.abs(H).max(axis=(1, 2))
    assert np.mean(res <= 1e-5 * hmax) >= 0.99


def test_newton_fp64_on_reference_numbered_mesh_matches_oracle(sg):
    """The step on generate_cuboid_Tet4_mesh's own numbering (reverse Cuthill-McKee nodes,
    reordered elements): FP64 GPU solve against the oracle on the same arrays, same Newton and
    CG iteration counts and positions within 1e-8 of |x - x0|."""
    from oracle import oracle as O

    p, s = make(sg, "tet4_6p_rcm")
    st = s.solve()
    P = O.Problem(p, 1)
    P.set_x(p["x_init"])
    so = P.solve(O.default_settings(cg_rel_tolerance=1e-3))
    assert st["solver_return"] == 0 and so["solver_return"] == 0
    assert st["newton_iterations"] == so["newton_iterations"]
    assert st["cg_iterations"] == so["cg_iterations"]
    x, xo = s.get_positions(), P.get_x()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo - p["x0"]) < 1e-8
