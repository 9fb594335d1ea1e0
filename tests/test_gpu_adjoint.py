"""GPU adjoint (symxg_adjoint, symxg_rollout_forward/backward) against the oracle's FP64
adjoint (sparse direct solve of the true Hessian, closed-form mixed derivatives; itself
checked against finite differences in test_adjoint_cpu.py) and against central differences
of GPU solves.

Tolerances: FP64 path 1e-8 of max |.| for lambda and the parameter gradients at the same
state; mixed path 1e-4; finite differences 1e-5 relative (h = 1e-3 along a direction over
all element moduli); rollout 1e-5 relative (the GPU and oracle forward solves agree to their
Newton tolerance, not bitwise).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SOLVE = dict(residual_tolerance_abs=1e-9, cg_rel_tolerance=1e-10, max_iterations=200)


@pytest.fixture(scope="module")
def sg(lib):
    import symx_gb300

    return symx_gb300


def gpu_solve(sg, p, precision="fp64", **kw):
    s = sg.ElasticSolver(p)
    s.set_settings(precision=precision, **dict(SOLVE, **kw))
    s.set_state(p["x_init"], p["x0"], p["v0"])
    st = s.solve()
    # an Armijo stall (SYMXG_SOLVER_TOO_MANY_ARMIJO_ITERATIONS) at the rounding floor of the
    # energy counts as converged
    assert st["solver_return"] == 0 or (st["solver_return"] == 4 and st["final_residual"] < 1e-7), st
    return s


def close(a, b, tol):
    return np.max(np.abs(a - b)) <= tol * max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("case", ["tet4_6p", "hex8_3"])
def test_quasistatic_adjoint_fp64_matches_oracle(sg, case):
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.adjoint_problem(case)
    s = gpu_solve(sg, p)
    w = problems.normal(21, p["X"].size)
    out = s.adjoint(w, rel_tol=1e-12)
    assert out["info"]["converged"] == 1
    P = O.Problem(p, 1)
    P.set_x(s.get_positions())
    ref = O.adjoint(P, p, w)
    for k in ("lambda", "dLdmu", "dLdlam"):
        assert close(out[k], ref[k], 1e-8), k
    assert not np.any(out["dLdx0"]) and not np.any(out["dLdv0"])


def test_step_adjoint_inertia_terms_match_oracle(sg):
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.step_problem("tet4_6p")
    s = gpu_solve(sg, p)
    w = problems.normal(22, p["X"].size)
    out = s.adjoint(w, rel_tol=1e-12)
    P = O.Problem(p, 1)
    P.set_x(s.get_positions())
    ref = O.adjoint(P, p, w)
    for k in ("lambda", "dLdmu", "dLdlam", "dLdx0", "dLdv0"):
        assert close(out[k], ref[k], 1e-8), k


def test_adjoint_mixed_precision_matches_oracle(sg):
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.adjoint_problem("tet4_6p")
    s = gpu_solve(sg, p, precision="mixed")
    w = problems.normal(23, p["X"].size)
    out = s.adjoint(w, rel_tol=1e-7)
    assert out["info"]["converged"] == 1
    P = O.Problem(p, 1)
    P.set_x(s.get_positions())
    ref = O.adjoint(P, p, w)
    for k in ("lambda", "dLdmu", "dLdlam"):
        assert close(out[k], ref[k], 1e-4), k


def test_quasistatic_adjoint_matches_finite_differences(sg):
    from symx_gb300 import problems

    p = problems.adjoint_problem("tet4_3", k_bc=1e5)
    w = problems.normal(24, p["X"].size)  # L = w . x

    def loss(logE):
        mu, lam = problems.lame(np.exp(logE), 0.3)
        return float(w @ gpu_solve(sg, dict(p, mu=mu, lam=lam), residual_tolerance_abs=1e-11).get_positions().ravel())

    s = gpu_solve(sg, p, residual_tolerance_abs=1e-11)
    out = s.adjoint(w, rel_tol=1e-12)
    dLdp = p["mu"] * out["dLdmu"] + p["lam"] * out["dLdlam"]
    dp = 1.0 + 0.3 * problems.normal(25, p["logE"].size)
    h = 1e-3  # the solves stop at the energy's rounding floor; truncation O(h^2) stays ~1e-6
    fd = (loss(p["logE"] + h * dp) - loss(p["logE"] - h * dp)) / (2 * h)
    assert abs(fd - dLdp @ dp) <= 1e-5 * abs(fd), (fd, dLdp @ dp)


def test_rollout_gradient_matches_oracle_and_is_checkpoint_independent(sg):
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.rollout_problem("tet4_3", k_bc=1e5)
    n_steps = 4
    grads = []
    for every in (1, 3):
        s = sg.ElasticSolver(p)
        s.set_settings(precision="fp64", **dict(SOLVE, residual_tolerance_abs=1e-8))
        s.set_state(p["x_init"], p["x0"], p["v0"])
        info = s.rollout_forward(n_steps, every)
        assert info["steps"] == n_steps and info["checkpoints"] == -(-n_steps // every)
        xN = s.get_positions()
        d = xN.mean(axis=0) - p["target"]
        dLdx = np.tile(d / xN.shape[0], (xN.shape[0], 1))
        g = s.rollout_backward(dLdx, rel_tol=1e-12)
        assert g["info"]["recomputed_steps"] == n_steps
        grads.append(g)
    for k in ("dLdx0", "dLdv0", "dLdmu", "dLdlam"):
        assert np.array_equal(grads[0][k], grads[1][k]), k  # recomputation is bitwise deterministic
    settings = O.default_settings(residual_tolerance_abs=1e-10, cg_rel_tolerance=1e-12, cg_abs_tolerance=1e-14,
                                  max_iterations=200)
    states = O.rollout(p, n_steps, settings)
    assert close(xN, states[-1][0], 1e-8)
    ref = O.rollout_adjoint(p, states, dLdx)
    for k in ("dLdv0", "dLdmu", "dLdlam"):
        assert close(grads[0][k], ref[k], 1e-5), k
