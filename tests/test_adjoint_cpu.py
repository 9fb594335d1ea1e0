"""The FP64 adjoint restated in the oracle (sparse direct solve of the true Hessian plus
closed-form mixed derivatives), checked on the CPU against central finite differences of
full Newton solves.  Tolerance: 1e-5 relative (h = 1e-6 on ln E, h = 1e-4 along a random
direction of x0 and v0)."""
import numpy as np

from oracle import oracle as O
from symx_gb300 import problems

# residual floor ~3e-10: the 1e8 penalty stiffness times the rounding of x
TIGHT = dict(residual_tolerance_abs=1e-9, cg_rel_tolerance=1e-12, cg_abs_tolerance=1e-14, max_iterations=200)


def solve(p, mu, lam, x0=None, v0=None):
    q = dict(p, mu=mu, lam=lam)
    if x0 is not None:
        q["x0"], q["x_init"] = x0, x0
    if v0 is not None:
        q["v0"] = v0
    P = O.Problem(q, 1)
    st = P.solve(O.default_settings(**TIGHT))
    # an Armijo stall at the rounding floor of the energy counts as converged
    assert st["solver_return"] == 0 or (st["solver_return"] == 6 and st["final_residual"] < 1e-8), st
    return P, q


def test_oracle_quasistatic_adjoint_matches_finite_differences():
    p = problems.adjoint_problem("tet4_3")
    Pt, _ = solve(p, p["mu_target"], p["lam_target"])
    x_star = Pt.get_x()
    P, q = solve(p, p["mu"], p["lam"])
    x = P.get_x()
    adj = O.adjoint(P, q, (x - x_star).ravel())
    dLdp = p["mu"] * adj["dLdmu"] + p["lam"] * adj["dLdlam"]

    def loss(logE):
        mu, lam = problems.lame(np.exp(logE), 0.3)
        Q, _ = solve(p, mu, lam)
        return 0.5 * np.sum((Q.get_x() - x_star) ** 2)

    h = 1e-6
    for e in problems.splitmix64(99, 4) % p["conn"].shape[0]:
        lp, lm = p["logE"].copy(), p["logE"].copy()
        lp[e] += h
        lm[e] -= h
        fd = (loss(lp) - loss(lm)) / (2 * h)
        assert abs(fd - dLdp[e]) <= 1e-5 * max(abs(fd), 1e-3 * np.max(np.abs(dLdp))), (e, fd, dLdp[e])


def test_oracle_step_adjoint_inertia_terms_match_finite_differences():
    # softer boundary penalty: its stiffness sets the residual floor, and the inertia term
    # (m / dt^2 ~ 1) turns that floor into position noise the differences must stay above
    p = problems.step_problem("tet4_3", k_bc=1e5)
    rng_dir = problems.normal(5, p["X"].size).reshape(-1, 3)
    P, q = solve(p, p["mu"], p["lam"])
    x = P.get_x()
    w = problems.normal(6, x.size).reshape(-1, 3)  # L = w . x
    adj = O.adjoint(P, q, w.ravel())

    def loss(x0=None, v0=None):
        Q, _ = solve(p, p["mu"], p["lam"], x0=x0, v0=v0)
        return float(np.sum(w * Q.get_x()))

    h = 1e-4
    fd_v = (loss(v0=p["v0"] + h * rng_dir) - loss(v0=p["v0"] - h * rng_dir)) / (2 * h)
    assert abs(fd_v - adj["dLdv0"] @ rng_dir.ravel()) <= 1e-5 * abs(fd_v)
    fd_x = (loss(x0=p["x0"] + h * rng_dir) - loss(x0=p["x0"] - h * rng_dir)) / (2 * h)
    assert abs(fd_x - adj["dLdx0"] @ rng_dir.ravel()) <= 1e-5 * abs(fd_x)


def test_oracle_rollout_adjoint_matches_finite_differences():
    p = problems.rollout_problem("tet4_3", k_bc=1e5)
    settings = O.default_settings(**dict(TIGHT, residual_tolerance_abs=1e-11))
    n_steps = 3

    def loss(v0=None, logE=None):
        q = dict(p)
        if v0 is not None:
            q["v0"] = v0
        if logE is not None:
            q["mu"], q["lam"] = problems.lame(np.exp(logE), 0.3)
        xN = O.rollout(q, n_steps, settings)[-1][0]
        d = xN.mean(axis=0) - p["target"]
        return 0.5 * float(d @ d), xN

    _, xN = loss()
    d = xN.mean(axis=0) - p["target"]
    dLdx = np.tile(d / xN.shape[0], (xN.shape[0], 1))
    g = O.rollout_adjoint(p, O.rollout(p, n_steps, settings), dLdx)
    # a common velocity change moves the centroid: a well-conditioned difference
    direction = np.tile([1.0, 0.5, -0.3], (p["v0"].shape[0], 1)) + 0.1 * problems.normal(8, p["v0"].size).reshape(-1, 3)
    h = 1e-4
    fd = (loss(v0=p["v0"] + h * direction)[0] - loss(v0=p["v0"] - h * direction)[0]) / (2 * h)
    assert abs(fd - g["dLdv0"] @ direction.ravel()) <= 1e-5 * abs(fd)
    # ln E along a direction over all elements (one element's modulus barely moves the centroid)
    dLdp = p["mu"] * g["dLdmu"] + p["lam"] * g["dLdlam"]
    dp = 1.0 + 0.3 * problems.normal(9, p["logE"].size)
    fd = (loss(logE=p["logE"] + h * dp)[0] - loss(logE=p["logE"] - h * dp)[0]) / (2 * h)
    assert abs(fd - dLdp @ dp) <= 1e-5 * abs(fd), (fd, dLdp @ dp)
