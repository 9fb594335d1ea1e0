"""ctypes view of oracle/_build/liboracle.so.  Test infrastructure (the checker only)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_oracle import build

_lib = None


class Settings(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int), ("min_iterations", C.c_int),
        ("residual_tolerance_abs", C.c_double), ("residual_tolerance_rel", C.c_double),
        ("step_tolerance", C.c_double), ("max_iterations_as_success", C.c_int),
        ("projection_eps", C.c_double), ("mirroring", C.c_int),
        ("cg_max_iterations", C.c_int), ("cg_abs_tolerance", C.c_double),
        ("cg_rel_tolerance", C.c_double), ("armijo_beta", C.c_double), ("max_armijo", C.c_int),
        ("bailout_residual", C.c_double),
        ("projection_mode", C.c_int), ("project_on_demand_countdown", C.c_int),
        ("ppn_tightening_factor", C.c_double), ("ppn_release_factor", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("solver_return", C.c_int), ("newton_iterations", C.c_int), ("cg_iterations", C.c_int),
        ("ls_bt_iterations", C.c_int), ("final_residual", C.c_double), ("final_energy", C.c_double),
        ("t_eval", C.c_double), ("t_project", C.c_double), ("t_assembly", C.c_double),
        ("t_linear_solve", C.c_double), ("t_line_search", C.c_double), ("t_total", C.c_double),
        ("n_hessians", C.c_longlong), ("n_projected_hessians", C.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        P = C.c_void_p
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P, P, P, P, P, C.c_int, P, P,
                                    C.c_double, P, C.c_double, C.c_int]
        L.oracle_destroy.argtypes = [P]
        for f in ("oracle_set_x", "oracle_get_x"):
            getattr(L, f).argtypes = [P, P]
        L.oracle_evaluate.argtypes = [P, P, P]
        L.oracle_assemble.argtypes = [P, C.c_int, C.c_double, P, P, P, P, P]
        L.oracle_solve.argtypes = [P, C.POINTER(Settings), C.POINTER(Stats)]
        L.oracle_default_settings.argtypes = [C.POINTER(Settings)]
        L.oracle_nh_element_batch.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P]
        L.oracle_project_pd_batch.argtypes = [C.c_int, C.c_int, P, C.c_double, C.c_int, P]
        L.oracle_num_threads.restype = C.c_int
        L.oracle_set_state.argtypes = [P, P, P]
        L.oracle_bcsr_pcg.argtypes = [C.c_int32, P, P, P, P, P, C.c_double, C.c_double, C.c_int32, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def default_settings(**kw) -> Settings:
    s = Settings()
    lib().oracle_default_settings(C.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def nh_element_batch(x, X, mu, lam, want_hess=True):
    """x, X: (n, nodes, 3).  Returns E (n,), g (n, 3*nodes), H (n, 3*nodes, 3*nodes)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    n, nodes = x.shape[0], x.shape[1]
    m = 3 * nodes
    E = np.empty(n)
    g = np.empty((n, m))
    H = np.empty((n, m, m)) if want_hess else None
    rc = lib().oracle_nh_element_batch(nodes, n, _p(x), _p(X), _p(np.ascontiguousarray(mu, dtype=np.float64)),
                                       _p(np.ascontiguousarray(lam, dtype=np.float64)), _p(E), _p(g), _p(H))
    assert rc == 0
    return E, g, H


def project_pd_batch(mats, eps=1e-10, mirroring=False):
    a = np.array(mats, dtype=np.float64, copy=True, order="C")
    changed = np.zeros(a.shape[0], dtype=np.uint8)
    lib().oracle_project_pd_batch(a.shape[1], a.shape[0], _p(a), eps, int(mirroring), _p(changed))
    return a, changed.astype(bool)


class Problem:
    """The clamped Neo-Hookean implicit-Euler step of symx_gb300.problems.step_problem."""

    def __init__(self, p: dict, n_threads: int = 0):
        self._keep = {k: np.ascontiguousarray(v) for k, v in p.items() if isinstance(v, np.ndarray)}
        k = self._keep
        self.nv, self.ne, self.nodes = k["X"].shape[0], k["conn"].shape[0], k["conn"].shape[1]
        self.h = lib().oracle_create(
            self.nv, self.ne, self.nodes, _p(k["conn"].astype(np.int32)), _p(k["X"]), _p(k["x0"]), _p(k["v0"]),
            _p(k["x_init"]), _p(k["mass"]), _p(k["mu"]), _p(k["lam"]), int(k["bc_idx"].size),
            _p(k["bc_idx"].astype(np.int32)), _p(k["bc_target"]), float(p["dt"]),
            _p(np.asarray(p["gravity"], dtype=np.float64)), float(p["k_bc"]), int(n_threads))
        assert self.h

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def set_x(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        lib().oracle_set_x(self.h, _p(x))

    def get_x(self):
        x = np.empty((self.nv, 3))
        lib().oracle_get_x(self.h, _p(x))
        return x

    def evaluate(self):
        E = np.zeros(1)
        g = np.empty(3 * self.nv)
        lib().oracle_evaluate(self.h, _p(E), _p(g))
        return E[0], g

    def assemble(self, project=True, eps=1e-10):
        nnzb = np.zeros(1, dtype=np.int32)
        lib().oracle_assemble(self.h, int(project), eps, _p(nnzb), None, None, None, None)
        rowptr = np.empty(self.nv + 1, dtype=np.int32)
        cols = np.empty(nnzb[0], dtype=np.int32)
        vals = np.empty((nnzb[0], 3, 3))
        m = 3 * self.nodes
        eh = np.empty((self.ne, m, m))
        lib().oracle_assemble(self.h, int(project), eps, _p(nnzb), _p(rowptr), _p(cols), _p(vals), _p(eh))
        return rowptr, cols, vals, eh

    def set_state(self, x0=None, v0=None):
        a = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (x0, v0)]
        lib().oracle_set_state(self.h, _p(a[0]), _p(a[1]))

    def solve(self, settings: Settings | None = None) -> dict:
        s = settings or default_settings()
        st = Stats()
        lib().oracle_solve(self.h, C.byref(s), C.byref(st))
        return st.as_dict()


def bcsr_pcg(rowptr, cols, vals, b, abs_tol, rel_tol, max_iter):
    """bsm::solve_pcg with the block-diagonal preconditioner on a 3x3-block CSR matrix
    (vals (nnzb, 3, 3)), x0 = 0.  Returns (x, iterations, converged)."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    it = np.zeros(1, dtype=np.int32)
    conv = np.zeros(1, dtype=np.int32)
    rc = lib().oracle_bcsr_pcg(rowptr.size - 1, _p(rowptr), _p(cols), _p(vals), _p(b), _p(x), abs_tol, rel_tol,
                               max_iter, _p(it), _p(conv))
    if rc != 0:
        raise ValueError("a block row has no diagonal block")
    return x, int(it[0]), bool(conv[0])


def adjoint(P: "Problem", p: dict, dLdx, solver: str = "direct"):
    """FP64 adjoint at the oracle's current positions: lambda = H^-1 dL/dx with H the true
    (unprojected) Hessian, solved with a sparse direct factorisation, and the parameter
    gradients -lambda . dg/dq in closed form: the Neo-Hookean element gradient is linear in
    (mu, lambda), so dg_e/dmu_e = g_e(mu=1, lambda=0) and dg_e/dlambda_e = g_e(0, 1); the
    inertia gradient m (x - x0 - dt v0 - dt^2 g) / dt^2 gives -dg/dx0 = m / dt^2 and
    -dg/dv0 = m / dt.  solver: "direct" (sparse LU) or "pcg" (the oracle's PCG to 1e-12, for
    systems too large to factor).  Returns a dict of lambda, dLdmu, dLdlam, dLdx0, dLdv0 (flat)."""
    import scipy.sparse.linalg as spla

    rp, cols, vals, _ = P.assemble(project=False)
    b = np.asarray(dLdx, dtype=np.float64).ravel()
    if solver == "direct":
        lam = spla.spsolve(bcsr_to_scipy(rp, cols, vals).tocsc(), b)
    else:  # large systems: the oracle's block-Jacobi PCG to 1e-12
        lam, _, conv = bcsr_pcg(rp, cols, vals, b, 0.0, 1e-12, 100000)
        if not conv:
            raise RuntimeError("oracle adjoint PCG did not converge")
    x = P.get_x()
    X, conn = p["X"], p["conn"]
    ne = conn.shape[0]
    one, zero = np.ones(ne), np.zeros(ne)
    _, g_mu, _ = nh_element_batch(x[conn], X[conn], one, zero, want_hess=False)
    _, g_lam, _ = nh_element_batch(x[conn], X[conn], zero, one, want_hess=False)
    lam_e = lam.reshape(-1, 3)[conn].reshape(ne, -1)
    out = {"lambda": lam, "dLdmu": -(lam_e * g_mu).sum(1), "dLdlam": -(lam_e * g_lam).sum(1)}
    if float(p["dt"]) > 0.0:
        ml = p["mass"][:, None] * lam.reshape(-1, 3)
        out["dLdx0"] = (ml / p["dt"] ** 2).ravel()
        out["dLdv0"] = (ml / p["dt"]).ravel()
    else:
        out["dLdx0"] = np.zeros_like(lam)
        out["dLdv0"] = np.zeros_like(lam)
    return out


def rollout(p: dict, n_steps: int, settings: "Settings"):
    """Forward implicit-Euler rollout: each step solves from x = x0, then x0 <- x,
    v0 <- (x - x0_old) / dt.  Returns the states [(x_n, v_n)] for n = 0..n_steps."""
    P = Problem(p, 1)
    x0, v0 = np.array(p["x0"], dtype=np.float64), np.array(p["v0"], dtype=np.float64)
    states = [(x0.copy(), v0.copy())]
    for _ in range(n_steps):
        P.set_state(x0, v0)
        P.set_x(x0)
        st = P.solve(settings)
        if not (st["solver_return"] == 0 or (st["solver_return"] == 6 and st["final_residual"] < 1e-7)):
            raise RuntimeError(f"oracle rollout step did not converge: {st}")
        x = P.get_x()
        v0 = (x - x0) / p["dt"]
        x0 = x
        states.append((x0.copy(), v0.copy()))
    return states


def rollout_adjoint(p: dict, states, dLdx_final, dLdv_final=None):
    """Reverse-time adjoint of `rollout` in FP64 (per step the oracle adjoint at the step's
    solution): returns dL/dx_0, dL/dv_0 (flat) and dL/dmu, dL/dlam (per element)."""
    dt = float(p["dt"])
    ax = np.asarray(dLdx_final, dtype=np.float64).ravel().copy()
    av = np.zeros_like(ax) if dLdv_final is None else np.asarray(dLdv_final, dtype=np.float64).ravel().copy()
    dmu = np.zeros(p["conn"].shape[0])
    dlam = np.zeros_like(dmu)
    P = Problem(p, 1)
    for n in range(len(states) - 2, -1, -1):
        (xn, vn), (xn1, _) = states[n], states[n + 1]
        P.set_state(xn, vn)
        P.set_x(xn1)
        q = dict(p, x0=xn, v0=vn)
        adj = adjoint(P, q, ax + av / dt)
        dmu += adj["dLdmu"]
        dlam += adj["dLdlam"]
        ax, av = adj["dLdx0"] - av / dt, adj["dLdv0"]
    return {"dLdx0": ax, "dLdv0": av, "dLdmu": dmu, "dLdlam": dlam}


def bcsr_to_dense(rowptr, cols, vals):
    nb = rowptr.size - 1
    A = np.zeros((3 * nb, 3 * nb))
    for r in range(nb):
        for k in range(rowptr[r], rowptr[r + 1]):
            c = cols[k]
            A[3 * r:3 * r + 3, 3 * c:3 * c + 3] += vals[k]
    return A


def bcsr_to_scipy(rowptr, cols, vals):
    import scipy.sparse as sp
    nb = rowptr.size - 1
    return sp.bsr_matrix((vals, cols, rowptr), shape=(3 * nb, 3 * nb)).tocsr()
