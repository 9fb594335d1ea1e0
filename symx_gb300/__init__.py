"""symx_gb300: SymX's second-order solve path on NVIDIA GB300 (sm_103a).

The product is the C++/CUDA library symx_gb300/_build/libsymxg.so (C++ API in
include/symx, C ABI in include/symx_gb300.h).  This Python module is a thin ctypes
view of the C ABI for tests, benchmarks and scripting.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import PRECISION_FP64, PRECISION_MIXED, SOLVER_RETURN, SymxgError, check, load

__all__ = ["ElasticSolver", "load", "check", "SymxgError", "PRECISION_FP64", "PRECISION_MIXED", "component_major",
           "SOLVER_RETURN", "project_pd", "bcsr_spmv", "bcsr_pcg"]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class ElasticSolver:
    """Clamped Neo-Hookean implicit-Euler step (symxg_elastic_create) on the GPU.

    `problem` is a dict as produced by symx_gb300.problems.step_problem: X, conn, mu, lam,
    mass (or None for a quasistatic solve), dt, gravity, bc_idx, bc_target, k_bc; the
    state (x_init, x0, v0) is set with set_state().
    """

    def __init__(self, problem: dict, cache_dir: str | None = None):
        L = load()
        self._keep = {}
        X = _f64(problem["X"])
        conn = np.ascontiguousarray(problem["conn"], dtype=np.int32)
        mu = _f64(problem["mu"])
        lam = _f64(problem["lam"])
        mass = None if problem.get("mass") is None else _f64(problem["mass"])
        bc_idx = np.ascontiguousarray(problem.get("bc_idx", np.zeros(0)), dtype=np.int32)
        bc_t = _f64(problem.get("bc_target", np.zeros((0, 3))))
        self._keep.update(X=X, conn=conn, mu=mu, lam=lam, mass=mass, bc_idx=bc_idx, bc_t=bc_t)
        p = capi.ElasticProblem()
        p.n_vertices = X.shape[0]
        p.n_elements = conn.shape[0]
        p.nodes_per_element = conn.shape[1]
        p.connectivity = _ptr(conn)
        p.rest_positions = _ptr(X)
        p.mu = _ptr(mu)
        p.lam = _ptr(lam)
        p.mass = _ptr(mass)
        p.dt = float(problem.get("dt", 1.0 / 60.0))
        g = problem.get("gravity", (0.0, 0.0, 0.0))
        p.gravity = (C.c_double * 3)(*[float(v) for v in g])
        p.n_bc = bc_idx.size
        p.bc_vertices = _ptr(bc_idx)
        p.bc_targets = _ptr(bc_t)
        p.bc_stiffness = float(problem.get("k_bc", 0.0))
        h = C.c_void_p()
        check(L.symxg_elastic_create(C.byref(p), cache_dir.encode() if cache_dir else None, C.byref(h)))
        self.h = h
        self.nv = X.shape[0]
        self.nodes = conn.shape[1]
        self.n_potentials = 1 + (mass is not None) + (bc_idx.size > 0)
        self.settings = self.default_settings()

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            load().symxg_destroy(h)
            self.h = None

    @staticmethod
    def default_settings() -> capi.NewtonSettings:
        s = capi.NewtonSettings()
        load().symxg_default_settings(C.byref(s))
        return s

    def set_settings(self, **kw):
        for k, v in kw.items():
            if k == "precision" and isinstance(v, str):
                v = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED}[v]
            if not hasattr(self.settings, k):
                raise AttributeError(k)
            setattr(self.settings, k, v)
        check(load().symxg_set_settings(self.h, C.byref(self.settings)))

    def set_state(self, x=None, x0=None, v0=None):
        a = [None if v is None else _f64(v, (self.nv, 3)) for v in (x, x0, v0)]
        check(load().symxg_set_state(self.h, *[_ptr(v) for v in a]))

    def get_positions(self):
        x = np.empty((self.nv, 3))
        check(load().symxg_get_positions(self.h, _ptr(x)))
        return x

    def solve(self):
        ret = C.c_int32()
        st = capi.SolveStats()
        check(load().symxg_solve(self.h, C.byref(ret), C.byref(st)))
        return st.as_dict()

    def upload(self):
        check(load().symxg_upload(self.h))

    def solve_device(self):
        ret = C.c_int32()
        st = capi.SolveStats()
        check(load().symxg_solve_device(self.h, C.byref(ret), C.byref(st)))
        return st.as_dict()

    def download(self):
        check(load().symxg_download(self.h))

    def evaluate(self):
        E = np.zeros(1)
        g = np.empty(3 * self.nv)
        check(load().symxg_evaluate(self.h, _ptr(E), _ptr(g)))
        return float(E[0]), g

    def evaluate_energy(self):
        E = np.zeros(1)
        check(load().symxg_evaluate_energy(self.h, _ptr(E)))
        return float(E[0])

    def assembled_hessian(self, project=True):
        nb = C.c_int32()
        nnzb = C.c_int64()
        L = load()
        check(L.symxg_assembled_hessian(self.h, int(project), C.byref(nb), C.byref(nnzb), None, None, None))
        rp = np.empty(nb.value + 1, dtype=np.int32)
        cols = np.empty(nnzb.value, dtype=np.int32)
        vals = np.empty((nnzb.value, 3, 3))
        check(L.symxg_assembled_hessian(self.h, int(project), C.byref(nb), C.byref(nnzb), _ptr(rp), _ptr(cols),
                                        _ptr(vals)))
        return rp, cols, vals

    def element_outputs(self, potential=0, project=False, n_elements=None, nodes=None):
        n = n_elements if n_elements is not None else self._keep["conn"].shape[0]
        m = 3 * (nodes if nodes is not None else self.nodes)
        E = np.empty(n)
        g = np.empty((n, m))
        H = np.empty((n, m, m))
        check(load().symxg_element_outputs(self.h, potential, int(project), _ptr(E), _ptr(g), _ptr(H)))
        return E, g, H

    def adjoint(self, dLdx, rel_tol=1e-10, max_iterations=20000):
        """symxg_adjoint at the current device state: returns lambda, dLdmu, dLdlam (per
        element), dLdx0, dLdv0 (per vertex, zero without inertia) and the PCG info."""
        nd = 3 * self.nv
        ne = self._keep["conn"].shape[0]
        b = _f64(dLdx).ravel()
        out = {"lambda": np.empty(nd), "dLdmu": np.empty(ne), "dLdlam": np.empty(ne), "dLdx0": np.empty(nd),
               "dLdv0": np.empty(nd)}
        info = capi.AdjointInfo()
        check(load().symxg_adjoint(self.h, _ptr(b), float(rel_tol), int(max_iterations), _ptr(out["lambda"]),
                                   _ptr(out["dLdmu"]), _ptr(out["dLdlam"]), _ptr(out["dLdx0"]), _ptr(out["dLdv0"]),
                                   C.byref(info)))
        out["info"] = info.as_dict()
        return out

    def rollout_forward(self, n_steps, checkpoint_every):
        info = capi.RolloutInfo()
        check(load().symxg_rollout_forward(self.h, int(n_steps), int(checkpoint_every), C.byref(info)))
        return info.as_dict()

    def rollout_backward(self, dLdx_final, dLdv_final=None, rel_tol=1e-10, max_iterations=20000):
        """Reverse-time adjoint of the last rollout: dL/dx_0, dL/dv_0 (per vertex), dL/dmu,
        dL/dlam (per element) and the rollout info."""
        nd = 3 * self.nv
        ne = self._keep["conn"].shape[0]
        bx = _f64(dLdx_final).ravel()
        bv = None if dLdv_final is None else _f64(dLdv_final).ravel()
        out = {"dLdx0": np.empty(nd), "dLdv0": np.empty(nd), "dLdmu": np.empty(ne), "dLdlam": np.empty(ne)}
        info = capi.RolloutInfo()
        check(load().symxg_rollout_backward(self.h, _ptr(bx), _ptr(bv), float(rel_tol), int(max_iterations),
                                            _ptr(out["dLdx0"]), _ptr(out["dLdv0"]), _ptr(out["dLdmu"]),
                                            _ptr(out["dLdlam"]), C.byref(info)))
        out["info"] = info.as_dict()
        return out

    def op_counts(self, potential=0):
        c = np.zeros(3, dtype=np.int64)
        check(load().symxg_op_counts(self.h, potential, _ptr(c)))
        return c


def project_pd(H, eps=1e-10, mirroring=False, stream=None):
    """Project a CUDA torch tensor of shape (count, n, n) in place (block-major storage is
    handled here: the tensor is row-major, converted around the kernel call)."""
    import torch

    count, n, _ = H.shape
    k = n // 3
    bm = H.reshape(count, k, 3, k, 3).permute(0, 1, 3, 2, 4).contiguous()
    flag = torch.zeros(1, dtype=torch.int32, device=H.device)
    L = load()
    s = C.c_void_p(stream if stream is not None else torch.cuda.current_stream(H.device).cuda_stream)
    if H.dtype == torch.float32:
        check(L.symxg_project_pd_f32(C.c_void_p(bm.data_ptr()), n, count, C.c_float(eps), int(mirroring),
                                     C.c_void_p(flag.data_ptr()), s))
    elif H.dtype == torch.float64:
        check(L.symxg_project_pd_f64(C.c_void_p(bm.data_ptr()), n, count, eps, int(mirroring),
                                     C.c_void_p(flag.data_ptr()), s))
    else:
        raise TypeError("float32 or float64 expected")
    H.copy_(bm.permute(0, 1, 3, 2, 4).reshape(count, n, n))
    return bool(flag.item())


def component_major(vals):
    """(nnzb, 3, 3) block values -> the (9, nnzb) component-major layout of the BCSR kernels."""
    return vals.reshape(vals.shape[0], 9).t().contiguous()


def bcsr_spmv(row_ptr, cols, vals_cm, x, y, stream=None):
    """y = A x on CUDA torch tensors: row_ptr/cols int32, vals_cm (9, nnzb) component-major
    (see component_major), x/y (3 * n_block_rows,)."""
    import torch

    L = load()
    s = C.c_void_p(stream if stream is not None else torch.cuda.current_stream(x.device).cuda_stream)
    f = L.symxg_bcsr_spmv_f32 if vals_cm.dtype == torch.float32 else L.symxg_bcsr_spmv_f64
    check(f(row_ptr.numel() - 1, C.c_void_p(row_ptr.data_ptr()), C.c_void_p(cols.data_ptr()),
            C.c_void_p(vals_cm.data_ptr()), vals_cm.stride(0), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), s))


def bcsr_pcg(row_ptr, cols, vals_cm, b, x, abs_tol=1e-10, rel_tol=1e-6, max_iterations=1000, stream=None):
    """Solve A x = b with block-Jacobi PCG (x starts at zero) on CUDA torch tensors: A as for
    bcsr_spmv, b/x (3 * n_block_rows,) in the dtype of vals_cm.  Returns the PcgInfo fields
    as a dict; raises SymxgError if a block row has no diagonal block."""
    import torch

    L = load()
    s = C.c_void_p(stream if stream is not None else torch.cuda.current_stream(x.device).cuda_stream)
    f = L.symxg_bcsr_pcg_f32 if vals_cm.dtype == torch.float32 else L.symxg_bcsr_pcg_f64
    info = capi.PcgInfo()
    check(f(row_ptr.numel() - 1, C.c_void_p(row_ptr.data_ptr()), C.c_void_p(cols.data_ptr()),
            C.c_void_p(vals_cm.data_ptr()), vals_cm.stride(0), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
            float(abs_tol), float(rel_tol), int(max_iterations), C.byref(info), s))
    return info.as_dict()
