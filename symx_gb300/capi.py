"""ctypes declarations of the C ABI in include/symx_gb300.h.

`load()` opens the in-tree libsymxg.so and fails loudly if it has not been built: there
is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsymxg.so")

PRECISION_FP64 = 0
PRECISION_MIXED = 1

SOLVER_RETURN = {
    0: "Successful", 1: "Running", 2: "InvalidInitialState", 3: "TooManyIterations",
    4: "TooManyArmijoIterations", 5: "LinearSystemSolveFailure",
    6: "TooManyInvalidIntermediateIterations", 7: "StepDoesNotDescend", 8: "InvalidConvergedState",
}

# Every symbol include/symx_gb300.h declares (checked by the CPU tests).
EXPORTS = [
    "symxg_last_error", "symxg_abi_version", "symxg_default_settings", "symxg_elastic_create",
    "symxg_destroy", "symxg_set_settings", "symxg_set_state", "symxg_get_positions", "symxg_solve",
    "symxg_upload", "symxg_solve_device", "symxg_download", "symxg_evaluate", "symxg_evaluate_energy",
    "symxg_assembled_hessian", "symxg_element_outputs", "symxg_op_counts", "symxg_project_pd_f32",
    "symxg_project_pd_f64", "symxg_bcsr_spmv_f32", "symxg_bcsr_spmv_f64", "symxg_launch_count",
    "symxg_bcsr_pcg_f32", "symxg_bcsr_pcg_f64", "symxg_bcsr_pcg_f32_noalloc", "symxg_adjoint",
    "symxg_generate_cuboid_mesh",
    "symxg_rollout_forward", "symxg_rollout_backward", "symxg_set_wait_poll_limit", "symxg_wait_poll_limit",
    "symxg_device_memory",
]


class ElasticProblem(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32), ("n_elements", C.c_int32), ("nodes_per_element", C.c_int32),
        ("connectivity", C.c_void_p), ("rest_positions", C.c_void_p), ("mu", C.c_void_p),
        ("lam", C.c_void_p), ("mass", C.c_void_p), ("dt", C.c_double), ("gravity", C.c_double * 3),
        ("n_bc", C.c_int32), ("bc_vertices", C.c_void_p), ("bc_targets", C.c_void_p),
        ("bc_stiffness", C.c_double),
    ]


class NewtonSettings(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int32), ("min_iterations", C.c_int32),
        ("residual_tolerance_abs", C.c_double), ("residual_tolerance_rel", C.c_double),
        ("step_tolerance", C.c_double), ("max_iterations_as_success", C.c_int32),
        ("step_cap", C.c_double), ("enable_armijo_backtracking", C.c_int32),
        ("line_search_armijo_beta", C.c_double), ("max_backtracking_armijo_iterations", C.c_int32),
        ("project_to_pd", C.c_int32), ("projection_eps", C.c_double),
        ("project_to_pd_use_mirroring", C.c_int32), ("cg_max_iterations", C.c_int32),
        ("cg_abs_tolerance", C.c_double), ("cg_rel_tolerance", C.c_double),
        ("bailout_residual", C.c_double), ("precision", C.c_int32), ("time_kernels", C.c_int32),
        ("project_on_demand_countdown", C.c_int32), ("ppn_tightening_factor", C.c_double),
        ("ppn_release_factor", C.c_double), ("projection_fp64_refinement", C.c_int32),
        ("cg_residual_replacement", C.c_int32), ("cg_fp64_partial_sums", C.c_int32), ("cg_lookahead", C.c_int32),
    ]


class SolveStats(C.Structure):
    _fields_ = [
        ("solver_return", C.c_int32), ("newton_iterations", C.c_int32), ("cg_iterations", C.c_int32),
        ("ls_bt_iterations", C.c_int32), ("final_residual", C.c_double), ("final_energy", C.c_double),
        ("projection_not_converged", C.c_int32), ("t_evaluate_P_grad_hess", C.c_double),
        ("t_project_to_PD", C.c_double), ("t_assembly", C.c_double),
        ("t_linear_system_solve", C.c_double), ("t_evaluate_P", C.c_double),
        ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
        ("spmv_launches", C.c_int64), ("spmv_seconds", C.c_double),
        ("project_launches", C.c_int64), ("project_seconds", C.c_double),
        ("pcg_solve_iterations", C.c_int64), ("pcg_solve_seconds", C.c_double),
        ("cg_iterations_per_newton", C.c_int32 * 16),
        ("n_hessians", C.c_int64), ("n_projected_hessians", C.c_int64),
        ("cg_residual_replacements", C.c_int32), ("pad", C.c_int32),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["cg_iterations_per_newton"] = [int(v) for v in self.cg_iterations_per_newton if v]
        d["solver_return_name"] = SOLVER_RETURN.get(self.solver_return, str(self.solver_return))
        return d


class PcgInfo(C.Structure):
    _fields_ = [
        ("converged", C.c_int32), ("n_iterations", C.c_int32), ("error", C.c_double),
        ("found_indefiniteness", C.c_int32), ("missing_diagonal", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointInfo(C.Structure):
    _fields_ = [("converged", C.c_int32), ("iterations", C.c_int32), ("error", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RolloutInfo(C.Structure):
    _fields_ = [
        ("steps", C.c_int32), ("checkpoints", C.c_int32), ("newton_iterations", C.c_int32),
        ("cg_iterations", C.c_int32), ("recomputed_steps", C.c_int32), ("adjoint_iterations", C.c_int32),
        ("armijo_polished_steps", C.c_int32), ("pad", C.c_int32),
        ("seconds_forward", C.c_double), ("seconds_backward", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


class SymxgError(RuntimeError):
    pass


def load(path: str | None = None):
    """Open libsymxg.so (built by symx_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise SymxgError(f"{p} is missing: build the CUDA library first (python -m symx_gb300.build)")
    L = C.CDLL(p)
    P = C.c_void_p
    I32, I64, D = C.c_int32, C.c_int64, C.c_double
    sig = {
        "symxg_last_error": ([], C.c_char_p),
        "symxg_abi_version": ([], C.c_int),
        "symxg_launch_count": ([], C.c_int64),
        "symxg_set_wait_poll_limit": ([C.c_int64], None),
        "symxg_wait_poll_limit": ([], C.c_int64),
        "symxg_device_memory": ([C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int32], None),
        "symxg_default_settings": ([C.POINTER(NewtonSettings)], None),
        "symxg_elastic_create": ([C.POINTER(ElasticProblem), C.c_char_p, C.POINTER(P)], C.c_int),
        "symxg_destroy": ([P], C.c_int),
        "symxg_set_settings": ([P, C.POINTER(NewtonSettings)], C.c_int),
        "symxg_set_state": ([P, P, P, P], C.c_int),
        "symxg_get_positions": ([P, P], C.c_int),
        "symxg_solve": ([P, C.POINTER(I32), C.POINTER(SolveStats)], C.c_int),
        "symxg_upload": ([P], C.c_int),
        "symxg_solve_device": ([P, C.POINTER(I32), C.POINTER(SolveStats)], C.c_int),
        "symxg_download": ([P], C.c_int),
        "symxg_evaluate": ([P, P, P], C.c_int),
        "symxg_evaluate_energy": ([P, P], C.c_int),
        "symxg_assembled_hessian": ([P, I32, C.POINTER(I32), C.POINTER(I64), P, P, P], C.c_int),
        "symxg_element_outputs": ([P, I32, I32, P, P, P], C.c_int),
        "symxg_op_counts": ([P, I32, P], C.c_int),
        "symxg_generate_cuboid_mesh": ([I32, P, P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I32), P, P], C.c_int),
        "symxg_project_pd_f32": ([P, I32, I64, C.c_float, I32, P, P], C.c_int),
        "symxg_project_pd_f64": ([P, I32, I64, D, I32, P, P], C.c_int),
        "symxg_bcsr_spmv_f32": ([I32, P, P, P, I64, P, P, P], C.c_int),
        "symxg_bcsr_spmv_f64": ([I32, P, P, P, I64, P, P, P], C.c_int),
        "symxg_bcsr_pcg_f32": ([I32, P, P, P, I64, P, P, D, D, I32, C.POINTER(PcgInfo), P], C.c_int),
        "symxg_bcsr_pcg_f64": ([I32, P, P, P, I64, P, P, D, D, I32, C.POINTER(PcgInfo), P], C.c_int),
        "symxg_bcsr_pcg_f32_noalloc": ([I32, P, P, P, I64, P, P, D, D, I32, C.POINTER(PcgInfo), P], C.c_int),
        "symxg_adjoint": ([P, P, D, I32, P, P, P, P, P, C.POINTER(AdjointInfo)], C.c_int),
        "symxg_rollout_forward": ([P, I32, I32, C.POINTER(RolloutInfo)], C.c_int),
        "symxg_rollout_backward": ([P, P, P, D, I32, P, P, P, P, C.POINTER(RolloutInfo)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(rc: int):
    if rc != 0:
        msg = load().symxg_last_error().decode(errors="replace")
        raise SymxgError(f"symx_gb300 call failed (status {rc}): {msg}")


# FEM_Element order of the reference (symx/src/solver/fem_integrators.h:9).
ELEMENT_TYPES = {"tet4": 0, "tet10": 1, "hex8": 2, "hex27": 3}


def generate_cuboid_mesh(kind: str, size, cells):
    """The reference's generate_cuboid_mesh (mesh_generation.cpp:306-327): box of `size`
    centred at the origin, reverse Cuthill-McKee node numbering.  Returns (vertices (nv, 3)
    float64, connectivity (ne, stride) int32)."""
    import numpy as np

    L = load()
    t = ELEMENT_TYPES[kind]
    sz = (C.c_double * 3)(*map(float, size))
    nc = (C.c_int32 * 3)(*map(int, cells))
    nv, ne, st = C.c_int64(), C.c_int64(), C.c_int32()
    check(L.symxg_generate_cuboid_mesh(t, sz, nc, C.byref(nv), C.byref(ne), C.byref(st), None, None))
    X = np.empty((nv.value, 3), dtype=np.float64)
    conn = np.empty((ne.value, st.value), dtype=np.int32)
    check(L.symxg_generate_cuboid_mesh(t, sz, nc, C.byref(nv), C.byref(ne), C.byref(st), X.ctypes.data,
                                       conn.ctypes.data))
    return X, conn
