"""Binary problem files shared by the reference harness (oracle/ref_harness.cpp), the C++ GPU
test program (tests/cpp/test_gpu_api.cpp) and the fixture generator.  Test infrastructure.

problem.bin (little-endian):
  int64  n_verts, n_elems, n_bc, nodes_per_elem
  f64    dt, gx, gy, gz, k_bc
  f64    X[nv*3], x0[nv*3], v0[nv*3], x_init[nv*3], mass[nv]
  int32  conn[ne*nodes]
  f64    mu[ne], lambda[ne]
  int32  bc_vertex[nbc];  f64 bc_target[nbc*3]
scene.bin (the contact scene):
  f64    ground_y, k_contact, k_spring, k_pull
  int64  n_handles;  int32 vertex[n];  f64 handle[n*3], target[n*3]
"""
from __future__ import annotations

import numpy as np


def write_problem(path, p):
    nv, ne, nn = p["X"].shape[0], p["conn"].shape[0], p["conn"].shape[1]
    with open(path, "wb") as f:
        np.array([nv, ne, p["bc_idx"].size, nn], dtype=np.int64).tofile(f)
        np.array([p["dt"], *p["gravity"], p["k_bc"]], dtype=np.float64).tofile(f)
        for k in ("X", "x0", "v0", "x_init"):
            np.ascontiguousarray(p[k], dtype=np.float64).tofile(f)
        np.ascontiguousarray(p["mass"], dtype=np.float64).tofile(f)
        np.ascontiguousarray(p["conn"], dtype=np.int32).tofile(f)
        np.ascontiguousarray(p["mu"], dtype=np.float64).tofile(f)
        np.ascontiguousarray(p["lam"], dtype=np.float64).tofile(f)
        np.ascontiguousarray(p["bc_idx"], dtype=np.int32).tofile(f)
        np.ascontiguousarray(p["bc_target"], dtype=np.float64).tofile(f)


def contact_scene(p):
    """The contact scene on a step problem: the ground plane 2 mm above the bottom face (so
    the bottom vertices start in contact), cubic contact stiffness 1e6, and three handles tied
    to the top vertices of the free end (largest x), pulled 2 mm up and 1 mm along z."""
    X = p["X"]
    top = np.flatnonzero(np.isclose(X[:, 1], X[:, 1].max()) & np.isclose(X[:, 0], X[:, 0].max()))
    hv = top[np.linspace(0, top.size - 1, 3).astype(int)].astype(np.int32)
    h0 = p["x_init"][hv].copy()
    return dict(ground_y=0.002, k_contact=1e6, k_spring=1e4, k_pull=1e3, vertex=hv, handle=h0,
                target=h0 + np.array([0.0, 0.002, 0.001]))


def write_scene(path, s):
    with open(path, "wb") as f:
        np.array([s["ground_y"], s["k_contact"], s["k_spring"], s["k_pull"]], dtype=np.float64).tofile(f)
        np.array([s["vertex"].size], dtype=np.int64).tofile(f)
        np.ascontiguousarray(s["vertex"], dtype=np.int32).tofile(f)
        np.ascontiguousarray(s["handle"], dtype=np.float64).tofile(f)
        np.ascontiguousarray(s["target"], dtype=np.float64).tofile(f)
