"""Synthetic inputs for the second-order solve path (host side, numpy).

Builds the structured meshes and seeded initial states that the solver is run
on.  The meshes follow the reference's generators:

* ``cuboid_tet4``: the structured cell grid of
  ``symx/src/solver/mesh_generation.cpp:38-91`` (vertex index
  ``i*(ny+1)*(nz+1) + j*(nz+1) + k``, every cell split into the same 6 tets
  around the v0-v6 diagonal, :76-83).
* ``cuboid_hex8``: ``mesh_generation.cpp:161-206`` (node order
  ``(-,-,-),(+,-,-),(+,+,-),(-,+,-)`` then the same at z+).

Two deliberate differences, both pure relabelings/translations that leave the
physics unchanged: the reference's reverse Cuthill-McKee renumbering
(``mesh_generation.cpp:89``) is not applied (the lexicographic numbering of a
structured grid is already banded), and the box is translated from
``[-L/2, L/2]`` to ``[0, L]`` so that the clamped face is ``x = 0``.  Configs with
``numbering="rcm"`` use the reference's numbering instead, built by the library's
``symxg_generate_cuboid_mesh``.

Random numbers come from a splitmix64 stream with a Box-Muller transform,
written out here so that the same seed gives the same inputs on every numpy
version and machine.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n consecutive outputs of the splitmix64 generator started at ``seed``."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = (np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """n doubles in (0, 1) from the top 53 bits of splitmix64."""
    z = splitmix64(seed, n)
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def normal(seed: int, n: int, mean: float = 0.0, std: float = 1.0) -> np.ndarray:
    """n standard-normal samples (Box-Muller over pairs of uniforms)."""
    m = (n + 1) // 2
    u = uniform01(seed, 2 * m)
    u1, u2 = u[0::2], u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.empty(2 * m)
    z[0::2] = r * np.cos(2.0 * np.pi * u2)
    z[1::2] = r * np.sin(2.0 * np.pi * u2)
    return mean + std * z[:n]


def _grid_vertices(nx, ny, nz, size):
    size = np.asarray(size, dtype=np.float64)
    delta = size / np.array([nx, ny, nz], dtype=np.float64)
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    ijk = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    return ijk * delta


def _cell_corners(nx, ny, nz):
    def index(i, j, k):
        return i * (ny + 1) * (nz + 1) + j * (nz + 1) + k

    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    v = [index(i, j, k), index(i + 1, j, k), index(i + 1, j + 1, k), index(i, j + 1, k),
         index(i, j, k + 1), index(i + 1, j, k + 1), index(i + 1, j + 1, k + 1), index(i, j + 1, k + 1)]
    return [a.astype(np.int32) for a in v]


def cuboid_tet4(nx: int, ny: int, nz: int, size):
    """Structured Tet4 box on [0, size]: (vertices (nv,3) f64, tets (6*cells,4) i32)."""
    X = _grid_vertices(nx, ny, nz, size)
    v0, v1, v2, v3, v4, v5, v6, v7 = _cell_corners(nx, ny, nz)
    tets = np.stack([
        np.stack([v0, v1, v6, v5], 1), np.stack([v0, v1, v2, v6], 1),
        np.stack([v0, v2, v3, v6], 1), np.stack([v0, v5, v6, v4], 1),
        np.stack([v0, v6, v3, v7], 1), np.stack([v0, v6, v7, v4], 1)], axis=1)
    return X, tets.reshape(-1, 4).astype(np.int32)


# Tet10 node order after the 4 corners: the midpoints of edges (0,1), (1,2), (2,0), (0,3),
# (1,3), (2,3), matching the quadratic shape functions (symx/src/solver/fem_integrators.h:56-76).
_TET10_EDGES = ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3))


def cuboid_tet10(nx: int, ny: int, nz: int, size):
    """Structured Tet10 box: the Tet4 split with a node at every edge midpoint
    (vertices (nv,3) f64, tets (6*cells,10) i32; corner vertices first)."""
    X, tets = cuboid_tet4(nx, ny, nz, size)
    nv = X.shape[0]
    pairs = np.stack([np.sort(tets[:, [a, b]], axis=1) for a, b in _TET10_EDGES], axis=1)  # (ne, 6, 2)
    keys = pairs[..., 0].astype(np.int64) * nv + pairs[..., 1]
    uniq, inv = np.unique(keys.ravel(), return_inverse=True)
    ua, ub = uniq // nv, uniq % nv
    mids = 0.5 * (X[ua] + X[ub])
    conn = np.concatenate([tets, (nv + inv.reshape(-1, 6)).astype(np.int32)], axis=1)
    return np.concatenate([X, mids], axis=0), conn.astype(np.int32)


def cuboid_hex8(nx: int, ny: int, nz: int, size):
    """Structured Hex8 box on [0, size]: (vertices (nv,3) f64, hexes (cells,8) i32)."""
    X = _grid_vertices(nx, ny, nz, size)
    hexes = np.stack(_cell_corners(nx, ny, nz), axis=1)
    return X, hexes.astype(np.int32)


def lame(youngs, poisson):
    """(mu, lambda) from Young's modulus and Poisson ratio (examples/NeoHookean.cpp:71-72)."""
    youngs = np.asarray(youngs, dtype=np.float64)
    mu = youngs / (2.0 * (1.0 + poisson))
    lam = youngs * poisson / ((1.0 + poisson) * (1.0 - 2.0 * poisson))
    return mu, lam


_HEX8_SIGNS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)


def element_volumes(X, conn):
    """Rest volume of each element (Tet4 and Tet10 with straight edges: |det|/6 of the
    corners; Hex8: 2x2x2 Gauss sum of det J)."""
    if conn.shape[1] in (4, 10):
        P = X[conn[:, :4]]
        D = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=2)
        return np.abs(np.linalg.det(D)) / 6.0
    P = X[conn]  # (ne, 8, 3)
    g = 1.0 / np.sqrt(3.0)
    vol = np.zeros(conn.shape[0])
    for q in _HEX8_SIGNS * g:
        dN = np.empty((8, 3))
        for a, s in enumerate(_HEX8_SIGNS):
            f = 0.5 * (1.0 + s * q)
            dN[a] = [0.5 * s[0] * f[1] * f[2], 0.5 * s[1] * f[0] * f[2], 0.5 * s[2] * f[0] * f[1]]
        J = np.einsum("eai,aj->eij", P, dN)
        vol += np.linalg.det(J)
    return vol


def lumped_mass(X, conn, density):
    """Per-vertex lumped mass: each element gives density*volume/nodes to each node
    (examples/dynamic_elasticity_with_contact.cpp:66-79)."""
    vol = element_volumes(X, conn)
    m = np.zeros(X.shape[0])
    share = density * vol / conn.shape[1]
    for a in range(conn.shape[1]):
        np.add.at(m, conn[:, a], share)
    return m


# Named workloads.  `cells` per axis, spacing h, and the seeds used for each random field.
CONFIGS = {
    # Plain FP64 Neo-Hookean Tet4 implicit-Euler step: 10^3 cells, 1,331 vertices, 6,000 tets.
    "tet4_10": dict(kind="tet4", cells=(10, 10, 10), h=0.01, perturb=0.0, seed=0),
    # Scaled-up step: 64^3 cells, 274,625 vertices, 1,572,864 tets, 5% spacing perturbation.
    "tet4_64": dict(kind="tet4", cells=(64, 64, 64), h=0.01, perturb=0.05, seed=1),
    # Hex8 slab, 128x128x32 cells, log-normal Young's modulus per element.
    "hex8_128x128x32": dict(kind="hex8", cells=(128, 128, 32), h=0.01, perturb=0.0, seed=2,
                            youngs_lognormal_sigma=0.5),
    # Smaller cases used by parity tests.
    "tet4_3": dict(kind="tet4", cells=(3, 3, 3), h=0.01, perturb=0.0, seed=10),
    "tet4_6p": dict(kind="tet4", cells=(6, 5, 4), h=0.01, perturb=0.05, seed=11),
    "hex8_3": dict(kind="hex8", cells=(3, 3, 2), h=0.01, perturb=0.0, seed=12,
                   youngs_lognormal_sigma=0.5),
    # Smaller Hex8 slab (65,536 elements) for kernel profiles.
    "hex8_64x64x16": dict(kind="hex8", cells=(64, 64, 16), h=0.01, perturb=0.0, seed=5,
                          youngs_lognormal_sigma=0.5),
    # Newton guess compressed to half height (plus a seeded 10% spacing jitter): the
    # unprojected Hessian is indefinite, so the adaptive projection modes retry and project.
    "tet4_5c": dict(kind="tet4", cells=(5, 4, 4), h=0.01, perturb=0.0, seed=13, init_compress_y=0.5,
                    init_perturb=0.1),
    # Quadratic tetrahedra (30 x 30 element Hessians, 4 quadrature points).
    "tet10_2": dict(kind="tet10", cells=(3, 2, 2), h=0.01, perturb=0.05, seed=14),
    # Quadratic tetrahedra at scale: 32^3 cells, 274,625 nodes (the 64^3 Tet4 node count),
    # 196,608 elements with 30 x 30 Hessians.
    "tet10_32": dict(kind="tet10", cells=(32, 32, 32), h=0.02, perturb=0.05, seed=15),
    # The 64^3 step on the reference's own mesh: generate_cuboid_Tet4_mesh with its reverse
    # Cuthill-McKee node numbering and element order (same statistics, other per-node draws).
    "tet4_64_rcm": dict(kind="tet4", cells=(64, 64, 64), h=0.01, perturb=0.05, seed=1, numbering="rcm"),
    "tet4_6p_rcm": dict(kind="tet4", cells=(6, 5, 4), h=0.01, perturb=0.05, seed=11, numbering="rcm"),
    "tet4_32": dict(kind="tet4", cells=(32, 32, 32), h=0.01, perturb=0.0, seed=3),
    # the metric's configuration at 32^3 cells: at-scale parity against the oracle's solve
    "tet4_32p": dict(kind="tet4", cells=(32, 32, 32), h=0.01, perturb=0.05, seed=7),
    "tet4_40": dict(kind="tet4", cells=(40, 40, 40), h=0.01, perturb=0.0, seed=4),
}


def step_problem(name_or_cfg, *, youngs=1e5, poisson=0.3, density=1000.0, dt=1.0 / 60.0,
                 gravity=(0.0, -9.81, 0.0), v_std=0.5, k_bc=1e8):
    """One implicit-Euler step of a clamped Neo-Hookean box.

    Returns a dict of numpy arrays: X (rest), x0 (previous positions), v0, x_init
    (initial Newton guess = x0), mass, conn, mu, lam (per element), bc_idx (vertices
    with x == 0), bc_target (their rest positions), and scalars dt, gravity, k_bc.
    """
    cfg = CONFIGS[name_or_cfg] if isinstance(name_or_cfg, str) else dict(name_or_cfg)
    nx, ny, nz = cfg["cells"]
    h = cfg["h"]
    size = (nx * h, ny * h, nz * h)
    if cfg.get("numbering") == "rcm":  # the reference's own mesh and numbering, moved to [0, L]
        from .capi import generate_cuboid_mesh

        X, conn = generate_cuboid_mesh(cfg["kind"], size, (nx, ny, nz))
        X = X + 0.5 * np.asarray(size)
        X[np.abs(X) < 1e-12 * max(size)] = 0.0  # exact zeros on the clamped face
    elif cfg["kind"] == "tet4":
        X, conn = cuboid_tet4(nx, ny, nz, size)
    elif cfg["kind"] == "tet10":
        X, conn = cuboid_tet10(nx, ny, nz, size)
    else:
        X, conn = cuboid_hex8(nx, ny, nz, size)
    nv, ne = X.shape[0], conn.shape[0]
    seed = int(cfg["seed"])
    sigma = cfg.get("youngs_lognormal_sigma", 0.0)
    if sigma > 0.0:
        E = np.exp(normal(seed * 1000 + 3, ne, mean=np.log(youngs), std=sigma))
    else:
        E = np.full(ne, youngs)
    mu, lam = lame(E, poisson)
    mass = lumped_mass(X, conn, density)
    v0 = normal(seed * 1000 + 1, nv * 3, std=v_std).reshape(nv, 3)
    x0 = X.copy()
    if cfg.get("perturb", 0.0) > 0.0:
        x0 = x0 + (cfg["perturb"] * h) * (2.0 * uniform01(seed * 1000 + 2, nv * 3) - 1.0).reshape(nv, 3)
    bc_idx = np.nonzero(X[:, 0] <= 1e-12)[0].astype(np.int32)
    x_init = x0.copy()
    if cfg.get("init_compress_y", 1.0) != 1.0:
        x_init[:, 1] *= cfg["init_compress_y"]
    if cfg.get("init_perturb", 0.0) > 0.0:
        x_init += (cfg["init_perturb"] * h) * (2.0 * uniform01(seed * 1000 + 4, nv * 3) - 1.0).reshape(nv, 3)
    return dict(
        name=cfg.get("name", name_or_cfg if isinstance(name_or_cfg, str) else "custom"),
        X=X, x0=x0, v0=v0, x_init=x_init, mass=mass, conn=conn, mu=mu, lam=lam,
        bc_idx=bc_idx, bc_target=X[bc_idx].copy(), dt=float(dt),
        gravity=np.asarray(gravity, dtype=np.float64), k_bc=float(k_bc),
    )


def adjoint_problem(name_or_cfg="tet4_32", *, youngs=1e5, poisson=0.3, log_std=0.3, seed=3, target_seed=4,
                    **kw):
    """Quasistatic adjoint case: a clamped Neo-Hookean box at equilibrium under gravity
    (dt = 0 selects the quasistatic form: gravity as the potential -m g.x, no inertia), with one
    parameter per element p_e = ln E_e ~ N(ln youngs, log_std^2) drawn from `seed`.  The target
    positions x* are the equilibrium of a second field drawn from `target_seed` (the caller
    solves for them).  Adds logE, mu_target, lam_target to the step_problem dict."""
    p = step_problem(name_or_cfg, youngs=youngs, poisson=poisson, **kw)
    ne = p["conn"].shape[0]
    logE = normal(seed * 1000 + 5, ne, mean=np.log(youngs), std=log_std)
    logE_t = normal(target_seed * 1000 + 5, ne, mean=np.log(youngs), std=log_std)
    p["mu"], p["lam"] = lame(np.exp(logE), poisson)
    p["mu_target"], p["lam_target"] = lame(np.exp(logE_t), poisson)
    p["logE"] = logE
    p["dt"] = 0.0
    p["x0"] = p["X"].copy()
    p["x_init"] = p["X"].copy()
    p["v0"] = np.zeros_like(p["X"])
    return p


def rollout_problem(name_or_cfg="tet4_40", *, youngs=1e5, poisson=0.3, log_std=0.3, seed=4, **kw):
    """Differentiable rollout case: implicit-Euler steps of a clamped Neo-Hookean box with
    v0 ~ N(0, 0.5^2) per component and per-element ln E_e ~ N(ln youngs, log_std^2) (both from
    `seed`), and a seeded target point for the final centroid (the box centroid displaced by
    N(0, (0.1 L)^2) per axis, L the largest box side)."""
    p = step_problem(name_or_cfg, youngs=youngs, poisson=poisson, **kw)
    ne = p["conn"].shape[0]
    logE = normal(seed * 1000 + 5, ne, mean=np.log(youngs), std=log_std)
    p["mu"], p["lam"] = lame(np.exp(logE), poisson)
    p["logE"] = logE
    p["x0"] = p["X"].copy()
    p["x_init"] = p["X"].copy()
    L = float(np.max(p["X"].max(axis=0) - p["X"].min(axis=0)))
    p["target"] = p["X"].mean(axis=0) + normal(seed * 1000 + 7, 3, std=0.1 * L)
    return p
