"""Regenerate the golden fixtures in tests/golden/ from the reference SymX itself.

Test infrastructure.  Runs oracle/_ref/symx_ref_harness (the unmodified reference,
compiled from its own sources by ``make -f oracle/Makefile.ref``) on seeded inputs
and stores its outputs as small .npz files.  Only this script needs the reference;
the tests read the committed .npz files.

    make -f oracle/Makefile.ref -j8 && python tests/golden/make_golden.py

Fixtures:
  elem_nh_tet4.npz     per-element NH Tet4 [E, g(12), H(144)] via Compiled<double>
                        (value_gradient_hessian, diff.cpp:209-214), 64 seeded elements
  project12.npz        project_to_PD_inplace (project_to_PD.cpp:12-32) on 48 12x12 matrices
  project24.npz        same on 12 24x24 matrices (the reference's dynamic-size path)
  doc_hessian_kat.npz  the 12x12 NH Hessian printed in docs/source/compilation.md:269-281
  <case>_eval.npz      E, gradient, element Hessians, BCSR triplets at the initial state
  <case>_solve.npz     final positions and iteration counts of NewtonsMethod::solve
  tet4_5c_modes.npz    NewtonsMethod::solve in each ProjectionToPD mode (indefinite start)
  meshes.npz           generate_cuboid_mesh (mesh_generation.cpp:306-327) for each element type
  elem_nh_hex27.npz    NH Hex27 [E, g(81)] over the reference's Hex27 rule and shape functions
  rcm.npz              reorder_connectivity_RCM (mesh_ordering.cpp:231-252) on relabelled,
                        disconnected connectivities with isolated nodes
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from symx_gb300 import problems  # noqa: E402
sys.path.insert(0, HERE)
from problem_io import contact_scene, write_problem, write_scene  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "symx_ref_harness")
sys.path.insert(0, ROOT)
from __graft_entry__ import reference_dir  # noqa: E402  ($SYMX_REFERENCE_DIR or oracle/Makefile.ref's REF)

REF_DOC = os.path.join(reference_dir(), "docs", "source", "compilation.md")


def run(*args):
    subprocess.run([HARNESS, *map(str, args)], check=True, stdout=subprocess.DEVNULL)


def random_tets(seed, n):
    """Seeded Tet4 inputs: rest shapes around a regular tet, deformations from mild to
    strong compression, a few nearly inverted."""
    rows = np.empty((n, 26))
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    u = problems.uniform01(seed, n * 40).reshape(n, 40)
    for e in range(n):
        Xr = 0.01 * (base + 0.2 * (u[e, 0:12].reshape(4, 3) - 0.5))
        strength = [0.05, 0.3, 0.8][e % 3]
        x = Xr + 0.01 * strength * (u[e, 12:24].reshape(4, 3) - 0.5)
        x += u[e, 24:27] * 0.1  # rigid translation
        mu, lam = problems.lame(1e5 * (0.5 + u[e, 27]), 0.3 + 0.15 * u[e, 28])
        rows[e, 0:12] = x.ravel()
        rows[e, 12:24] = Xr.ravel()
        rows[e, 24], rows[e, 25] = mu, lam
    return rows


def make_elem(tmp):
    n = 64
    rows = random_tets(7, n)
    fin = os.path.join(tmp, "elem_in.bin")
    fout = os.path.join(tmp, "elem_out.bin")
    with open(fin, "wb") as f:
        np.array([n], dtype=np.int64).tofile(f)
        rows.tofile(f)
    run("elem", fin, fout)
    out = np.fromfile(fout, dtype=np.float64).reshape(n, 157)
    np.savez_compressed(os.path.join(HERE, "elem_nh_tet4.npz"), inputs=rows, outputs=out)
    return rows, out


def make_project(tmp, elem_out):
    # 12x12: real NH element Hessians (always indefinite or singular: rigid modes) and
    # seeded symmetric random matrices with a spread of negative eigenvalues.
    mats = [elem_out[i, 13:].reshape(12, 12) for i in range(32)]
    z = problems.normal(21, 16 * 144).reshape(16, 12, 12)
    for i in range(16):
        a = z[i] + z[i].T
        a += np.eye(12) * (1.0 * (i % 4) - 1.0)
        mats.append(a * 10.0 ** (i % 5 - 2))
    fixtures = {}
    for n, mlist, name in ((12, mats, "project12"), (24, None, "project24")):
        if mlist is None:
            z = problems.normal(22, 12 * 576).reshape(12, 24, 24)
            mlist = [(z[i] + z[i].T) * 10.0 ** (i % 4) + np.eye(24) * (i % 3 - 1.0) for i in range(12)]
        arr = np.stack(mlist).astype(np.float64)
        fin = os.path.join(tmp, f"{name}_in.bin")
        fout = os.path.join(tmp, f"{name}_out.bin")
        with open(fin, "wb") as f:
            np.array([arr.shape[0], n], dtype=np.int64).tofile(f)
            arr.tofile(f)
        run("project", fin, fout)
        out = np.fromfile(fout, dtype=np.float64).reshape(arr.shape)
        changed = np.fromfile(fout + ".changed", dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), inputs=arr, outputs=out, changed=changed)
        fixtures[name] = out
    return fixtures


def make_doc_kat():
    text = open(REF_DOC).read()
    m = re.search(r"Hessian = \n(.*?)```", text, re.S)
    rows = [list(map(float, line.split())) for line in m.group(1).strip().splitlines()]
    H = np.array(rows)
    assert H.shape == (12, 12)
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    X = np.array([[0, 0, 0], [0.9, 0, 0], [0, 0.8, 0], [0, 0, 0.7]], dtype=np.float64)
    mu, lam = problems.lame(1e6, 0.3)
    np.savez_compressed(os.path.join(HERE, "doc_hessian_kat.npz"), H=H, x=x, X=X, mu=mu, lam=lam,
                        source="docs/source/compilation.md:269-281 (printed to 6 significant digits)")


def make_case(tmp, case, solve_iters=(1, -1), keep_triplets=True):
    p = problems.step_problem(case)
    pfile = os.path.join(tmp, f"{case}.bin")
    write_problem(pfile, p)
    ev = os.path.join(tmp, f"{case}_eval")
    os.makedirs(ev, exist_ok=True)
    run("eval", pfile, ev, 1)
    rd = lambda name, dt: np.fromfile(os.path.join(ev, name), dtype=dt)  # noqa: E731
    E = rd("E.bin", np.float64)[0]
    grad = rd("grad.bin", np.float64)
    sizes = rd("hess_elem_size.bin", np.int32)
    hv = rd("hess_elem.bin", np.float64)
    hp = rd("hess_elem_projected.bin", np.float64)
    ti = rd("bcsr_triplet_idx.bin", np.int32).reshape(-1, 2)
    tv = rd("bcsr_triplet_val.bin", np.float64)
    ne = p["conn"].shape[0]
    n_el = 3 * p["conn"].shape[1]
    # element Hessians of the elastic potential come first (definition order)
    assert np.all(sizes[:ne] == n_el)
    H_el = hv[: ne * n_el * n_el].reshape(ne, n_el, n_el)
    H_el_p = hp[: ne * n_el * n_el].reshape(ne, n_el, n_el)
    ndof = grad.size
    out = dict(E=E, E_only=rd("E_only.bin", np.float64)[0], grad=grad, ndof=ndof)
    sample = np.unique(np.linspace(0, ne - 1, min(ne, 48)).astype(np.int64))
    out.update(hess_sample_idx=sample, hess_sample=H_el[sample], hess_sample_projected=H_el_p[sample])
    # the assembled projected matrix: exact triplets for small cases, products with seeded
    # vectors (a size-independent fingerprint) for all cases
    import scipy.sparse as sp
    A = sp.coo_matrix((tv, (ti[:, 0], ti[:, 1])), shape=(ndof, ndof)).tocsr()
    V = problems.normal(99, 2 * ndof).reshape(2, ndof)
    out.update(probe_vectors=V, probe_products=np.stack([A @ v for v in V]),
               diag=A.diagonal(), nnz=A.nnz)
    if keep_triplets:
        out.update(triplet_idx=ti, triplet_val=tv)
    np.savez_compressed(os.path.join(HERE, f"{case}_eval.npz"), **out)

    sol = {}
    for iters in solve_iters:
        sd = os.path.join(tmp, f"{case}_solve_{iters}")
        os.makedirs(sd, exist_ok=True)
        subprocess.run([HARNESS, "solve", pfile, sd, "1", str(iters), "1e-3"],
                       check=False, stdout=open(os.path.join(sd, "log.txt"), "w"))
        stats = json.load(open(os.path.join(sd, "stats.json")))
        tag = "full" if iters < 0 else f"it{iters}"
        sol[f"x_{tag}"] = np.fromfile(os.path.join(sd, "x_final.bin"), dtype=np.float64).reshape(-1, 3)
        for k in ("return", "newton_iterations", "cg_iterations", "ls_bt_iterations"):
            sol[f"{k}_{tag}"] = stats[k]
        sol[f"log_{tag}"] = open(os.path.join(sd, "log.txt")).read()
    np.savez_compressed(os.path.join(HERE, f"{case}_solve.npz"), **sol)
    return out, sol


def make_mixed(tmp):
    """d(dE/dx)/dmu and d(dE/dx)/dlambda of the NH Tet4 element through the reference's own
    gradient() and Compiled<double>: on the seeded elements of elem_nh_tet4 and on every
    element of tet4_6p at its initial state."""
    rows_rand = random_tets(7, 64)
    p = problems.step_problem("tet4_6p")
    c = p["conn"]
    rows_mesh = np.concatenate([p["x_init"][c].reshape(-1, 12), p["X"][c].reshape(-1, 12), p["mu"][:, None],
                                p["lam"][:, None]], axis=1)
    out = {}
    for tag, rows in (("random", rows_rand), ("tet4_6p", rows_mesh)):
        fin, fout = os.path.join(tmp, f"mixed_{tag}.in"), os.path.join(tmp, f"mixed_{tag}.out")
        with open(fin, "wb") as f:
            np.array([rows.shape[0]], dtype=np.int64).tofile(f)
            rows.tofile(f)
        run("mixed", fin, fout)
        res = np.fromfile(fout).reshape(rows.shape[0], 24)
        out[f"inputs_{tag}"] = rows
        out[f"dg_dmu_{tag}"] = res[:, :12]
        out[f"dg_dlam_{tag}"] = res[:, 12:]
    np.savez_compressed(os.path.join(HERE, "mixed_nh_tet4.npz"), **out)
    return out


def make_contact(tmp, case="tet4_6p"):
    """The step problem plus a conditional ground contact and a second DoF set (handles):
    energy and gradient at the initial state and the solve, from the reference."""
    p = problems.step_problem(case)
    scene = contact_scene(p)
    pfile, sfile = os.path.join(tmp, f"{case}_c.bin"), os.path.join(tmp, f"{case}_scene.bin")
    write_problem(pfile, p)
    write_scene(sfile, scene)
    sd = os.path.join(tmp, f"{case}_contact")
    os.makedirs(sd, exist_ok=True)
    subprocess.run([HARNESS, "contact", pfile, sfile, sd, "1"], check=True, stdout=open(os.path.join(sd, "log.txt"), "w"))
    rd = lambda name: np.fromfile(os.path.join(sd, name), dtype=np.float64)  # noqa: E731
    stats = json.load(open(os.path.join(sd, "stats.json")))
    out = dict(E=rd("E.bin")[0], grad=rd("grad.bin"), x_full=rd("x_final.bin").reshape(-1, 3),
               h_full=rd("h_final.bin").reshape(-1, 3), **{k: stats[k] for k in stats},
               log=open(os.path.join(sd, "log.txt")).read())
    np.savez_compressed(os.path.join(HERE, f"{case}_contact.npz"), **out)
    return out


MODES = {0: "newton", 1: "projected", 2: "on_demand", 3: "progressive"}


def make_modes(tmp, case="tet4_5c"):
    """NewtonsMethod::solve in each ProjectionToPD mode on a case whose unprojected Hessian is
    indefinite: final positions, return code, iteration counts and projected-Hessian counts."""
    p = problems.step_problem(case)
    pfile = os.path.join(tmp, f"{case}.bin")
    write_problem(pfile, p)
    out = {}
    for mode, tag in MODES.items():
        sd = os.path.join(tmp, f"{case}_mode{mode}")
        os.makedirs(sd, exist_ok=True)
        subprocess.run([HARNESS, "solve", pfile, sd, "1", "-1", "1e-3", str(mode)], check=False, timeout=120,
                       stdout=open(os.path.join(sd, "log.txt"), "w"))
        stats = json.load(open(os.path.join(sd, "stats.json")))
        out[f"x_{tag}"] = np.fromfile(os.path.join(sd, "x_final.bin"), dtype=np.float64).reshape(-1, 3)
        for k in ("return", "newton_iterations", "cg_iterations", "ls_bt_iterations", "n_hessians",
                  "n_projected_hessians"):
            out[f"{k}_{tag}"] = stats[k]
    np.savez_compressed(os.path.join(HERE, f"{case}_modes.npz"), **out)
    return out


# (precision, element type as FEM_Element's index, cells per axis, box size)
MESH_CASES = [
    ("d", 0, (3, 2, 4), (0.3, 0.2, 0.4)),
    ("d", 0, (7, 5, 6), (1.0, 0.5, 0.75)),
    ("f", 0, (4, 4, 3), (0.04, 0.04, 0.03)),
    ("d", 1, (2, 3, 2), (1.0, 1.5, 1.0)),
    ("d", 2, (5, 3, 4), (1.28, 1.28, 0.32)),
    ("f", 2, (3, 3, 3), (0.3, 0.3, 0.3)),
    ("d", 3, (2, 2, 3), (2.0, 1.0, 1.0)),
]


def read_mesh(path, prec):
    hdr = np.fromfile(path, dtype=np.int64, count=3)
    nv, ne, stride = (int(v) for v in hdr)
    ft = np.float32 if prec == "f" else np.float64
    verts = np.fromfile(path, dtype=ft, count=nv * 3, offset=24).reshape(nv, 3)
    conn = np.fromfile(path, dtype=np.int32, offset=24 + nv * 3 * verts.itemsize).reshape(ne, stride)
    return verts, conn


def make_meshes(tmp):
    out = {}
    for i, (prec, etype, n, size) in enumerate(MESH_CASES):
        path = os.path.join(tmp, f"mesh{i}.bin")
        run("mesh", prec, etype, *n, *(repr(float(s)) for s in size), path)
        out[f"vertices_{i}"], out[f"conn_{i}"] = read_mesh(path, prec)
    out["cases"] = np.array(json.dumps(MESH_CASES))
    np.savez_compressed(os.path.join(HERE, "meshes.npz"), **out)
    return out


# Hex27 node positions in half cells (the reference's node order, mesh_generation.cpp:253-295)
HEX27_AT = [(0, 0, 0), (2, 0, 0), (2, 2, 0), (0, 2, 0), (0, 0, 2), (2, 0, 2), (2, 2, 2), (0, 2, 2),
            (1, 0, 0), (2, 1, 0), (1, 2, 0), (0, 1, 0), (1, 0, 2), (2, 1, 2), (1, 2, 2), (0, 1, 2),
            (0, 0, 1), (2, 0, 1), (2, 2, 1), (0, 2, 1), (0, 1, 1), (2, 1, 1), (1, 2, 1), (1, 0, 1),
            (1, 1, 0), (1, 1, 2), (1, 1, 1)]


def make_elem27(tmp, n=6):
    rng = np.random.default_rng(27)
    base = 0.005 * np.array(HEX27_AT, dtype=np.float64)  # 1 cm cube
    rows = []
    for _ in range(n):
        X = base + 2e-4 * (rng.random(base.shape) - 0.5)
        A = np.eye(3) + 0.15 * (rng.random((3, 3)) - 0.5)
        x = X @ A.T + 3e-4 * (rng.random(base.shape) - 0.5)
        mu, lam = problems.lame(1e5 * np.exp(0.3 * rng.standard_normal()), 0.3)
        rows.append(np.concatenate([x.ravel(), X.ravel(), [mu, lam]]))
    rows = np.array(rows)
    fin, fout = os.path.join(tmp, "e27.in"), os.path.join(tmp, "e27.out")
    with open(fin, "wb") as f:
        np.array([n], dtype=np.int64).tofile(f)
        rows.tofile(f)
    run("elem27", fin, fout)
    out = np.fromfile(fout).reshape(n, 82)
    np.savez_compressed(os.path.join(HERE, "elem_nh_hex27.npz"), inputs=rows, outputs=out)
    return out


def rcm_inputs():
    """Seeded connectivities for reorder_connectivity_RCM: (stride, num_nodes, conn, reorder_elements)."""
    rng = np.random.default_rng(21)
    cases = []
    # two disjoint Tet4 boxes and three isolated nodes, nodes and elements shuffled
    _, a = problems.cuboid_tet4(3, 2, 2, (1.0, 1.0, 1.0))
    _, b = problems.cuboid_tet4(2, 2, 1, (1.0, 1.0, 1.0))
    na = int(a.max()) + 1
    conn = np.concatenate([a, b + na])
    nn = int(conn.max()) + 1 + 3
    perm = rng.permutation(nn).astype(np.int32)
    cases.append((4, nn, perm[conn][rng.permutation(conn.shape[0])], 1))
    # a relabelled Hex8 box, elements kept in place
    _, h = problems.cuboid_hex8(3, 3, 2, (1.0, 1.0, 1.0))
    nn = int(h.max()) + 1
    cases.append((8, nn, rng.permutation(nn).astype(np.int32)[h], 0))
    # a relabelled Tet10 box
    _, t = problems.cuboid_tet10(2, 1, 2, (1.0, 1.0, 1.0))
    nn = int(t.max()) + 1
    cases.append((10, nn, rng.permutation(nn).astype(np.int32)[t][rng.permutation(t.shape[0])], 1))
    return cases


def make_rcm(tmp):
    out = {}
    for i, (stride, nn, conn, reorder) in enumerate(rcm_inputs()):
        fin, fout = os.path.join(tmp, f"rcm{i}.in"), os.path.join(tmp, f"rcm{i}.out")
        with open(fin, "wb") as f:
            np.array([stride, conn.shape[0], nn], dtype=np.int64).tofile(f)
            np.ascontiguousarray(conn, dtype=np.int32).tofile(f)
        run("rcm", fin, fout, reorder)
        res = np.fromfile(fout, dtype=np.int32)
        out[f"in_{i}"] = conn.astype(np.int32)
        out[f"meta_{i}"] = np.array([stride, nn, reorder], dtype=np.int64)
        out[f"old_to_new_{i}"] = res[:nn]
        out[f"conn_{i}"] = res[nn:].reshape(conn.shape)
    np.savez_compressed(os.path.join(HERE, "rcm.npz"), **out)
    return out


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: make -f oracle/Makefile.ref -j8")
    if sys.argv[1:] == ["meshes"]:  # only the mesh-generator and ordering fixtures
        with tempfile.TemporaryDirectory() as tmp:
            make_meshes(tmp)
            make_rcm(tmp)
            print(make_elem27(tmp)[:, :3])
        return
    if sys.argv[1:] == ["contact"]:  # conditional potential + second DoF set, and the mixed derivatives
        with tempfile.TemporaryDirectory() as tmp:
            out = make_contact(tmp)
            print({k: out[k] for k in ("E", "return", "newton_iterations", "cg_iterations")})
            mx = make_mixed(tmp)
            print(mx["dg_dmu_random"][0, :3])
        return
    if sys.argv[1:] == ["modes"]:  # only the projection-mode fixture
        with tempfile.TemporaryDirectory() as tmp:
            print(make_modes(tmp))
        return
    if len(sys.argv) == 3 and sys.argv[1] == "case":  # one problem's eval and solve fixtures
        with tempfile.TemporaryDirectory() as tmp:
            out, sol = make_case(tmp, sys.argv[2], keep_triplets=sys.argv[2] != "tet10_2")
            print({k: v for k, v in sol.items() if not k.startswith(("x_", "log_"))})
        return
    with tempfile.TemporaryDirectory() as tmp:
        rows, out = make_elem(tmp)
        make_project(tmp, out)
        make_doc_kat()
        make_case(tmp, "tet4_3")
        make_case(tmp, "tet4_6p")
        make_case(tmp, "hex8_3")
        make_case(tmp, "tet4_10", keep_triplets=False)
        make_case(tmp, "tet10_2", keep_triplets=False)
        make_modes(tmp)
        make_meshes(tmp)
        make_rcm(tmp)
        make_elem27(tmp)
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
