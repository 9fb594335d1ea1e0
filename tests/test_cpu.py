"""CPU tests: the oracle against the reference's golden vectors, the C ABI library loading
and exporting every declared symbol, argument validation, and the C++ API (symbolic front
end, differentiation, NVRTC compilation of the generated kernels)."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from symx_gb300 import problems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["tet4_3", "tet4_6p", "hex8_3", "tet4_10", "tet10_2"]


# ------------------------------------------------------------------ oracle pinning
def test_oracle_element_matches_reference(golden):
    d = golden("elem_nh_tet4")
    rows, ref = d["inputs"], d["outputs"]
    E, g, H = O.nh_element_batch(rows[:, :12].reshape(-1, 4, 3), rows[:, 12:24].reshape(-1, 4, 3), rows[:, 24], rows[:, 25])
    assert np.max(np.abs(E - ref[:, 0]) / np.abs(ref[:, 0])) < 1e-11
    assert np.max(np.abs(g - ref[:, 1:13])) < 1e-12 * np.max(np.abs(ref[:, 1:13]))
    assert np.max(np.abs(H.reshape(-1, 144) - ref[:, 13:])) < 1e-12 * np.max(np.abs(ref[:, 13:]))


def test_doc_hessian_kat_structure(golden):
    """docs/source/compilation.md:269-281 prints a 12x12 Hessian for this element; the
    reference's own current code (run through oracle/_ref) gives different values for these
    inputs, so the printed values are not used as a pin.  Its zero pattern and symmetry are."""
    k = golden("doc_hessian_kat")
    _, _, H = O.nh_element_batch(k["x"][None], k["X"][None], np.array([float(k["mu"])]), np.array([float(k["lam"])]))
    H = H[0]
    assert np.array_equal(np.abs(H) < 1e-9 * np.abs(H).max(), k["H"] == 0)
    assert np.allclose(H, H.T, atol=1e-9 * np.abs(H).max())


@pytest.mark.parametrize("name", ["project12", "project24"])
def test_oracle_projection_matches_reference(golden, name):
    d = golden(name)
    out, changed = O.project_pd_batch(d["inputs"])
    for i in range(out.shape[0]):
        assert np.max(np.abs(out[i] - d["outputs"][i])) <= 1e-12 * np.max(np.abs(d["inputs"][i]))
    assert np.array_equal(changed, d["changed"].astype(bool))


@pytest.mark.parametrize("case", CASES)
def test_oracle_problem_matches_reference(golden, case):
    p = problems.step_problem(case)
    P = O.Problem(p, 1)
    ev = golden(f"{case}_eval")
    E, g = P.evaluate()
    assert abs(E - ev["E"]) <= 1e-13 * abs(ev["E"])
    assert np.max(np.abs(g - ev["grad"])) <= 1e-11 * np.max(np.abs(ev["grad"]))
    rp, cols, vals, _ = P.assemble(True)
    A = O.bcsr_to_scipy(rp, cols, vals)
    assert A.nnz == int(ev["nnz"])
    for v, ref in zip(ev["probe_vectors"], ev["probe_products"]):
        assert np.max(np.abs(A @ v - ref)) <= 1e-12 * np.max(np.abs(ref))
    sol = golden(f"{case}_solve")
    P.set_x(p["x_init"])
    st = P.solve(O.default_settings(cg_rel_tolerance=1e-3))
    assert st["solver_return"] == 0
    assert st["newton_iterations"] == int(sol["newton_iterations_full"])
    assert st["cg_iterations"] == int(sol["cg_iterations_full"])
    x = P.get_x()
    assert np.linalg.norm(x - sol["x_full"]) / np.linalg.norm(sol["x_full"] - p["x0"]) < 1e-10


MODES = {0: "newton", 1: "projected", 2: "on_demand", 3: "progressive"}
REF_TO_ORACLE_RETURN = {0: 0, 5: 4, 7: 5}  # SolverReturn values (solver_utils.h:15-26) -> oracle codes


@pytest.mark.parametrize("mode", sorted(MODES))
def test_oracle_projection_modes_match_reference(golden, mode):
    """NewtonsMethod::solve in each ProjectionToPD mode from an indefinite start (tet4_5c):
    the same return code, Newton and CG iterations, Hessian and projected-Hessian counts, and
    final positions as the reference."""
    d, tag = golden("tet4_5c_modes"), MODES[mode]
    p = problems.step_problem("tet4_5c")
    P = O.Problem(p, 1)
    st = P.solve(O.default_settings(cg_rel_tolerance=1e-3, projection_mode=mode))
    assert st["solver_return"] == REF_TO_ORACLE_RETURN[int(d[f"return_{tag}"])]
    for k in ("newton_iterations", "cg_iterations", "n_hessians", "n_projected_hessians"):
        assert st[k] == int(d[f"{k}_{tag}"]), k
    x = P.get_x()
    assert np.linalg.norm(x - d[f"x_{tag}"]) / np.linalg.norm(d[f"x_{tag}"] - p["x0"]) < 1e-10


def test_oracle_pcg_solves_assembled_system():
    import scipy.sparse.linalg as spla

    from symx_gb300 import problems

    p = problems.step_problem("tet4_6p")
    rp, cols, vals, _ = O.Problem(p, 1).assemble(True)
    A = O.bcsr_to_scipy(rp, cols, vals)
    b = problems.normal(3, A.shape[0])
    x, it, conv = O.bcsr_pcg(rp, cols, vals, b, 1e-14, 1e-12, 5000)
    xe = spla.spsolve(A.tocsc(), b)
    assert conv and 0 < it < 5000
    assert np.max(np.abs(x - xe)) <= 1e-8 * np.max(np.abs(xe))
    x, it, conv = O.bcsr_pcg(rp, cols, vals, np.zeros_like(b), 1e-12, 1e-6, 100)
    assert conv and it == 0 and not np.any(x)
    x, it, conv = O.bcsr_pcg(rp, cols, -vals, b, 1e-12, 1e-6, 100)
    assert not conv and it == 1
    with pytest.raises(ValueError):
        O.bcsr_pcg(np.array([0, 1, 2]), np.array([1, 0]), vals[:2], b[:6], 1e-12, 1e-6, 10)


def test_oracle_failure_codes():
    p = problems.step_problem("tet4_3")
    P = O.Problem(p, 1)
    st = P.solve(O.default_settings(cg_rel_tolerance=1e-3, max_iterations=1))
    assert st["solver_return"] == 2  # too many iterations
    P.set_x(p["x_init"])
    st = P.solve(O.default_settings(cg_rel_tolerance=1e-3, armijo_beta=1e6, max_armijo=3))
    assert st["solver_return"] == 6  # Armijo failure


def test_problem_sizes():
    # mesh sizes of the named workloads (vertices, elements)
    for name, nv, ne in (("tet4_10", 1331, 6000), ("tet4_32", 35937, 196608)):
        c = problems.CONFIGS[name]
        X, conn = problems.cuboid_tet4(*c["cells"], [n * c["h"] for n in c["cells"]])
        assert X.shape == (nv, 3) and conn.shape == (ne, 4)
    X, conn = problems.cuboid_hex8(4, 3, 2, (0.04, 0.03, 0.02))
    assert X.shape == (60, 3) and conn.shape == (24, 8)
    # every tet has positive rest volume (orientation of the 6-tet split)
    X, conn = problems.cuboid_tet4(3, 3, 3, (0.03, 0.03, 0.03))
    P = X[conn]
    D = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=2)
    assert np.all(np.linalg.det(D) > 0)
    # seeded normals are reproducible and standard
    z = problems.normal(3, 200000)
    assert np.array_equal(z, problems.normal(3, 200000))
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01


# ------------------------------------------------------------------ C ABI
def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "symx_gb300.h")).read()
    return sorted(set(re.findall(r"\b(symxg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    from symx_gb300 import capi

    declared = _declared_symbols()
    assert sorted(capi.EXPORTS) == declared
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.symxg_abi_version() == 5


def test_invalid_arguments_are_reported(lib):
    import ctypes as C

    from symx_gb300 import capi

    p = capi.ElasticProblem()
    p.n_vertices = 4
    p.n_elements = 1
    p.nodes_per_element = 5  # invalid element type
    h = C.c_void_p()
    rc = lib.symxg_elastic_create(C.byref(p), None, C.byref(h))
    assert rc == 1
    assert b"nodes_per_element" in lib.symxg_last_error()
    conn = np.array([[0, 1, 2, 7]], dtype=np.int32)  # vertex 7 does not exist
    X = np.zeros((4, 3))
    mu = np.ones(1)
    p.nodes_per_element = 4
    p.connectivity = conn.ctypes.data_as(C.c_void_p)
    p.rest_positions = X.ctypes.data_as(C.c_void_p)
    p.mu = mu.ctypes.data_as(C.c_void_p)
    p.lam = mu.ctypes.data_as(C.c_void_p)
    rc = lib.symxg_elastic_create(C.byref(p), None, C.byref(h))
    assert rc == 1 and b"out of range" in lib.symxg_last_error()
    assert lib.symxg_project_pd_f32(None, 12, 1, C.c_float(1e-10), 0, None, None) == 1
    assert lib.symxg_project_pd_f64(C.c_void_p(8), 13, 1, 1e-10, 0, C.c_void_p(8), None) == 1
    s = capi.NewtonSettings()
    lib.symxg_default_settings(C.byref(s))
    assert s.residual_tolerance_abs == 1e-6 and s.cg_rel_tolerance == 1e-4 and s.max_backtracking_armijo_iterations == 20
    # projection modes and their parameters: symx::NewtonSettings defaults (solver_utils.h:219-228)
    assert s.project_to_pd == 1 and s.project_on_demand_countdown == 4
    assert s.ppn_tightening_factor == 0.5 and s.ppn_release_factor == 2.0


# ------------------------------------------------------------------ C++ API
@pytest.fixture(scope="module")
def cpp_test(lib):
    exe = os.path.join(ROOT, "symx_gb300", "_build", "test_cpu_api")
    src = os.path.join(ROOT, "tests", "cpp", "test_cpu_api.cpp")
    libdir = os.path.join(ROOT, "symx_gb300", "_build")
    from symx_gb300.build import cuda_home

    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(cuda_home(), "include"), src, "-o", exe, "-L" + libdir, "-lsymxg",
                    "-Wl,-rpath," + libdir], check=True)
    return exe


def test_cpp_symbolic_selftest(cpp_test):
    r = subprocess.run([cpp_test, "selftest"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "selftest PASS" in r.stdout


def test_cpp_symbolic_nh_matches_reference(cpp_test, golden, tmp_path):
    d = golden("elem_nh_tet4")
    rows, ref = d["inputs"], d["outputs"]
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([rows.shape[0]], dtype=np.int64).tofile(f)
        rows.tofile(f)
    subprocess.run([cpp_test, "nh_elem", str(fin), str(fout)], check=True)
    out = np.fromfile(fout).reshape(-1, 157)
    for sl in (slice(0, 1), slice(1, 13), slice(13, 157)):
        assert np.max(np.abs(out[:, sl] - ref[:, sl])) <= 1e-13 * np.max(np.abs(ref[:, sl]))


def test_cpp_generated_kernels_compile_with_nvrtc(cpp_test, tmp_path):
    r = subprocess.run([cpp_test, "nvrtc", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "nvrtc PASS" in r.stdout


def test_cpp_compiled_generates_and_caches_without_a_device(compiled_test, tmp_path):
    """Compiled<double> without a GPU: the kernel is generated and NVRTC-compiled, its
    source, CUBIN and cache record are written, and loading fails with a clear error."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present: the GPU test covers Compiled<T>")
    r = subprocess.run([compiled_test, "nogpu", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "compiled PASS" in r.stdout


def test_host_build_of_projection_matches_reference(golden, tmp_path):
    """The device projection code built for the host: full and translation-deflated
    decompositions against the reference's project_to_PD_inplace on the 12x12 fixtures
    (32 Neo-Hookean element Hessians, which deflate, and 16 random symmetric matrices,
    which must be refused by the deflation test)."""
    exe = tmp_path / "test_projection_host"
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cpp", "test_projection_host.cpp"),
                    "-o", str(exe)], check=True)
    d = golden("project12")
    inp, ref = d["inputs"], d["outputs"]
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([inp.shape[0], 12], dtype=np.int64).tofile(f)
        inp.astype(np.float64).tofile(f)
    r = subprocess.run([str(exe), str(fin), str(fout)], capture_output=True, text=True, check=True)
    assert "not_converged 0" in r.stdout
    raw = np.fromfile(fout, dtype=np.uint8)
    n = inp.size
    out = raw[:32 * n].view(np.float64).reshape(4, *inp.shape)
    status = raw[32 * n:].view(np.int32).reshape(2, -1)
    nh = np.arange(inp.shape[0]) < 32
    assert np.all(status[:, nh] >= 0) and np.all(status[:, ~nh] == -1)
    scale = np.max(np.abs(inp), axis=(1, 2))[:, None, None]
    for mode, tol in ((0, 1e-9), (1, 1e-9), (2, 1e-4), (3, 1e-4)):
        err = np.abs(out[mode] - ref) / scale
        sel = nh if mode in (1, 3) else slice(None)
        assert np.max(err[sel]) <= tol, mode


def test_cpp_mesh_generators_match_reference(cpp_test, golden, tmp_path):
    """generate_cuboid_{Tet4,Tet10,Hex8,Hex27}_mesh: vertices and connectivity, node for node
    and element for element, equal to the reference's (RCM node order, reversed element walk)."""
    import json

    d = golden("meshes")
    for i, (prec, etype, n, size) in enumerate(json.loads(str(d["cases"]))):
        out = tmp_path / f"mesh{i}.bin"
        subprocess.run([cpp_test, "mesh", prec, str(etype), *map(str, n), *(repr(float(s)) for s in size), str(out)],
                       check=True)
        nv, ne, stride = (int(v) for v in np.fromfile(out, dtype=np.int64, count=3))
        ft = np.float32 if prec == "f" else np.float64
        verts = np.fromfile(out, dtype=ft, count=nv * 3, offset=24).reshape(nv, 3)
        conn = np.fromfile(out, dtype=np.int32, offset=24 + verts.nbytes).reshape(ne, stride)
        np.testing.assert_array_equal(conn, d[f"conn_{i}"], err_msg=f"case {i}")
        # Coordinates: one rounding of min + i * spacing apart at most.  The reference's release
        # build fuses that multiply-add in some components and not in others (Eigen packets
        # under -mfma); this library always fuses it.
        ulp = np.finfo(ft).eps * max(size)
        np.testing.assert_allclose(verts, d[f"vertices_{i}"], rtol=0, atol=ulp, err_msg=f"case {i}")
        assert sorted(set(conn.ravel())) == list(range(nv)) or stride in (10, 27)


def test_c_abi_mesh_generator_matches_reference(golden):
    """symxg_generate_cuboid_mesh gives the reference's connectivity, and the configs built on it
    clamp the whole x = 0 face."""
    import json

    from symx_gb300 import capi

    d = golden("meshes")
    cases = json.loads(str(d["cases"]))
    for i, (prec, etype, n, size) in enumerate(cases):
        if prec != "d":
            continue
        kind = [k for k, v in capi.ELEMENT_TYPES.items() if v == etype][0]
        X, conn = capi.generate_cuboid_mesh(kind, size, n)
        np.testing.assert_array_equal(conn, d[f"conn_{i}"], err_msg=f"case {i}")
        np.testing.assert_allclose(X, d[f"vertices_{i}"], rtol=0, atol=np.finfo(float).eps * max(size))
    with pytest.raises(capi.SymxgError, match="element_type"):
        capi.check(
            capi.load().symxg_generate_cuboid_mesh(7, (capi.C.c_double * 3)(1, 1, 1), (capi.C.c_int32 * 3)(1, 1, 1),
                                                   capi.C.byref(capi.C.c_int64()), capi.C.byref(capi.C.c_int64()),
                                                   capi.C.byref(capi.C.c_int32()), None, None))
    p = problems.step_problem("tet4_6p_rcm")
    nx, ny, nz = problems.CONFIGS["tet4_6p_rcm"]["cells"]
    assert p["conn"].shape == (6 * nx * ny * nz, 4)
    assert p["bc_idx"].size == (ny + 1) * (nz + 1)
    assert np.min(p["X"]) == 0.0


def test_cpp_rcm_reorder_matches_reference(cpp_test, golden, tmp_path):
    """reorder_connectivity_RCM on shuffled labels, two components and isolated nodes (one
    pseudo-peripheral root per component), with and without the element walk: the node
    permutation and the reordered connectivity equal the reference's."""
    d = golden("rcm")
    i = 0
    while f"meta_{i}" in d:
        stride, nn, reorder = (int(v) for v in d[f"meta_{i}"])
        conn = d[f"in_{i}"]
        fin, fout = tmp_path / f"rcm{i}.in", tmp_path / f"rcm{i}.out"
        with open(fin, "wb") as f:
            np.array([stride, conn.shape[0], nn], dtype=np.int64).tofile(f)
            conn.astype(np.int32).tofile(f)
        subprocess.run([cpp_test, "rcm", str(fin), str(fout), str(reorder)], check=True)
        res = np.fromfile(fout, dtype=np.int32)
        np.testing.assert_array_equal(res[:nn], d[f"old_to_new_{i}"], err_msg=f"case {i}")
        np.testing.assert_array_equal(res[nn:].reshape(conn.shape), d[f"conn_{i}"], err_msg=f"case {i}")
        i += 1
    assert i == 3


def test_cpp_hex27_element_matches_reference(cpp_test, golden, tmp_path):
    """Hex27: the triquadratic shape functions, node order and 27-point rule give the reference's
    Neo-Hookean element energy and gradient (six distorted elements)."""
    d = golden("elem_nh_hex27")
    rows, ref = d["inputs"], d["outputs"]
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([rows.shape[0]], dtype=np.int64).tofile(f)
        rows.tofile(f)
    subprocess.run([cpp_test, "nh_elem27", str(fin), str(fout)], check=True)
    out = np.fromfile(fout).reshape(-1, 82)
    assert np.max(np.abs(out[:, 0] - ref[:, 0])) <= 1e-12 * np.max(np.abs(ref[:, 0]))
    assert np.max(np.abs(out[:, 1:] - ref[:, 1:])) <= 1e-12 * np.max(np.abs(ref[:, 1:]))


def test_oracle_mixed_derivatives_match_reference_symbolic(golden):
    """The oracle's adjoint uses dg/dmu = g(mu = 1, lambda = 0) and dg/dlambda = g(0, 1) (the
    Neo-Hookean energy is linear in both); the reference's own gradient() of the element
    gradient gives the same values (tests/golden/mixed_nh_tet4.npz)."""
    d = golden("mixed_nh_tet4")
    for tag in ("random", "tet4_6p"):
        rows = d[f"inputs_{tag}"]
        x, X = rows[:, :12].reshape(-1, 4, 3), rows[:, 12:24].reshape(-1, 4, 3)
        one, zero = np.ones(rows.shape[0]), np.zeros(rows.shape[0])
        _, g_mu, _ = O.nh_element_batch(x, X, one, zero, want_hess=False)
        _, g_lam, _ = O.nh_element_batch(x, X, zero, one, want_hess=False)
        for got, ref in ((g_mu, d[f"dg_dmu_{tag}"]), (g_lam, d[f"dg_dlam_{tag}"])):
            assert np.max(np.abs(got.reshape(ref.shape) - ref)) <= 1e-12 * np.max(np.abs(ref))
