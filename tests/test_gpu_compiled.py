"""Compiled<T> on the GPU through the C++ API (tests/cpp/test_compiled.cpp): the reference's
compilation tests (chain of every operation in double and float, several expressions,
branches, log guard, caching, thread buffers, matrix inputs, check mode) plus batched
evaluation, and the Neo-Hookean Tet4 value/gradient/Hessian of 64 elements against the
reference's own outputs (golden fixture elem_nh_tet4; error <= 1e-12 of each block's
largest magnitude)."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cpp_compiled_on_gpu(compiled_test, golden, tmp_path):
    d = golden("elem_nh_tet4")
    rows, ref = d["inputs"], d["outputs"]
    fin, fref = tmp_path / "in.bin", tmp_path / "ref.bin"
    with open(fin, "wb") as f:
        np.array([rows.shape[0]], dtype=np.int64).tofile(f)
        np.ascontiguousarray(rows, dtype=np.float64).tofile(f)
    np.ascontiguousarray(ref, dtype=np.float64).tofile(fref)
    folder = tmp_path / "codegen"
    folder.mkdir()
    r = subprocess.run([compiled_test, "gpu", str(folder), str(fin), str(fref)], capture_output=True, text=True,
                       timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "compiled PASS" in r.stdout


def test_cpp_compiled_hex27_element_on_gpu(compiled_test, golden, tmp_path):
    """A Hex27 Neo-Hookean element (81 DoFs, 27 quadrature points) through Compiled<double> on the
    GPU gives the reference's energy and gradient within 1e-12."""
    d = golden("elem_nh_hex27")
    rows, ref = d["inputs"], d["outputs"]
    fin, fref = tmp_path / "in.bin", tmp_path / "ref.bin"
    with open(fin, "wb") as f:
        np.array([rows.shape[0]], dtype=np.int64).tofile(f)
        np.ascontiguousarray(rows, dtype=np.float64).tofile(f)
    np.ascontiguousarray(ref, dtype=np.float64).tofile(fref)
    folder = tmp_path / "codegen"
    folder.mkdir()
    r = subprocess.run([compiled_test, "hex27", str(folder), str(fin), str(fref)], capture_output=True, text=True,
                       timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "compiled PASS" in r.stdout
