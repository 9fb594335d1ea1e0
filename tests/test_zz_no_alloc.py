"""Allocation-free PCG (symxg_bcsr_pcg_f32_noalloc) against the allocating entry point
(symxg_bcsr_pcg_f32), both called through the C ABI with ctypes.

Tolerance: the two solutions agree within 1e-6 of max |x| (single precision, the same
kernels on the same grid; they are expected to be equal), with equal iteration counts.
The file is named to be collected last, so it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(case="tet4_10", seed=21):
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.step_problem(case)
    rp, cols, vals, _ = O.Problem(p, 1).assemble(True)
    return rp, cols, vals, problems.normal(seed, 3 * (rp.size - 1))


def _call(fn, dev, x, rel_tol=1e-5):
    from symx_gb300 import capi

    rp, cols, vals, b = dev
    info = capi.PcgInfo()
    rc = fn(rp.numel() - 1, C.c_void_p(rp.data_ptr()), C.c_void_p(cols.data_ptr()), C.c_void_p(vals.data_ptr()),
            vals.stride(0), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), 1e-12, rel_tol, 2000, C.byref(info),
            None)
    return rc, info


def test_noalloc_matches_allocating_entry_point(lib):
    import torch

    import symx_gb300 as sg

    rp, cols, vals, b = _system()
    dev = (torch.tensor(rp, device="cuda"), torch.tensor(cols, device="cuda"),
           sg.component_major(torch.tensor(vals, dtype=torch.float32, device="cuda")),
           torch.tensor(b, dtype=torch.float32, device="cuda"))
    x_ref = torch.full((b.size,), float("nan"), dtype=torch.float32, device="cuda")
    x = [torch.full_like(x_ref, float("nan")) for _ in range(3)]
    torch.cuda.synchronize()

    rc, ref = _call(lib.symxg_bcsr_pcg_f32, dev, x_ref)
    assert rc == 0, lib.symxg_last_error()
    assert ref.converged == 1
    xr = x_ref.cpu().numpy()
    scale = np.max(np.abs(xr))

    # first call on the device: sets up the scratch address
    rc, info = _call(lib.symxg_bcsr_pcg_f32_noalloc, dev, x[0])
    assert rc == 0, lib.symxg_last_error()
    # two calls in a row after set-up, with device memory use observed around them
    free_before, _ = torch.cuda.mem_get_info()
    results = [_call(lib.symxg_bcsr_pcg_f32_noalloc, dev, x[k]) for k in (1, 2)]
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before

    for k, (rc, info) in zip((0, 1, 2), [(rc, info)] + results):
        assert rc == 0, lib.symxg_last_error()
        assert info.converged == 1 and info.found_indefiniteness == 0 and info.missing_diagonal == 0
        assert info.n_iterations == ref.n_iterations
        assert abs(info.error - ref.error) <= 1e-6 * max(ref.error, 1e-30)
        assert np.max(np.abs(x[k].cpu().numpy() - xr)) <= 1e-6 * scale


def test_noalloc_refuses_systems_above_its_limit(lib):
    import torch

    n = 65536 + 1
    # a valid (empty) matrix of n block rows: refused by the size check before any launch
    rp = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    cols = torch.zeros(1, dtype=torch.int32, device="cuda")
    vals = torch.zeros(9, 1, dtype=torch.float32, device="cuda")
    b = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
    x = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
    rc, info = _call(lib.symxg_bcsr_pcg_f32_noalloc, (rp, cols, vals, b), x)
    assert rc == 1  # SYMXG_ERR_INVALID_ARGUMENT
    assert b"maximum of 65536" in lib.symxg_last_error()
    assert info.n_iterations == 0
