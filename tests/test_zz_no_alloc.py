"""The mixed-precision solve that allocates nothing, against the one that allocates.

gbllt_dposv_mixed_dev takes its scratch (the FP32 working matrix, panel operands, residuals)
from the CUDA stream-ordered pool.  Callers whose device memory belongs to their own caching
allocator or a fixed budget, and plug-ins handed only their buffers, use
gbllt_dposv_mixed_dev_noalloc, whose scratch is a fixed area inside the library image.  Both are called here through the C ABI
on the same inputs, the no-allocation one twice in a row (the second call finds the area as the
first call left it), and must agree within the tolerance this suite uses for double-precision
results (1e-12 relative), each reaching a normwise backward error <= 1e-14.

This file is collected last so that a run that stops at the first failure has run everything
else before it.
"""
import ctypes

import numpy as np
import pytest


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry(oracle, gbllt):
    torch = pytest.importorskip("torch")
    n, k = 1024, 4
    a = oracle.gen_gram(n, seed=21)
    b = np.asfortranarray(oracle.normal(22, n * k).reshape(n, k, order="F"))
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # column-major view of the symmetric A
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    s = torch.cuda.current_stream().cuda_stream
    opts = gbllt.mixed_opts("tf32x3", 10, 1e-14, True)

    X_ref = torch.zeros_like(B)
    rc, rep = gbllt.posv_mixed_dev(A, n, n, B, n, X_ref, n, k, opts, "L", s)
    torch.cuda.synchronize()
    assert rc == gbllt.SUCCESS and rep["converged"]
    xr = X_ref.cpu().numpy()

    L = gbllt.lib()
    for _ in range(2):
        X = torch.full_like(B, float("nan"))
        r = gbllt.MixedReport()
        rc = L.gbllt_dposv_mixed_dev_noalloc(b"L", n, k, A.data_ptr(), n, B.data_ptr(), n, X.data_ptr(), n,
                                             ctypes.byref(opts), ctypes.byref(r), s)
        torch.cuda.synchronize()
        assert rc == gbllt.SUCCESS, L.gbllt_last_error()
        d = r.as_dict()
        assert d["converged"] and d["backward_error"] <= 1e-14
        x = X.cpu().numpy()
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= 1e-12
        assert oracle.backward_error(a, np.asfortranarray(x.T), b) <= 1e-14


@pytest.mark.gpu
def test_noalloc_accepts_its_stated_maximum(oracle, gbllt):
    # n = 2048 with 64 right-hand sides and the FP64 fallback enabled fits the fixed area
    torch = pytest.importorskip("torch")
    n, k = 2048, 64
    a = oracle.gen_gram(n, seed=23)
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(oracle.normal(24, n * k).reshape(k, n))).cuda()
    X = torch.zeros_like(B)
    opts = gbllt.mixed_opts("tf32x3", 10, 1e-14, True)
    r = gbllt.MixedReport()
    rc = gbllt.lib().gbllt_dposv_mixed_dev_noalloc(b"L", n, k, A.data_ptr(), n, B.data_ptr(), n, X.data_ptr(), n,
                                                   ctypes.byref(opts), ctypes.byref(r),
                                                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == gbllt.SUCCESS, gbllt.lib().gbllt_last_error()
    assert r.converged and r.backward_error <= 1e-14


@pytest.mark.gpu
def test_noalloc_fallback_runs_inside_the_fixed_area(oracle, gbllt):
    # n = 2048, 64 right-hand sides, with one refinement step and an unreachable tolerance: the
    # refinement stops unconverged and the plain FP64 factorisation solves the system, its n x n
    # copy of A carved from the same fixed area.  Compared with the allocating entry under the same
    # options, twice in a row.
    torch = pytest.importorskip("torch")
    n, k = 2048, 64
    a = oracle.gen_gram(n, seed=25)
    b = np.asfortranarray(oracle.normal(26, n * k).reshape(n, k, order="F"))
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    s = torch.cuda.current_stream().cuda_stream
    opts = gbllt.mixed_opts("bf16", 1, 1e-300, True)
    X_ref = torch.zeros_like(B)
    rc, rep = gbllt.posv_mixed_dev(A, n, n, B, n, X_ref, n, k, opts, "L", s, raise_on_error=False)
    torch.cuda.synchronize()
    assert rc == gbllt.SUCCESS and rep["used_fallback"] == 1
    xr = X_ref.cpu().numpy()
    L = gbllt.lib()
    for _ in range(2):
        X = torch.full_like(B, float("nan"))
        r = gbllt.MixedReport()
        rc = L.gbllt_dposv_mixed_dev_noalloc(b"L", n, k, A.data_ptr(), n, B.data_ptr(), n, X.data_ptr(), n,
                                             ctypes.byref(opts), ctypes.byref(r), s)
        torch.cuda.synchronize()
        assert rc == gbllt.SUCCESS, L.gbllt_last_error()
        assert r.used_fallback == 1 and r.info == 0 and r.steps == 1
        x = X.cpu().numpy()
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= 1e-12
        assert oracle.backward_error(a, np.asfortranarray(x.T), b) <= 1e-14


def test_noalloc_rejects_sizes_beyond_its_scratch(gbllt):
    # n = 8192 needs far more scratch than the fixed area: rejected on the host, before any device work
    L = gbllt.lib()
    r = gbllt.MixedReport()
    rc = L.gbllt_dposv_mixed_dev_noalloc(b"L", 8192, 1, 16, 8192, 16, 8192, 16, 8192, None, ctypes.byref(r), None)
    assert rc == gbllt.ERR_SCRATCH_LIMIT
    assert b"scratch" in L.gbllt_last_error()
