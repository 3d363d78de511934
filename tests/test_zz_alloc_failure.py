"""Host-side fault injection: allocation failures (the failure-detection plan without a GPU fault).

GBLLT_INJECT_ALLOC_FAILURE=1 makes every device allocation of the library fail before CUDA is
called.  Each entry point must then return GBLLT_ERR_ALLOC (with a message) rather than crash or
compute, and once the variable is cleared the next calls must succeed: the device and the library
stay usable.  Collected last so that a failure here cannot disturb the other GPU tests.
"""
import ctypes
import os

import numpy as np
import pytest

import gbllt as G

pytestmark = pytest.mark.gpu


def _spd(oracle, n):
    return np.asfortranarray(oracle.gen_gram(n, seed=5))


def test_allocation_failures_are_reported_and_recoverable(oracle):
    torch = pytest.importorskip("torch")
    n = 200
    a = _spd(oracle, n)
    b = np.asfortranarray(oracle.normal(6, n * 2).reshape(n, 2, order="F"))
    L = G.lib()
    info = ctypes.c_int64(0)
    os.environ["GBLLT_INJECT_ALLOC_FAILURE"] = "1"
    try:
        f = np.array(a, order="F", copy=True)
        assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", n, f.ctypes.data, n, ctypes.byref(info)) == G.ERR_ALLOC
        assert np.array_equal(f, a)  # nothing was computed
        assert L.gbllt_last_error()
        x = np.array(b, order="F", copy=True)
        assert L.gbllt_dposv(G.COL_MAJOR, b"L", n, 2, f.ctypes.data, n, x.ctypes.data, n,
                             ctypes.byref(info)) == G.ERR_ALLOC
        da = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
        db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
        dx = torch.zeros_like(db)
        rc, _ = G.posv_mixed_dev(da, n, n, db, n, dx, n, 2, G.mixed_opts("bf16x6"), "L",
                                 torch.cuda.current_stream().cuda_stream, raise_on_error=False)
        assert rc == G.ERR_ALLOC
        sizes = np.array([5, 17, 40], dtype=np.int64)
        plan = ctypes.c_void_p()
        assert L.gbllt_batch_plan_create(3, sizes.ctypes.data, 8, ctypes.byref(plan)) == G.ERR_ALLOC
        r = ctypes.c_double(0)
        assert L.gbllt_dpocon(G.COL_MAJOR, b"L", n, a.ctypes.data, n, 1.0, ctypes.byref(r)) == G.ERR_ALLOC
        v = oracle.normal(7, n)
        assert L.gbllt_drank_update(G.COL_MAJOR, b"L", n, f.ctypes.data, n, v.ctypes.data, 1.0,
                                    ctypes.byref(info)) == G.ERR_ALLOC
    finally:
        del os.environ["GBLLT_INJECT_ALLOC_FAILURE"]
    # the same calls now succeed
    f = np.array(a, order="F", copy=True)
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", n, f.ctypes.data, n, ctypes.byref(info)) == 0 and info.value == 0
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, "L") == 0
    assert np.linalg.norm(np.tril(f) - np.tril(ref)) <= 1e-12 * np.linalg.norm(np.tril(ref))
    x = np.array(b, order="F", copy=True)
    G.posv(np.array(a, order="F", copy=True), x)
    assert oracle.backward_error(a, x, b) <= 1e-15
