"""C ABI checks that need no GPU: the library loads, exports every function declared in
include/gbllt.h, rejects illegal arguments with the LAPACK convention (-i for argument i,
lapack/cholesky.cpp:17-24) before touching a device, and never falls back to the CPU."""
import ctypes

import numpy as np
import pytest

import gbllt as G


def test_library_exports_every_header_function():
    L = G.lib()
    declared = G.header_functions()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/gbllt.h but not exported"
    # the ctypes table covers exactly the header
    assert set(G.SIGNATURES) == set(declared)


def test_version():
    assert G.lib().gbllt_version() >= 100


def test_no_unexpected_exports():
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", str(G.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    ours = {s for s in exported if s.startswith("gbllt_")}
    assert ours == set(G.header_functions())


def _i64p(v=0):
    return ctypes.byref(ctypes.c_int64(v))


def test_potrf_argument_errors():
    L = G.lib()
    a = np.eye(4, order="F")
    p = a.ctypes.data
    info = ctypes.c_int64(0)
    assert L.gbllt_dpotrf(7, b"L", 4, p, 4, ctypes.byref(info)) == -1      # layout
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"X", 4, p, 4, ctypes.byref(info)) == -2
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", -1, p, 4, ctypes.byref(info)) == -3
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", 4, None, 4, ctypes.byref(info)) == -4
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", 4, p, 3, ctypes.byref(info)) == -5
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", 4, p, 4, None) == -6
    # n = 0 is a successful no-op (the empty-matrix case of test/cholesky.cpp:515)
    assert L.gbllt_dpotrf(G.COL_MAJOR, b"L", 0, None, 1, ctypes.byref(info)) == 0 and info.value == 0
    assert L.gbllt_spotrf(G.COL_MAJOR, b"u", 4, np.eye(4, dtype=np.float32, order="F").ctypes.data, 2,
                          ctypes.byref(info)) == -5


def test_potrs_argument_errors():
    L = G.lib()
    a = np.eye(4, order="F")
    b = np.ones((4, 2), order="F")
    assert L.gbllt_dpotrs(G.COL_MAJOR, b"L", 4, -2, a.ctypes.data, 4, b.ctypes.data, 4) == -4
    assert L.gbllt_dpotrs(G.COL_MAJOR, b"L", 4, 2, a.ctypes.data, 4, b.ctypes.data, 3) == -8
    assert L.gbllt_dpotrs(G.ROW_MAJOR, b"L", 4, 2, a.ctypes.data, 4, b.ctypes.data, 1) == -8
    assert L.gbllt_dpotrs(G.COL_MAJOR, b"L", 4, 0, a.ctypes.data, 4, None, 4) == 0
    assert L.gbllt_dposv(G.COL_MAJOR, b"L", 4, 2, a.ctypes.data, 4, b.ctypes.data, 4, None) == -9


def test_dev_argument_errors():
    L = G.lib()
    assert L.gbllt_dpotrf_dev(b"Q", 4, 1, 4, 1, None) == -1
    assert L.gbllt_dpotrf_dev(b"L", 4, 1, 2, 1, None) == -4
    assert L.gbllt_dpotrf_dev(b"L", 4, 1, 4, None, None) == -5
    assert L.gbllt_dpotrs_dev(b"L", 4, 1, 1, 4, 1, 2, None) == -7


def test_no_cpu_fallback_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    a = np.eye(8, order="F")
    info = ctypes.c_int64(0)
    rc = G.lib().gbllt_dpotrf(G.COL_MAJOR, b"L", 8, a.ctypes.data, 8, ctypes.byref(info))
    assert rc == G.ERR_NO_DEVICE
    assert np.array_equal(a, np.eye(8))  # untouched: nothing was computed on the host
