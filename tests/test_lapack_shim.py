"""The Fortran-ABI LAPACK routines (libgbllt_lapack.so): dpotrf_, spotrf_, dpotrs_, spotrs_.

They keep the interface of Eigen's LAPACK build (lapack/cholesky.cpp:14-72): arguments by
reference, argument errors as info = -i after a call to xerbla_ (whose default prints the
reference's message, blas/xerbla.cpp:15-19), and info = k + 1 for a non-positive pivot at column k.
CPU tests cover loading, exports, argument errors and the absence of a CPU fallback; GPU tests
compare factors and solutions with the oracle.
"""
import ctypes
import subprocess

import numpy as np
import pytest

import gbllt as G

ROUTINES = ["dpotrf_", "spotrf_", "dpotrs_", "spotrs_", "dsyrk_", "ssyrk_", "dtrsm_", "strsm_"]


def test_shim_exports_the_lapack_routines():
    G.lapack()
    out = subprocess.run(["nm", "-D", "--defined-only", str(G.LAPACK_PATH)], capture_output=True, text=True).stdout
    syms = {l.split()[-1]: l.split()[-2] for l in out.splitlines()}
    for r in ROUTINES:
        assert syms.get(r) == "T", r
    assert syms.get("xerbla_") == "W"  # weak: an application's own handler wins
    # header and binding agree
    text = (G.PKG_DIR.parent / "include" / "gbllt_lapack.h").read_text()
    for r in ROUTINES + ["xerbla_"]:
        assert f" {r}(" in text
    assert set(G.LAPACK_SIGNATURES) == set(ROUTINES)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_potrf_argument_errors_go_through_xerbla(capfd, dt):
    a = np.eye(4, dtype=dt, order="F")
    name = ("D" if dt == np.float64 else "S") + "POTRF"
    assert G.lapack_potrf(a, "X") == -1
    assert G.lapack_potrf(a, "L", n=-1) == -2
    assert G.lapack_potrf(a, "L", lda=3) == -4
    out = capfd.readouterr().out
    assert f"Eigen BLAS ERROR #1: {name}" in out
    assert f"Eigen BLAS ERROR #2: {name}" in out
    assert f"Eigen BLAS ERROR #4: {name}" in out
    assert np.array_equal(a, np.eye(4, dtype=dt))


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_potrs_argument_errors_go_through_xerbla(capfd, dt):
    a = np.eye(4, dtype=dt, order="F")
    b = np.ones((4, 2), dtype=dt, order="F")
    name = ("D" if dt == np.float64 else "S") + "POTRS"
    assert G.lapack_potrs(a, b, "q") == -1
    assert G.lapack_potrs(a, b, "L", nrhs=-1) == -3
    assert G.lapack_potrs(a, b, "L", ldb=3) == -7
    out = capfd.readouterr().out
    for i in (1, 3, 7):
        assert f"Eigen BLAS ERROR #{i}: {name}" in out


def test_empty_problems_succeed():
    a = np.zeros((1, 1), order="F")
    assert G.lapack_potrf(a, "L", n=0) == 0
    assert G.lapack_potrs(a, np.zeros((1, 1), order="F"), "U", n=0, nrhs=0, ldb=1) == 0
    assert G.lapack_potrs(a, np.zeros((1, 1), order="F"), "L", n=1, nrhs=0, ldb=1) == 0


def test_no_cpu_fallback_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    a = np.eye(8, order="F")
    assert G.lapack_potrf(a, "L") == G.ERR_NO_DEVICE  # a gbllt code, not a LAPACK info
    assert np.array_equal(a, np.eye(8))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 33, 200, 777])
@pytest.mark.parametrize("uplo", ["L", "U", "l", "u"])
@pytest.mark.parametrize("dt", ["d", "s"])
def test_gpu_lapack_matches_oracle(oracle, n, uplo, dt):
    dtype = np.float64 if dt == "d" else np.float32
    a = np.asfortranarray(oracle.gen_gram(n, seed=7 + n).astype(dtype))
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, uplo.upper()) == 0
    f = np.array(a, order="F", copy=True)
    assert G.lapack_potrf(f, uplo) == 0
    tri = np.tril if uplo in "Ll" else np.triu
    tol = 1e-12 if dt == "d" else 1e-4
    assert np.linalg.norm(tri(f) - tri(ref)) <= tol * np.linalg.norm(tri(ref))
    other = np.triu(np.ones((n, n), bool), 1) if uplo in "Ll" else np.tril(np.ones((n, n), bool), -1)
    assert np.array_equal(f[other], a[other])  # the other triangle is not touched
    b = np.asfortranarray(oracle.normal(5, n * 3).reshape(n, 3, order="F").astype(dtype))
    x = np.array(b, order="F", copy=True)
    assert G.lapack_potrs(f, x, uplo) == 0
    xr = np.array(b, order="F", copy=True)
    oracle.potrs(ref, xr, uplo.upper())
    assert np.linalg.norm(x - xr) <= tol * 10 * np.linalg.norm(xr)


@pytest.mark.gpu
@pytest.mark.parametrize("col", [0, 5, 64, 100])
def test_gpu_lapack_failing_column(oracle, col):
    n = 130
    a = np.asfortranarray(oracle.gen_gram(n, seed=3))
    a[col, col] = -1.0
    ref = np.array(a, order="F", copy=True)
    want = oracle.potrf(ref, "L")
    assert want == col + 1
    f = np.array(a, order="F", copy=True)
    assert G.lapack_potrf(f, "L") == want
