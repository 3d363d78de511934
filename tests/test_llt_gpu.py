"""Parity of the GPU plain-precision LLT (factor + solve) with Eigen and with the oracle.

All calls go through the C ABI (libgbllt.so).  Tolerances (relative Frobenius norms):
  - double factor vs Eigen / oracle on G G^T/n + I inputs: <= 1e-12 (hard bound 1e-10 at n=1024)
  - double factor on Eigen-test-style inputs (larger condition numbers): <= 1e-9
  - float factor: <= 1e-4 (Eigen's float test precision is 1e-3, test/main.h:410-411)
  - normwise backward error ||AX-B||/(||A|| ||X||) of double solves: <= 1e-14
  - failing column (info): exact.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden_input, load_golden, rel, tri

pytestmark = pytest.mark.gpu

CASES = load_golden()


def _tol(c):
    return {"d": 1e-12 if c["kind"] == "gram" else 1e-9, "s": 1e-4}[c["dtype"]]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['kind']}-{c['n']}-{c['dtype']}{c['uplo']}")
def test_gpu_matches_eigen_golden(oracle, gbllt, case):
    _, a, b = golden_input(oracle, case)
    f = np.array(a, order="F", copy=True)
    info = gbllt.potrf(f, case["uplo"])
    assert info == case["fail"] + 1
    if case["fail"] >= 0:
        return
    assert rel(tri(f, case["uplo"]), case["factor"]) <= _tol(case)
    x = np.array(b, order="F", copy=True)
    gbllt.potrs(f, x, case["uplo"])
    assert rel(x, case["x"]) <= _tol(case) * (10 if case["kind"] == "gram" else 100)


@pytest.mark.parametrize("n", [1, 2, 3, 31, 63, 64, 65, 127, 129, 200, 511, 777])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("dt", ["d", "s"])
def test_gpu_matches_oracle(oracle, gbllt, n, uplo, dt):
    dtype = np.float64 if dt == "d" else np.float32
    a = np.asfortranarray(oracle.gen_gram(n, seed=40 + n).astype(dtype))
    # poison the strict other triangle: it must come back bit-identical
    other = np.triu_indices(n, 1) if uplo == "L" else np.tril_indices(n, -1)
    a[other] = np.asarray(-777.25, dtype=dtype)
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, uplo) == 0
    f = np.array(a, order="F", copy=True)
    assert gbllt.potrf(f, uplo) == 0
    assert np.all(f[other] == dtype(-777.25))
    tol = 1e-12 if dt == "d" else 1e-4
    assert rel(tri(f, uplo), tri(ref, uplo)) <= tol
    k = 5
    b = np.asfortranarray(oracle.normal(3, n * k).reshape(n, k, order="F").astype(dtype))
    x = np.array(b, order="F", copy=True)
    gbllt.potrs(f, x, uplo)
    xr = np.array(b, order="F", copy=True)
    oracle.potrs(ref, xr, uplo)
    assert rel(x, xr) <= tol * 10
    be = oracle.backward_error(a, x, b, uplo)
    assert be <= (1e-15 if dt == "d" else 4 * n * 2.0 ** -24)


def test_gpu_posv_config1(oracle, gbllt):
    """n=1024, 16 RHS, A = G G^T/n + I (the reference's CPU-runnable configuration)."""
    n, k = 1024, 16
    a = oracle.gen_gram(n, seed=1)
    b = np.asfortranarray(oracle.normal(2, n * k).reshape(k, n).T)
    f, xr, info = oracle.solve(a, b)
    assert info == 0
    fg = np.array(a, order="F", copy=True)
    xg = np.array(b, order="F", copy=True)
    assert gbllt.posv(fg, xg) == 0
    assert rel(np.tril(fg), np.tril(f)) <= 1e-12
    assert rel(xg, xr) <= 1e-11
    assert oracle.backward_error(a, xg, b) <= 1e-15


def test_gpu_row_major_and_info_mapping(oracle, gbllt):
    n = 150
    a = oracle.gen_gram(n, seed=77)
    arow = np.ascontiguousarray(a)  # row-major storage of the same (symmetric) matrix
    info = ctypes.c_int64(-5)
    rc = gbllt.lib().gbllt_dpotrf(gbllt.ROW_MAJOR, b"L", n, arow.ctypes.data, n, ctypes.byref(info))
    assert rc == 0 and info.value == 0
    ref = np.array(a, order="F")
    oracle.potrf(ref, "L")
    # a row-major lower factor: arow[i, j] for i >= j holds L(i, j)
    assert rel(np.tril(arow), np.tril(ref)) <= 1e-12
    b = np.ascontiguousarray(oracle.normal(5, n * 4).reshape(n, 4))
    x = b.copy()
    rc = gbllt.lib().gbllt_dpotrs(gbllt.ROW_MAJOR, b"L", n, 4, arow.ctypes.data, n, x.ctypes.data, 4)
    assert rc == 0
    assert oracle.backward_error(np.asfortranarray(a), np.asfortranarray(x), np.asfortranarray(b)) <= 1e-15


@pytest.mark.parametrize("k", [0, 1, 63, 64, 65, 500, 999])
def test_gpu_failing_column(oracle, gbllt, k):
    n = 1000
    a = oracle.gen_gram(n, seed=3)
    a[k, k] = -1.0
    ref = np.array(a, order="F")
    assert oracle.blocked(ref) == k
    f = np.array(a, order="F")
    assert gbllt.potrf(f, "L") == k + 1
    fu = np.array(a, order="F")
    assert gbllt.potrf(fu, "U") == k + 1


def test_gpu_negative_definite(oracle, gbllt):
    a = np.asfortranarray(-oracle.gen_gram(80))
    assert gbllt.potrf(a, "L") == 1


def test_gpu_device_api_with_torch(oracle, gbllt):
    torch = pytest.importorskip("torch")
    n, k = 300, 7
    a = oracle.gen_gram(n, seed=8)
    b = np.asfortranarray(oracle.normal(9, n * k).reshape(n, k, order="F"))
    # column-major device storage: a torch tensor holding A^T row-major (A is symmetric anyway)
    lda = 320
    d = torch.zeros((n, lda), dtype=torch.float64, device="cuda")
    d[:, :n] = torch.from_numpy(np.ascontiguousarray(a.T))
    info = torch.full((1,), -9, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    gbllt.potrf_dev(d, n, lda, info, "L", s)
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    gbllt.potrs_dev(d, n, lda, db, k, n, "L", s)
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    fg = d[:, :n].cpu().numpy().T
    ref = np.array(a, order="F")
    oracle.potrf(ref)
    assert rel(np.tril(fg), np.tril(ref)) <= 1e-12
    assert np.all(d[:, n:].cpu().numpy() == 0)  # padding rows beyond n untouched
    x = np.asfortranarray(db.cpu().numpy().T)
    assert oracle.backward_error(a, x, b) <= 1e-15


@pytest.mark.slow
def test_gpu_full_size_config2_backward_error(oracle, gbllt):
    """n=16384, 64 RHS, Householder spectrum with kappa=1e6 (full size): normwise backward error."""
    torch = pytest.importorskip("torch")
    n, k = 16384, 64
    a = oracle.gen_householder(n, 1e6)
    b = np.asfortranarray(oracle.normal(12, n * k).reshape(k, n).T)
    d = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # = A (symmetric), column-major view
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    info = torch.zeros(1, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    gbllt.potrf_dev(d, n, n, info, "L", s)
    gbllt.potrs_dev(d, n, n, db, k, n, "L", s)
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    x = np.asfortranarray(db.cpu().numpy().T)
    cols = [0, 17, 63]
    be = oracle.backward_error(a, np.asfortranarray(x[:, cols]), np.asfortranarray(b[:, cols]))
    assert be <= 1e-14


def test_gpu_diagonal_pivots_are_square_roots(gbllt):
    """The FP64 diagonal-block kernel forms each pivot's reciprocal square root by Newton-Raphson
    from an FP32 estimate (library sqrt outside the FP32 range).  On a diagonal matrix the factor is
    the square root of each entry: it must match numpy's correctly rounded sqrt within 4 ulp, over
    magnitudes 1e-300 .. 1e300 (both code paths), and the solve must divide by them."""
    n = 192
    e = np.linspace(-300, 300, n)
    d = 10.0 ** e
    d[::7] *= 1.0 + 1e-9 * np.arange(len(d[::7]))  # mantissas other than powers of ten
    a = np.asfortranarray(np.diag(d))
    f = np.array(a, order="F", copy=True)
    assert gbllt.potrf(f, "L") == 0
    want = np.sqrt(d)
    got = np.diag(f)
    assert np.all(np.abs(got - want) <= 4 * np.spacing(want))
    assert np.all(np.tril(f, -1) == 0)
    x = np.asfortranarray(np.ones((n, 1)))
    gbllt.potrs(f, x, "L")
    assert np.allclose(x[:, 0] * d, 1.0, rtol=1e-14, atol=0)
