"""The residual R = B - A X of the refinement (gbllt_dsyresid_dev), A symmetric in one triangle.

Two methods: the FP64 pipe, and the tensor cores with error-free slicing (eight 7-bit BF16 slices of
A's rows and X's columns, exact FP32 accumulation in 256-deep chunks, exact int64 combination).
The bar for the tensor-core method:
  - integer inputs whose exact products fit in FP64 give the exact residual, bit for bit (this is
    what the chunked accumulation must guarantee);
  - general inputs agree with an extended-precision reference to 2^-50 relative to (|A||X|)_ij,
    including rows and columns scaled over 200 orders of magnitude;
  - a non-finite entry of A or X gives a NaN residual.
The FP64-pipe method is held to its own rounding bound (n u relative to (|A||X|)_ij).
"""
import ctypes

import numpy as np
import pytest

import gbllt as G

AUTO, FP64, TENSOR = 0, 1, 2


def _sym_full(a):
    return np.tril(a) + np.tril(a, -1).T


def _run(torch, a, x, b, uplo="L", method=TENSOR, lda=None):
    n, k = x.shape
    lda = n if lda is None else lda
    store = np.zeros((n, lda))  # row-major (n x lda) = column-major lda x n with leading dimension lda
    store[:, :n] = (a if uplo == "L" else a).T  # column j of A at row j of the row-major buffer
    dA = torch.from_numpy(np.ascontiguousarray(store)).cuda()
    dX = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    dR = torch.full((k, n), 7.0, dtype=torch.float64, device="cuda")
    rc = G.lib().gbllt_dsyresid_dev(uplo.encode(), n, k, dA.data_ptr(), lda, dX.data_ptr(), n, dB.data_ptr(), n,
                                    dR.data_ptr(), n, method, None)
    torch.cuda.synchronize()
    G.check("gbllt_dsyresid_dev", rc)
    return dR.cpu().numpy().T


def _reference(af, x, b):
    """B - A X in extended precision (numpy's longdouble), rounded to FP64 at the end."""
    ld = np.longdouble
    return (b.astype(ld) - af.astype(ld) @ x.astype(ld)).astype(np.float64)


def test_residual_argument_errors():
    L = G.lib()
    assert L.gbllt_dsyresid_dev(b"Q", 4, 1, 1, 4, 1, 4, 1, 4, 1, 4, 0, None) == -1
    assert L.gbllt_dsyresid_dev(b"L", -1, 1, 1, 4, 1, 4, 1, 4, 1, 4, 0, None) == -2
    assert L.gbllt_dsyresid_dev(b"L", 4, -1, 1, 4, 1, 4, 1, 4, 1, 4, 0, None) == -3
    assert L.gbllt_dsyresid_dev(b"L", 4, 1, None, 4, 1, 4, 1, 4, 1, 4, 0, None) == -4
    assert L.gbllt_dsyresid_dev(b"L", 4, 1, 1, 3, 1, 4, 1, 4, 1, 4, 0, None) == -5
    assert L.gbllt_dsyresid_dev(b"L", 4, 1, 1, 4, 1, 4, 1, 4, 1, 2, 0, None) == -11
    assert L.gbllt_dsyresid_dev(b"L", 4, 1, 1, 4, 1, 4, 1, 4, 1, 4, 5, None) == -12
    assert L.gbllt_dsyresid_dev(b"L", 4, 1, 1, 4, 1, 4, 1, 4, 1, 4, -1, None) == -12
    assert L.gbllt_dsyresid_dev(b"L", 0, 1, None, 1, None, 1, None, 1, None, 1, AUTO, None) == 0


@pytest.mark.gpu
# from n = 2048 the product runs K-split (2 to 8 ranges of whole chunks, summed exactly in int64)
@pytest.mark.parametrize("n,k", [(1, 1), (63, 5), (300, 64), (1000, 70), (2049, 3), (4096, 16), (8192, 64)])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_tensor_residual_exact_on_integers(oracle, n, k, uplo):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n + k)
    af = rng.integers(-1000, 1001, (n, n)).astype(np.float64)
    af = np.tril(af) + np.tril(af, -1).T
    x = rng.integers(-1000, 1001, (n, k)).astype(np.float64)
    b = rng.integers(-10**9, 10**9, (n, k)).astype(np.float64)
    want = b - af @ x  # every partial sum is an integer below 2^53: exact in FP64
    a = np.tril(af) if uplo == "L" else np.triu(af)
    a = a + (np.triu(np.full((n, n), 1e300), 1) if uplo == "L" else np.tril(np.full((n, n), 1e300), -1))
    got = _run(torch, a, x, b, uplo, TENSOR)
    assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(17, 1), (500, 64), (1537, 8), (4100, 2)])
@pytest.mark.parametrize("method", [TENSOR, FP64])
def test_residual_accuracy(oracle, n, k, method):
    torch = pytest.importorskip("torch")
    g = oracle.normal(n, n * n).reshape(n, n)
    af = g + g.T
    x = oracle.normal(n + 1, n * k).reshape(n, k)
    b = af @ x + 1e-10 * oracle.normal(n + 2, n * k).reshape(n, k)  # a residual much smaller than AX
    got = _run(torch, np.tril(af), x, b, "L", method)
    want = _reference(af, x, b)
    scale = np.abs(af) @ np.abs(x)
    err = np.max(np.abs(got - want) / scale)
    assert err <= (2.0 ** -50 if method == TENSOR else n * 2.0 ** -53), err


@pytest.mark.gpu
def test_tensor_residual_wide_scales(oracle):
    """Rows of A and columns of X scaled by powers of ten over 200 orders of magnitude (the per-row
    and per-column exponents of the slicing)."""
    torch = pytest.importorskip("torch")
    n, k = 700, 5
    d = 10.0 ** np.linspace(-100, 100, n)
    g = oracle.normal(3, n * n).reshape(n, n)
    af = (g + g.T) * np.sqrt(np.outer(d, d))
    x = oracle.normal(4, n * k).reshape(n, k) * 10.0 ** np.array([-50, 0, 10, 100, -120])
    b = oracle.normal(5, n * k).reshape(n, k)
    got = _run(torch, np.tril(af), x, b, "L", TENSOR)
    want = _reference(af, x, b)
    scale = np.abs(af) @ np.abs(x) + np.abs(b)
    assert np.max(np.abs(got - want) / scale) <= 2.0 ** -50


@pytest.mark.gpu
@pytest.mark.parametrize("where", ["a", "x"])
@pytest.mark.parametrize("n", [130, 4100])
def test_tensor_residual_nonfinite_gives_nan(oracle, where, n):
    torch = pytest.importorskip("torch")
    k = 3
    g = oracle.normal(8, n * n).reshape(n, n)
    af = g + g.T
    x = oracle.normal(9, n * k).reshape(n, k)
    if where == "a":
        af[70, 3] = af[3, 70] = np.inf
    else:
        x[11, 1] = np.nan
    got = _run(torch, np.tril(af), x, np.zeros((n, k)), "L", TENSOR)
    assert np.all(np.isnan(got))


@pytest.mark.gpu
def test_tensor_residual_leading_dimension(oracle):
    torch = pytest.importorskip("torch")
    n, k = 200, 4
    g = oracle.normal(10, n * n).reshape(n, n)
    af = g + g.T
    x = oracle.normal(11, n * k).reshape(n, k)
    b = oracle.normal(12, n * k).reshape(n, k)
    got = _run(torch, np.tril(af), x, b, "L", TENSOR, lda=213)
    want = _reference(af, x, b)
    assert np.max(np.abs(got - want) / (np.abs(af) @ np.abs(x) + np.abs(b))) <= 2.0 ** -50
