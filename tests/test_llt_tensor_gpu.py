"""Parity of the FP64 factorisation where its trailing updates run on the tensor cores.

From n = 1024 the FP64 factorisation works in 256-wide panels whose updates are FP64-exact products
on the BF16 tensor cores (error-free slicing into 8 integer slices per operand, exact FP32
accumulation, int64 combination).  Every test here is at n >= 1024, so that path is the one that
runs; all calls go through the C ABI.  Tolerances (relative Frobenius norms against the oracle's
restatement of Eigen's blocked LLT):
  - factor of G G^T/n + I (kappa ~ 10): <= 1e-12;
  - factor of a Householder-spectrum matrix with condition number kappa: <= n * u * sqrt(kappa),
    u = 2^-53 (the first-order bound on a Cholesky factor's forward error);
  - graded D (G G^T/n + I) D with D spanning 1e-100 .. 1e100: the row-scaled factor D^-1 L within
    1e-12 (L = D L_M, and the slicing scales each row and column by its own power of two);
  - normwise backward error of the solve: <= 1e-15 (1e-14 at n = 16384, kappa = 1e6);
  - a factor whose columns are graded (A = L_M E^2 L_M^T): ||A - L L^T||_F / ||A||_F within 10x of
    the oracle's and <= 4 n u;
  - failing column (info): exact.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel, tri

pytestmark = pytest.mark.gpu

U = 2.0 ** -53


def _poison_other(a, uplo, value=-777.25):
    n = a.shape[0]
    other = np.triu_indices(n, 1) if uplo == "L" else np.tril_indices(n, -1)
    a[other] = value
    return other


@pytest.mark.parametrize("n", [1025, 1280, 2049, 4097])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_tensor_path_factor_matches_oracle(oracle, gbllt, n, uplo):
    a = np.asfortranarray(oracle.gen_gram(n, seed=100 + n))
    other = _poison_other(a, uplo)
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, uplo) == 0
    f = np.array(a, order="F", copy=True)
    assert gbllt.potrf(f, uplo) == 0
    assert np.all(f[other] == -777.25)  # the other triangle comes back bit-identical
    assert rel(tri(f, uplo), tri(ref, uplo)) <= 1e-12
    k = 3
    b = np.asfortranarray(oracle.normal(7, n * k).reshape(n, k, order="F"))
    x = np.array(b, order="F", copy=True)
    gbllt.potrs(f, x, uplo)
    assert oracle.backward_error(a, x, b, uplo) <= 1e-15


@pytest.mark.parametrize("n", [1280, 2049])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_tensor_path_row_major(oracle, gbllt, n, uplo):
    a = oracle.gen_gram(n, seed=200 + n)
    arow = np.ascontiguousarray(a)  # row-major storage of the same symmetric matrix
    info = ctypes.c_int64(-5)
    rc = gbllt.lib().gbllt_dpotrf(gbllt.ROW_MAJOR, uplo.encode(), n, arow.ctypes.data, n, ctypes.byref(info))
    assert rc == 0 and info.value == 0
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, uplo) == 0
    # row-major element (i, j) is arow[i, j]: the same triangle of the same matrix as column-major
    assert rel(tri(arow, uplo), tri(ref, uplo)) <= 1e-12


@pytest.mark.parametrize("n,kappa", [(2049, 1e6), (4097, 1e4)])
def test_tensor_path_householder_spectrum(oracle, gbllt, n, kappa):
    a = oracle.gen_householder(n, kappa)
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, "L") == 0
    f = np.array(a, order="F", copy=True)
    assert gbllt.potrf(f, "L") == 0
    assert rel(np.tril(f), np.tril(ref)) <= n * U * np.sqrt(kappa)
    b = np.asfortranarray(oracle.normal(8, n * 2).reshape(n, 2, order="F"))
    x = np.array(b, order="F", copy=True)
    gbllt.potrs(f, x, "L")
    assert oracle.backward_error(a, x, b) <= 1e-15


@pytest.mark.parametrize("k", [0, 255, 256, 700, 1500])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_tensor_path_failing_column(oracle, gbllt, k, uplo):
    # the failing pivot is reached after k columns of tensor-core updates (n = 2048 >= 1024)
    n = 2048
    a = oracle.gen_gram(n, seed=5)
    a[k, k] = -1.0
    ref = np.array(a, order="F")
    assert oracle.blocked(ref) == k
    f = np.array(a, order="F")
    assert gbllt.potrf(f, uplo) == k + 1


@pytest.mark.parametrize("k", [300, 1000, 4400])
def test_tensor_path_failing_column_lookahead(oracle, gbllt, k):
    # from n = 4096 the trailing updates run one panel ahead on a side stream: a failing pivot there
    # stops the updates still queued and reports the oracle's column
    n = 4500
    a = oracle.gen_gram(n, seed=6)
    a[k, k] = -1.0
    assert oracle.blocked(np.array(a, order="F")) == k
    for uplo in ("L", "U"):
        f = np.array(a, order="F")
        assert gbllt.potrf(f, uplo) == k + 1


def test_tensor_path_loses_definiteness_mid_factorisation(oracle, gbllt):
    # A = G G^T/n + s I with s just below -lambda_min(G G^T/n) at a late column: the failure comes
    # from the accumulated trailing updates, not from an input diagonal entry
    n = 1536
    g = np.asfortranarray(oracle.normal(9, n * n).reshape(n, n, order="F"))
    m = g[:, : n // 2] @ g[:, : n // 2].T / n  # rank n/2: semidefinite
    a = np.asfortranarray(m - 1e-3 * np.eye(n))
    want = oracle.blocked(np.array(a, order="F"))
    assert want >= 256  # the break-down happens after several tensor-core panels
    for uplo in ("L", "U"):
        f = np.array(a, order="F")
        assert gbllt.potrf(f, uplo) == want + 1


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_tensor_path_graded_matrix(oracle, gbllt, uplo):
    # D (G G^T/n + I) D, D log-spaced over 1e-100 .. 1e100 in a random order: entries span 1e-200 ..
    # 1e200 and every panel mixes rows of wildly different scale
    n = 2049
    m = oracle.gen_gram(n, seed=33)
    d = 10.0 ** np.linspace(-100, 100, n)
    d = d[np.random.default_rng(34).permutation(n)]
    a = np.asfortranarray(d[:, None] * m * d[None, :])
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, uplo) == 0
    f = np.array(a, order="F", copy=True)
    assert gbllt.potrf(f, uplo) == 0
    # L = D L_M (lower), U = L^T: compare the factor with its rows (columns for U) scaled back
    if uplo == "L":
        fs, rs = np.tril(f) / d[:, None], np.tril(ref) / d[:, None]
    else:
        fs, rs = np.triu(f) / d[None, :], np.triu(ref) / d[None, :]
    assert np.all(np.isfinite(fs))
    assert rel(fs, rs) <= 1e-12


def test_tensor_path_column_graded_reconstruction(oracle, gbllt):
    # A = L_M E^2 L_M^T: the factor's columns are scaled by E (1e-4 .. 1e4, random order), so each row
    # of a panel mixes entries of very different size and the slicing's per-row scale is set by the
    # largest.  The factor of such a matrix is ill-determined in its small columns, so the check is
    # backward stability: ||A - L L^T||_F / ||A||_F within 10x of the oracle's own and below 4 n u.
    n = 1536
    lm = np.tril(oracle.normal(35, n * n).reshape(n, n)) / np.sqrt(n)
    np.fill_diagonal(lm, 1.0 + np.abs(np.diag(lm)))
    e = 10.0 ** np.linspace(-4, 4, n)
    e = e[np.random.default_rng(36).permutation(n)]
    lt = lm * e[None, :]
    a = np.asfortranarray(lt @ lt.T)
    a = np.asfortranarray((a + a.T) / 2)
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, "L") == 0
    f = np.array(a, order="F", copy=True)
    assert gbllt.potrf(f, "L") == 0
    na = np.linalg.norm(a)
    r_ref = np.linalg.norm(a - np.tril(ref) @ np.tril(ref).T) / na
    r_gpu = np.linalg.norm(a - np.tril(f) @ np.tril(f).T) / na
    assert r_gpu <= max(10 * r_ref, 1e-16) and r_gpu <= 4 * n * U


@pytest.mark.parametrize("n,k", [(2048, 16), (2100, 70), (4097, 33)])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_tensor_path_blocked_solve(oracle, gbllt, n, k, uplo):
    # from n = 2048 and 16 right-hand sides the FP64 solve runs in 256-row panels: the look-back sweep
    # on each diagonal block and FP64-exact tensor-core products for the rest of the right-hand sides
    a = oracle.gen_householder(n, 1e4)
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, uplo) == 0  # the oracle's factor: the solves are compared on the same L
    b = np.asfortranarray(oracle.normal(40, n * k).reshape(n, k, order="F"))
    x = np.array(b, order="F", copy=True)
    gbllt.potrs(f, x, uplo)
    xr = np.array(b, order="F", copy=True)
    oracle.potrs(f, xr, uplo)
    assert rel(x, xr) <= 1e-12
    cols = [0, k // 2, k - 1]
    assert oracle.backward_error(a, np.asfortranarray(x[:, cols]), np.asfortranarray(b[:, cols]), uplo) <= 1e-15


@pytest.mark.slow
def test_tensor_path_full_size_config2_factor(oracle, gbllt):
    """n = 16384, 64 RHS, Householder spectrum with kappa = 1e6 (full size): the factor against the
    oracle's, and the backward error of every right-hand side."""
    torch = pytest.importorskip("torch")
    n, k, kappa = 16384, 64, 1e6
    a = oracle.gen_householder(n, kappa)
    b = np.asfortranarray(oracle.normal(12, n * k).reshape(k, n).T)
    d = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # = A (symmetric), column-major view
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    info = torch.zeros(1, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    gbllt.potrf_dev(d, n, n, info, "L", s)
    gbllt.potrs_dev(d, n, n, db, k, n, "L", s)
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    fg = d.cpu().numpy().T  # column-major factor
    ref = np.array(a, order="F", copy=True)
    assert oracle.potrf(ref, "L") == 0
    assert rel(np.tril(fg), np.tril(ref)) <= n * U * np.sqrt(kappa)
    # every right-hand side: an FP64 residual on the GPU (cuBLAS, independent of this library) ...
    A = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    X = db.T
    B = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    be_all = float(torch.linalg.norm(A @ X - B) / (torch.linalg.norm(A) * torch.linalg.norm(X)))
    assert be_all <= 1e-14
    # ... and three of them in the oracle's double-double residual
    x = np.asfortranarray(db.cpu().numpy().T)
    cols = [0, 31, 63]
    assert oracle.backward_error(a, np.asfortranarray(x[:, cols]), np.asfortranarray(b[:, cols])) <= 1e-14
