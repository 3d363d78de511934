"""BLAS level 3 of the Cholesky path: SYRK and TRSM (Eigen's blas/level3_impl.h:78-160, 355-417).

Pinned by Eigen's own BLAS (tests/golden/blas_golden.npz, from tests/golden/make_blas_golden.py,
which compiles blas/double.cpp + single.cpp + xerbla.cpp where they lie): the oracle's restatements
(oracle.syrk, oracle.trsm) must reproduce every case -- each uplo / trans for SYRK with beta = 0
(C's input triangle NaN-poisoned, so it must not be read), 1 and other values; each side / uplo /
trans / diag for TRSM with the other triangle of A filled with 1e30 (it must not be read) -- to
1e-13 (double) / 1e-5 (float).  The GPU entry points gbllt_?syrk[_dev] / gbllt_?trsm[_dev] and the
Fortran routines dsyrk_/ssyrk_/dtrsm_/strsm_ must match the same fixtures and the oracle at larger
sizes; the other triangle of C is untouched.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import gbllt as G

GOLDEN = Path(__file__).resolve().parent / "golden" / "blas_golden.npz"


def _oracle_module():
    import sys
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import oracle
    return oracle


def _load():
    sys_o = _oracle_module()
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_blas_golden", Path(__file__).resolve().parent / "golden" /
                                                  "make_blas_golden.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    z = np.load(GOLDEN)
    syrk, trsm = [], []
    for i, m in enumerate(z["syrk_meta"]):
        up, tr, n, k, dt, sd = (int(v) for v in m)
        alpha, beta = (float(v) for v in z["syrk_ab"][i])
        uplo, trans = "U" if up else "L", "T" if tr else "N"
        dtype = np.float64 if dt == 0 else np.float32
        syrk.append(dict(uplo=uplo, trans=trans, n=n, k=k, alpha=alpha, beta=beta, dtype=dtype, seed=sd,
                         want=z["syrk_vals"][z["syrk_off"][i]:z["syrk_off"][i + 1]]))
    for i, m in enumerate(z["trsm_meta"]):
        sd_, up, tr, dg, mm, nn, dt, sd = (int(v) for v in m)
        dtype = np.float64 if dt == 0 else np.float32
        trsm.append(dict(side="R" if sd_ else "L", uplo="U" if up else "L", trans="T" if tr else "N",
                         diag="U" if dg else "N", m=mm, n=nn, alpha=float(z["trsm_alpha"][i]), dtype=dtype, seed=sd,
                         want=z["trsm_vals"][z["trsm_off"][i]:z["trsm_off"][i + 1]].reshape(mm, nn, order="F")))
    return gen, syrk, trsm


GEN, SYRK, TRSM = _load()
SYRK_IDS = [f"{c['uplo']}{c['trans']}-{c['n']}x{c['k']}-a{c['alpha']}-b{c['beta']}-"
            f"{'d' if c['dtype'] == np.float64 else 's'}" for c in SYRK]
TRSM_IDS = [f"{c['side']}{c['uplo']}{c['trans']}{c['diag']}-{c['m']}x{c['n']}-a{c['alpha']}-"
            f"{'d' if c['dtype'] == np.float64 else 's'}" for c in TRSM]


def _tol(dtype):
    return 1e-13 if dtype == np.float64 else 1e-5


def _rel(got, want):
    den = np.linalg.norm(want)
    return np.linalg.norm(got - want) / (den if den > 0 else 1.0)


def _tri_idx(uplo, n):
    return np.tril_indices(n) if uplo == "L" else np.triu_indices(n)


def _syrk_in(c):
    return GEN.syrk_inputs(c["uplo"], c["trans"], c["n"], c["k"], c["beta"], c["dtype"], c["seed"])


def _trsm_in(c):
    return GEN.trsm_inputs(c["side"], c["uplo"], c["m"], c["n"], c["dtype"], c["seed"])


# ---- oracle against Eigen's BLAS ----------------------------------------------------------------

@pytest.mark.parametrize("c", SYRK, ids=SYRK_IDS)
def test_oracle_syrk_matches_eigen(oracle, c):
    a, cc = _syrk_in(c)
    oracle.syrk(cc, a, c["uplo"], c["trans"], c["alpha"], c["beta"])
    got = cc[_tri_idx(c["uplo"], c["n"])].astype(np.float64)
    assert np.all(np.isfinite(got))
    assert _rel(got, c["want"]) <= _tol(c["dtype"])


@pytest.mark.parametrize("c", TRSM, ids=TRSM_IDS)
def test_oracle_trsm_matches_eigen(oracle, c):
    a, b = _trsm_in(c)
    oracle.trsm(b, a, c["side"], c["uplo"], c["trans"], c["diag"], c["alpha"])
    assert _rel(b.astype(np.float64), c["want"]) <= _tol(c["dtype"])


# ---- argument checks (CPU) ----------------------------------------------------------------------

def test_blas_c_abi_argument_errors():
    L = G.lib()
    a = np.eye(4, order="F")
    c = np.eye(4, order="F")
    # gbllt_dsyrk(layout, uplo, trans, n, k, alpha, a, lda, beta, c, ldc): positions shift by one
    assert L.gbllt_dsyrk(7, b"L", b"N", 4, 4, 1.0, a.ctypes.data, 4, 0.0, c.ctypes.data, 4) == -1
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"X", b"N", 4, 4, 1.0, a.ctypes.data, 4, 0.0, c.ctypes.data, 4) == -2
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"L", b"X", 4, 4, 1.0, a.ctypes.data, 4, 0.0, c.ctypes.data, 4) == -3
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"L", b"N", -1, 4, 1.0, a.ctypes.data, 4, 0.0, c.ctypes.data, 4) == -4
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"L", b"N", 4, -1, 1.0, a.ctypes.data, 4, 0.0, c.ctypes.data, 4) == -5
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"L", b"N", 4, 4, 1.0, a.ctypes.data, 3, 0.0, c.ctypes.data, 4) == -8
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"L", b"T", 4, 2, 1.0, a.ctypes.data, 1, 0.0, c.ctypes.data, 4) == -8
    assert L.gbllt_dsyrk(G.COL_MAJOR, b"L", b"N", 4, 4, 1.0, a.ctypes.data, 4, 0.0, c.ctypes.data, 3) == -11
    assert L.gbllt_dsyrk_dev(b"L", b"N", 4, 4, 1.0, 1, 4, 0.0, 1, 2, None) == -10
    # gbllt_dtrsm(layout, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb)
    b = np.ones((4, 3), order="F")
    args = lambda **kw: [kw.get("layout", G.COL_MAJOR), kw.get("side", b"L"), kw.get("uplo", b"L"),
                         kw.get("tr", b"N"), kw.get("diag", b"N"), kw.get("m", 4), kw.get("n", 3), 1.0,
                         a.ctypes.data, kw.get("lda", 4), b.ctypes.data, kw.get("ldb", 4)]
    assert L.gbllt_dtrsm(*args(layout=5)) == -1
    assert L.gbllt_dtrsm(*args(side=b"X")) == -2
    assert L.gbllt_dtrsm(*args(uplo=b"X")) == -3
    assert L.gbllt_dtrsm(*args(tr=b"X")) == -4
    assert L.gbllt_dtrsm(*args(diag=b"X")) == -5
    assert L.gbllt_dtrsm(*args(m=-1)) == -6
    assert L.gbllt_dtrsm(*args(n=-1)) == -7
    assert L.gbllt_dtrsm(*args(lda=3)) == -10
    assert L.gbllt_dtrsm(*args(side=b"R", lda=2)) == -10
    assert L.gbllt_dtrsm(*args(ldb=3)) == -12
    assert L.gbllt_dtrsm(*args(m=0)) == 0 and L.gbllt_dsyrk(G.COL_MAJOR, b"U", b"T", 0, 5, 1.0, None, 5, 0.0,
                                                            None, 1) == 0


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_fortran_blas_argument_errors_go_through_xerbla(capfd, dt):
    p = "D" if dt == np.float64 else "S"
    a = np.eye(4, dtype=dt, order="F")
    c = np.eye(4, dtype=dt, order="F")
    assert G.blas_syrk(c, a, "X") == 0  # the reference's xerbla_ returns 0
    assert G.blas_syrk(c, a, "L", "Q") == 0
    assert G.blas_syrk(c, a, "L", "N", n=-1) == 0
    assert G.blas_syrk(c, a, "L", "N", k=-2) == 0
    assert G.blas_syrk(c, a, "L", "N", lda=3) == 0
    assert G.blas_syrk(c, a, "L", "N", ldc=3) == 0
    b = np.ones((4, 2), dtype=dt, order="F")
    assert G.blas_trsm(b, a, "X") == 0
    assert G.blas_trsm(b, a, "L", "X") == 0
    assert G.blas_trsm(b, a, "L", "L", "X") == 0
    assert G.blas_trsm(b, a, "L", "L", "N", "X") == 0
    assert G.blas_trsm(b, a, "L", "L", "N", "N", m=-1) == 0
    assert G.blas_trsm(b, a, "L", "L", "N", "N", n=-1) == 0
    assert G.blas_trsm(b, a, "L", "L", "N", "N", lda=3) == 0
    assert G.blas_trsm(b, a, "L", "L", "N", "N", ldb=3) == 0
    out = capfd.readouterr().out
    for i in (1, 2, 3, 4, 7, 10):
        assert f"Eigen BLAS ERROR #{i}: {p}SYRK " in out
    for i in (1, 2, 3, 4, 5, 6, 9, 11):
        assert f"Eigen BLAS ERROR #{i}: {p}TRSM " in out
    assert np.array_equal(c, np.eye(4, dtype=dt)) and np.array_equal(b, np.ones((4, 2), dtype=dt))


# ---- GPU ----------------------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("c", SYRK, ids=SYRK_IDS)
def test_gpu_syrk_matches_eigen(c):
    a, cc = _syrk_in(c)
    orig = cc.copy(order="F")
    G.syrk(cc, a, c["uplo"], c["trans"], c["alpha"], c["beta"])
    got = cc[_tri_idx(c["uplo"], c["n"])].astype(np.float64)
    assert np.all(np.isfinite(got))
    assert _rel(got, c["want"]) <= _tol(c["dtype"])
    other = np.triu(np.ones(cc.shape, bool), 1) if c["uplo"] == "L" else np.tril(np.ones(cc.shape, bool), -1)
    assert np.array_equal(cc[other], orig[other])
    # and through the Fortran routine
    a2, c2 = _syrk_in(c)
    assert G.blas_syrk(c2, a2, c["uplo"], c["trans"], c["alpha"], c["beta"]) == 0
    assert _rel(c2[_tri_idx(c["uplo"], c["n"])].astype(np.float64), c["want"]) <= _tol(c["dtype"])


@pytest.mark.gpu
@pytest.mark.parametrize("c", TRSM, ids=TRSM_IDS)
def test_gpu_trsm_matches_eigen(c):
    a, b = _trsm_in(c)
    G.trsm(b, a, c["side"], c["uplo"], c["trans"], c["diag"], c["alpha"])
    tol = 1e-12 if c["dtype"] == np.float64 else 1e-5
    assert _rel(b.astype(np.float64), c["want"]) <= tol
    a2, b2 = _trsm_in(c)
    assert G.blas_trsm(b2, a2, c["side"], c["uplo"], c["trans"], c["diag"], c["alpha"]) == 0
    assert _rel(b2.astype(np.float64), c["want"]) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,k", [(1000, 64), (777, 300), (2049, 129)])
def test_gpu_syrk_sizes(oracle, uplo, trans, n, k):
    ar, ac = (n, k) if trans == "N" else (k, n)
    a = np.asfortranarray(oracle.normal(n + k, ar * ac).reshape(ar, ac, order="F"))
    c0 = np.asfortranarray(oracle.normal(n + k + 1, n * n).reshape(n, n, order="F"))
    want = c0.copy(order="F")
    oracle.syrk(want, a, uplo, trans, -1.0, 0.5)
    got = c0.copy(order="F")
    G.syrk(got, a, uplo, trans, -1.0, 0.5)
    idx = _tri_idx(uplo, n)
    assert _rel(got[idx], want[idx]) <= 1e-13
    # device entry on torch buffers (column-major = transposed row-major storage)
    torch = pytest.importorskip("torch")
    da = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    dc = torch.from_numpy(np.ascontiguousarray(c0.T)).cuda()
    G.check("dsyrk_dev", G.lib().gbllt_dsyrk_dev(uplo.encode(), trans.encode(), n, k, -1.0, da.data_ptr(), ar, 0.5,
                                                 dc.data_ptr(), n, None))
    torch.cuda.synchronize()
    gd = np.asfortranarray(dc.cpu().numpy().T)
    assert _rel(gd[idx], want[idx]) <= 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_gpu_trsm_sizes(oracle, side, uplo, trans, diag):
    m, n = (1100, 70) if side == "L" else (70, 1100)
    a, b = GEN.trsm_inputs(side, uplo, m, n, np.float64, 9)
    want = b.copy(order="F")
    oracle.trsm(want, a, side, uplo, trans, diag, 0.75)
    got = b.copy(order="F")
    G.trsm(got, a, side, uplo, trans, diag, 0.75)
    assert _rel(got, want) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_gpu_blas_row_major(oracle, dt):
    n, k = 150, 40
    a = oracle.normal(3, n * k).reshape(n, k).astype(dt)  # row-major n x k
    c = oracle.normal(4, n * n).reshape(n, n).astype(dt)
    want = np.asfortranarray(c.copy())
    oracle.syrk(want, np.asfortranarray(a), "L", "N", 2.0, 1.0)
    got = np.ascontiguousarray(c.copy())
    fn = G.lib().gbllt_dsyrk if dt == np.float64 else G.lib().gbllt_ssyrk
    assert fn(G.ROW_MAJOR, b"L", b"N", n, k, 2.0, a.ctypes.data, k, 1.0, got.ctypes.data, n) == 0
    tol = 1e-13 if dt == np.float64 else 1e-5
    assert _rel(np.tril(got), np.tril(want)) <= tol
    assert np.array_equal(np.triu(got, 1), np.triu(c, 1))
    at, bt = GEN.trsm_inputs("L", "U", n, 9, dt, 5)
    want = bt.copy(order="F")
    oracle.trsm(want, at, "L", "U", "T", "N", 1.0)
    arow, brow = np.ascontiguousarray(at), np.ascontiguousarray(bt)
    ft = G.lib().gbllt_dtrsm if dt == np.float64 else G.lib().gbllt_strsm
    assert ft(G.ROW_MAJOR, b"L", b"U", b"T", b"N", n, 9, 1.0, arow.ctypes.data, n, brow.ctypes.data, 9) == 0
    assert _rel(brow, want) <= (1e-12 if dt == np.float64 else 1e-5)
