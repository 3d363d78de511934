"""Pivoted LDL^T: LDLT<Matrix,UpLo>::compute and solve (Eigen/src/Cholesky/LDLT.h:497-613).

Pinned by Eigen's own results (tests/golden/ldlt_golden.npz, from tests/golden/make_ldlt_golden.py):
the known-answer matrices of Eigen's test/cholesky.cpp (cholesky_bug241, cholesky_definiteness,
cholesky_faillure_cases) and generated matrices of eight kinds.  The oracle's restatement of
ldlt_inplace<Lower>::unblocked (LDLT.h:297-403) must reproduce Eigen's transpositions, sign and info
exactly and its factor and solution to rounding (to the bit for a lower factor of order <= 128,
where Eigen's GEMV accumulates in one block); the GPU entry points gbllt_?ldlt[_dev] and
gbllt_?ldlt_solve[_dev] must give the same transpositions, sign and info and agree with the factor:
to the bit for a lower factor of order <= 64 (one diagonal block, computed in Eigen's order without
FMA), to 1e-12 (double) / 1e-5 (float) relative Frobenius norm otherwise.

Two kinds decide a pivot's being exactly zero by rounding noise ("wide", "lowrank": the pivots
after the numerical rank are ~1e-16 and may or may not round to 0, depending on the order of the
sums); for them sign and info are compared only where Eigen's own test compares them, and the factor
is checked through the reconstruction P^T L D L^T P = A, as test/cholesky.cpp:224-265 does.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import gbllt as G

GOLDEN = Path(__file__).resolve().parent / "golden" / "ldlt_golden.npz"
ROUNDING_KINDS = ("wide", "lowrank")


def _cases(oracle_mod):
    z = np.load(GOLDEN)
    out, ki = [], 0
    for i, m in enumerate(z["meta"]):
        code, n, seed, up, dt, sign, info = (int(v) for v in m)
        if code < 0:
            kind = "known"
            a = z["known"][ki:ki + n * n].reshape(n, n, order="F")
            ki += n * n
        else:
            kind = oracle_mod.LDLT_KINDS[code]
            a = oracle_mod.gen_sym(kind, n, seed)
        dtype = np.float64 if dt == 0 else np.float32
        out.append(dict(kind=kind, n=n, seed=seed, uplo="U" if up else "L", dtype=dtype,
                        a=np.asfortranarray(a.astype(dtype)), sign=sign, info=info,
                        factor=z["factors"][z["offsets"][i]:z["offsets"][i + 1]],
                        transp=z["transp"][z["toffsets"][i]:z["toffsets"][i + 1]],
                        x=z["xs"][z["toffsets"][i]:z["toffsets"][i + 1]]))
    return out


def _oracle_module():
    import sys
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import oracle
    return oracle


CASES = _cases(_oracle_module())
IDS = [f"{c['kind']}-{c['n']}-{c['uplo']}-{'d' if c['dtype'] == np.float64 else 's'}-{c['seed']}" for c in CASES]


def _pack(f, uplo):
    n = f.shape[0]
    idx = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    return f[idx].astype(np.float64)


def _tri(uplo):
    return np.tril if uplo == "L" else np.triu


def _rel(got, want):
    den = np.linalg.norm(want)
    return np.linalg.norm(got - want) / (den if den > 0 else 1.0)


def _reconstruct(f, transp, uplo):
    """P^T L D L^T P from a factor (LDLT::reconstructedMatrix, LDLT.h:636-663)."""
    n = f.shape[0]
    F = f.astype(np.float64)
    L = np.tril(F, -1) + np.eye(n) if uplo == "L" else np.triu(F, 1).T + np.eye(n)
    d = np.diag(F)
    m = (L * d) @ L.T
    for k in range(n - 1, -1, -1):  # res = P^T res: undo the swaps in reverse order
        p = transp[k]
        m[[k, p], :] = m[[p, k], :]
        m[:, [k, p]] = m[:, [p, k]]
    return m


def _pivots_replay(diag):
    """Eigen's pivot search on a diagonal (LDLT.h:323-346): first largest |d| of the corner, swap."""
    d = np.abs(np.asarray(diag, dtype=np.float64)).copy()
    n = d.shape[0]
    t = np.zeros(n, dtype=np.int32)
    for k in range(n):
        p = k + int(np.argmax(d[k:]))  # numpy's argmax returns the first maximum
        t[k] = p
        d[k], d[p] = d[p], d[k]
    return t


# ---- oracle against Eigen ----------------------------------------------------------------------

@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_ldlt_matches_eigen(oracle, c):
    f = np.array(c["a"], order="F", copy=True)
    ok, t, sign = oracle.ldlt(f, c["uplo"])
    assert np.array_equal(t, c["transp"])
    assert sign == c["sign"] and int(not ok) == c["info"]
    got = _pack(f, c["uplo"])
    if c["uplo"] == "L" and c["n"] <= 128:
        assert np.array_equal(got, c["factor"])
    else:
        tol = (1e-8 if c["kind"] == "wide" else 1e-12) if c["dtype"] == np.float64 else 1e-5
        assert _rel(got, c["factor"]) <= tol
    b = oracle.normal(c["seed"] + 7, c["n"]).astype(c["dtype"])
    oracle.ldlt_solve(f, t, b, c["uplo"])
    tol = (1e-3 if c["kind"] == "wide" else 1e-12) if c["dtype"] == np.float64 else 1e-4
    assert _rel(b.astype(np.float64), c["x"]) <= tol


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_pivot_order_host(oracle, seed, dtype):
    """The host pivot order (tournament tree) against a direct replay of Eigen's search, on
    diagonals with many ties (small integers of both signs and zeros) and on distinct values."""
    rng = np.random.default_rng(seed)
    n = [1, 2, 7, 64, 513, 2000][seed]
    diags = [rng.integers(-3, 4, n).astype(dtype), rng.standard_normal(n).astype(dtype),
             np.zeros(n, dtype), np.full(n, -2.0, dtype), np.arange(n, dtype=dtype), -np.arange(n, dtype=dtype)[::-1]]
    for d in diags:
        assert np.array_equal(G.ldlt_pivots(d), _pivots_replay(d))
    if n <= 64:  # and against the full restatement on a diagonal matrix
        a = np.asfortranarray(np.diag(diags[0]))
        _, t, _ = oracle.ldlt(a, "L")
        assert np.array_equal(G.ldlt_pivots(diags[0]), t)


def test_ldlt_argument_errors():
    L = G.lib()
    a = np.eye(4, order="F")
    t = np.zeros(4, np.int32)
    sg, info = ctypes.c_int32(0), ctypes.c_int64(0)
    P = ctypes.byref
    assert L.gbllt_dldlt(7, b"L", 4, a.ctypes.data, 4, t.ctypes.data, P(sg), P(info)) == -1
    assert L.gbllt_dldlt(G.COL_MAJOR, b"Q", 4, a.ctypes.data, 4, t.ctypes.data, P(sg), P(info)) == -2
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", -1, a.ctypes.data, 4, t.ctypes.data, P(sg), P(info)) == -3
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", 4, None, 4, t.ctypes.data, P(sg), P(info)) == -4
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", 4, a.ctypes.data, 3, t.ctypes.data, P(sg), P(info)) == -5
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, None, P(sg), P(info)) == -6
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, t.ctypes.data, None, P(info)) == -7
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, t.ctypes.data, P(sg), None) == -8
    assert L.gbllt_dldlt_dev(b"L", 4, 1, 3, t.ctypes.data, P(sg), P(info), None) == -4
    sg.value, info.value = 9, 9
    assert L.gbllt_dldlt(G.COL_MAJOR, b"L", 0, None, 1, None, P(sg), P(info)) == 0
    assert sg.value == 2 and info.value == 0  # size 0: ZeroSign, Success (LDLT.h:311-319)
    b = np.ones(4)
    bad = np.array([0, 1, 4, 3], np.int32)  # index 4 out of range
    assert L.gbllt_dldlt_solve(G.COL_MAJOR, b"L", 4, 1, a.ctypes.data, 4, bad.ctypes.data, b.ctypes.data, 4) == -7
    assert L.gbllt_dldlt_solve(G.COL_MAJOR, b"L", 4, 1, a.ctypes.data, 4, t.ctypes.data, b.ctypes.data, 3) == -9
    assert L.gbllt_dldlt_solve_dev(b"L", 4, 1, 1, 4, bad.ctypes.data, 1, 4, None) == -6
    assert L.gbllt_dldlt_pivots(-1, None, 1, None) == -1
    assert L.gbllt_dldlt_pivots(3, b.ctypes.data, 0, t.ctypes.data) == -3


# ---- GPU against Eigen and the oracle -----------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_ldlt_matches_eigen(c):
    f = np.array(c["a"], order="F", copy=True)
    info, t, sign = G.ldlt(f, c["uplo"])
    assert np.array_equal(t, c["transp"])
    other = np.triu(np.ones(f.shape, bool), 1) if c["uplo"] == "L" else np.tril(np.ones(f.shape, bool), -1)
    assert np.array_equal(f[other], c["a"][other])  # the other triangle is untouched
    got = _pack(f, c["uplo"])
    if c["kind"] in ROUNDING_KINDS:
        a = c["a"].astype(np.float64)
        tol = 1e-9 if c["kind"] == "wide" else 1e-12
        assert np.linalg.norm(_reconstruct(f, t, c["uplo"]) - a) <= tol * np.linalg.norm(a)
        return
    assert sign == c["sign"] and info == c["info"]
    if c["uplo"] == "L" and c["n"] <= 64:
        assert np.array_equal(got, c["factor"])
    else:
        assert _rel(got, c["factor"]) <= (1e-12 if c["dtype"] == np.float64 else 1e-5)
    b = _oracle_module().normal(c["seed"] + 7, c["n"]).astype(c["dtype"])
    G.ldlt_solve(f, t, b, c["uplo"])
    tol = 1e-11 if c["dtype"] == np.float64 else 1e-4
    assert _rel(b.astype(np.float64), c["x"]) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["lagrange", "lowrank", "wide"])
@pytest.mark.parametrize("n", [3, 40, 200])
def test_gpu_ldlt_consistent_solve(oracle, kind, n):
    """test/cholesky.cpp:214-265: for a right-hand side in the range of A, A x = b."""
    a = oracle.gen_sym(kind, n, n + 5)
    x0 = oracle.normal(n + 6, n)
    b = a @ x0
    f = np.array(a, order="F", copy=True)
    _, t, _ = G.ldlt(f, "L")
    x = b.copy()
    G.ldlt_solve(f, t, x, "L")
    d = np.abs(np.diag(f))
    tol = 1e-9 if d.min() > 0 else 1e-6  # the large tolerance of cholesky.cpp:268-272 with zero pivots
    if kind == "wide":
        tol = 1e-6
    assert np.linalg.norm(a @ x - b) <= tol * np.linalg.norm(b)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 127, 128, 129, 300, 1000, 2049])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("kind", ["gram", "indef"])
def test_gpu_ldlt_sizes(oracle, n, uplo, kind):
    a = oracle.gen_sym(kind, n, n + 11)
    ref = np.array(a, order="F", copy=True)
    ok, tr, sr = oracle.ldlt(ref, uplo)
    f = np.array(a, order="F", copy=True)
    info, t, sign = G.ldlt(f, uplo)
    assert np.array_equal(t, tr) and sign == sr and info == int(not ok) == 0
    tri = _tri(uplo)
    assert _rel(tri(f), tri(ref)) <= 1e-12
    if uplo == "L" and n <= 64:
        assert np.array_equal(tri(f), tri(ref))
    b = np.asfortranarray(oracle.normal(n + 12, n * 3).reshape(n, 3, order="F"))
    xr = b.copy(order="F")
    oracle.ldlt_solve(ref, tr, xr, uplo)
    x = b.copy(order="F")
    G.ldlt_solve(f, t, x, uplo)
    assert _rel(x, xr) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("nrhs", [1, 5, 17, 600])
def test_gpu_ldlt_dev_entries(oracle, uplo, nrhs):
    torch = pytest.importorskip("torch")
    n = 700
    a = oracle.gen_sym("indef", n, 3)
    ref = np.array(a, order="F", copy=True)
    ok, tr, sr = oracle.ldlt(ref, uplo)
    da = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # row-major a^T = column-major a
    info, t, sign = G.ldlt_dev(da, n, n, uplo)
    assert np.array_equal(t, tr) and sign == sr and info == 0
    f = np.asfortranarray(da.cpu().numpy().T)
    tri = _tri(uplo)
    assert _rel(tri(f), tri(ref)) <= 1e-12
    b = np.asfortranarray(oracle.normal(9, n * nrhs).reshape(n, nrhs, order="F"))
    xr = b.copy(order="F")
    oracle.ldlt_solve(ref, tr, xr, uplo)
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    G.ldlt_solve_dev(da, n, n, t, db, nrhs, n, uplo)
    torch.cuda.synchronize()
    x = np.asfortranarray(db.cpu().numpy().T)
    assert _rel(x, xr) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gpu_ldlt_row_major(oracle, dtype):
    n, k = 150, 4
    a = oracle.gen_sym("indef", n, 21).astype(dtype)
    ref = np.array(a, order="F", copy=True)
    ok, tr, sr = oracle.ldlt(ref, "L")
    # row-major storage of the same matrix: the lower triangle of a C-order array
    c = np.ascontiguousarray(a)
    t = np.zeros(n, np.int32)
    sg, info = ctypes.c_int32(0), ctypes.c_int64(0)
    fn = G.lib().gbllt_dldlt if dtype == np.float64 else G.lib().gbllt_sldlt
    assert fn(G.ROW_MAJOR, b"L", n, c.ctypes.data, n, t.ctypes.data, ctypes.byref(sg), ctypes.byref(info)) == 0
    assert np.array_equal(t, tr) and sg.value == sr and info.value == 0
    tol = 1e-12 if dtype == np.float64 else 1e-5
    assert _rel(np.tril(c), np.tril(ref)) <= tol
    b = np.ascontiguousarray(oracle.normal(22, n * k).reshape(n, k).astype(dtype))
    xr = np.asfortranarray(b)
    oracle.ldlt_solve(ref, tr, xr, "L")
    fs = G.lib().gbllt_dldlt_solve if dtype == np.float64 else G.lib().gbllt_sldlt_solve
    assert fs(G.ROW_MAJOR, b"L", n, k, c.ctypes.data, n, t.ctypes.data, b.ctypes.data, k) == 0
    assert _rel(b, xr) <= (1e-11 if dtype == np.float64 else 1e-4)


@pytest.mark.gpu
def test_gpu_ldlt_large_indefinite(oracle):
    """n = 4096: transpositions against the replayed pivot search, and the solve's backward error."""
    n = 4096
    a = oracle.gen_sym("indef", n, 5)
    f = np.array(a, order="F", copy=True)
    info, t, sign = G.ldlt(f, "L")
    assert info == 0 and sign == 3
    assert np.array_equal(t, _pivots_replay(np.diag(a)))
    b = oracle.normal(6, n)
    x = b.copy()
    G.ldlt_solve(f, t, x, "L")
    r = a @ x - b
    assert np.linalg.norm(r) <= 1e-14 * np.linalg.norm(a) * np.linalg.norm(x) * 10
