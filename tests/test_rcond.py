"""Condition estimate of the LLT path: LLT::rcond() (Eigen/src/Cholesky/LLT.h:166-171).

Pinned by Eigen's own rcond() values (tests/golden/rcond_golden.npz, from
tests/golden/make_rcond_golden.py).  The oracle restates the 1-norm of LLT::compute (LLT.h:443-453)
and the estimator (Eigen/src/Core/ConditionEstimator.h:56-171); the GPU entry points
gbllt_?lansy_l1_dev and gbllt_?pocon[_dev] are compared with both.  Eigen's own test accepts an
estimate within a factor of 10 of the true reciprocal condition number (test/cholesky.cpp:94-99);
the estimates here must match Eigen's to rounding.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import gbllt as G

GOLDEN = Path(__file__).resolve().parent / "golden" / "rcond_golden.npz"
KIND_NAMES = {0: "gram", 1: "householder", 2: "eigen"}


def make_input(oracle, kind, n, seed):
    if kind == "gram":
        return oracle.gen_gram(n, seed=seed)
    if kind == "householder":
        return oracle.gen_householder(n, 1e4, v_seed0=seed)
    s = np.zeros((n, n))
    for r in range(4):
        g = (2.0 * oracle.uniform(seed, n * n, offset=r * n * n) - 1.0).reshape(n, n, order="F")
        s += g @ g.T
    return np.asfortranarray(s)


def golden_cases():
    z = np.load(GOLDEN)
    out = []
    for m, r in zip(z["meta"], z["rcond"]):
        kind, n, seed, dt, up = (int(v) for v in m)
        out.append(dict(kind=KIND_NAMES[kind], n=n, seed=seed, dtype=np.float64 if dt == 0 else np.float32,
                        uplo="U" if up else "L", rcond=float(r)))
    return out


CASES = golden_cases()
IDS = [f"{c['kind']}-{c['n']}-{'d' if c['dtype'] == np.float64 else 's'}{c['uplo']}" for c in CASES]


def _factor(oracle, c):
    a = np.asfortranarray(make_input(oracle, c["kind"], c["n"], c["seed"]).astype(c["dtype"]))
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, c["uplo"]) == 0
    return a, f


def _tol(c):
    return 1e-9 if c["dtype"] == np.float64 else 2e-3


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_rcond_matches_eigen(oracle, c):
    a, f = _factor(oracle, c)
    anorm = oracle.sym_l1_norm(a, c["uplo"])
    full = np.tril(a) + np.tril(a, -1).T if c["uplo"] == "L" else np.triu(a) + np.triu(a, 1).T
    assert abs(anorm - np.abs(full.astype(np.float64)).sum(0).max()) <= 1e-6 * anorm
    r = oracle.rcond(f, anorm, c["uplo"])
    assert abs(r - c["rcond"]) <= _tol(c) * c["rcond"]
    # within a factor of 10 of the truth, as Eigen's own test requires
    true = 1.0 / (np.abs(full.astype(np.float64)).sum(0).max() * np.abs(np.linalg.inv(full.astype(np.float64))).sum(0).max())
    assert true / 10 <= r <= true * 10


def test_oracle_rcond_edge_cases(oracle):
    assert oracle.rcond(np.zeros((0, 0), order="F"), 1.0) == float("inf")
    assert oracle.rcond(np.ones((2, 2), order="F"), 0.0) == 0.0
    assert oracle.rcond(np.full((1, 1), 3.0, order="F"), 9.0) == 1.0


def test_pocon_argument_errors_and_trivial_cases():
    L = G.lib()
    a = np.eye(4, order="F")
    r = ctypes.c_double(-1)
    assert L.gbllt_dpocon(9, b"L", 4, a.ctypes.data, 4, 1.0, ctypes.byref(r)) == -1
    assert L.gbllt_dpocon(G.COL_MAJOR, b"x", 4, a.ctypes.data, 4, 1.0, ctypes.byref(r)) == -2
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", -1, a.ctypes.data, 4, 1.0, ctypes.byref(r)) == -3
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 4, None, 4, 1.0, ctypes.byref(r)) == -4
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 4, a.ctypes.data, 3, 1.0, ctypes.byref(r)) == -5
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, -1.0, ctypes.byref(r)) == -6
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, float("nan"), ctypes.byref(r)) == -6
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, 1.0, None) == -7
    assert L.gbllt_dpocon_dev(b"L", 4, 1, 3, 1.0, ctypes.byref(r), None) == -4
    assert L.gbllt_dlansy_l1_dev(b"L", 4, 1, 4, None, None) == -5
    # the cases ConditionEstimator.h:165-167 answers without the factor need no device
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 0, None, 1, 1.0, ctypes.byref(r)) == 0 and r.value == float("inf")
    assert L.gbllt_dpocon(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, 0.0, ctypes.byref(r)) == 0 and r.value == 0.0
    assert L.gbllt_dpocon(G.COL_MAJOR, b"U", 1, a.ctypes.data, 1, 2.0, ctypes.byref(r)) == 0 and r.value == 1.0


def test_pocon_needs_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = ctypes.c_double(-1)
    a = np.eye(4, order="F")
    assert G.lib().gbllt_dpocon(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, 1.0, ctypes.byref(r)) == G.ERR_NO_DEVICE


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_pocon_matches_eigen(oracle, c):
    a, f = _factor(oracle, c)
    anorm = oracle.sym_l1_norm(a, c["uplo"])
    r_host = G.pocon(f, anorm, c["uplo"])
    assert abs(r_host - c["rcond"]) <= _tol(c) * c["rcond"]
    # the same factor stored row-major
    ft = np.ascontiguousarray(f)  # same values, C order: seen row-major it is f
    r = ctypes.c_double(0) if c["dtype"] == np.float64 else ctypes.c_float(0)
    fn = G.lib().gbllt_dpocon if c["dtype"] == np.float64 else G.lib().gbllt_spocon
    assert fn(G.ROW_MAJOR, c["uplo"].encode(), c["n"], ft.ctypes.data, c["n"], anorm, ctypes.byref(r)) == 0
    assert abs(r.value - c["rcond"]) <= _tol(c) * c["rcond"]


@pytest.mark.gpu
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [1, 31, 33, 500, 2049])
def test_gpu_lansy_and_pocon_dev(oracle, uplo, dt, n):
    torch = pytest.importorskip("torch")
    a = np.asfortranarray(oracle.gen_householder(n, 1e3, v_seed0=5).astype(dt)) if n > 1 else np.full((1, 1), 2.0, dt)
    # poison the other triangle: neither entry point may read it
    other = np.triu_indices(n, 1) if uplo == "L" else np.tril_indices(n, -1)
    a[other] = np.asarray(1e30, dtype=dt)
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, uplo) == 0
    tdt = torch.float64 if dt == np.float64 else torch.float32
    da = torch.from_numpy(a.T.copy()).to("cuda", tdt)   # row-major copy of a^T = column-major a
    df = torch.from_numpy(f.T.copy()).to("cuda", tdt)
    dn = torch.zeros(1, dtype=tdt, device="cuda")
    G.lansy_l1_dev(da, n, n, dn, uplo, None, dt)
    want = oracle.sym_l1_norm(a, uplo)
    assert abs(float(dn.item()) - want) <= (1e-13 if dt == np.float64 else 1e-5) * want
    r = G.pocon_dev(df, n, n, float(dn.item()), uplo, None, dt)
    rr = oracle.rcond(f, float(dn.item()), uplo)
    assert abs(r - rr) <= (1e-9 if dt == np.float64 else 2e-3) * rr
