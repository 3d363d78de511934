"""Rank-1 update / downdate of a Cholesky factor: LLT::rankUpdate (Eigen/src/Cholesky/LLT.h:469-478).

Pinned by Eigen's own results (tests/golden/rank_update_golden.npz, from
tests/golden/make_rank_update_golden.py): the oracle's restatement of llt_rank_update_lower
(LLT.h:238-307, Givens rotations for sigma > 0, the beta recurrence otherwise) must reproduce Eigen's
updated factor and its NumericalIssue reports; the GPU entry points gbllt_?rank_update[_dev] must
match the oracle (1e-12 double, 1e-4 float, relative Frobenius on the factor) and report the same
failing column of a downdate.  Eigen's own test (test/cholesky.cpp:29-56) checks the reconstruction
A + sigma v v^T within its test precision; tests/test_eigen_backend.py runs it through the header.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import gbllt as G

GOLDEN = Path(__file__).resolve().parent / "golden" / "rank_update_golden.npz"


def _cases():
    z = np.load(GOLDEN)
    out = []
    for i, (m, sigma) in enumerate(zip(z["meta"], z["sigma"])):
        n, seed, up, dt, rc = (int(v) for v in m)
        out.append(dict(n=n, seed=seed, uplo="U" if up else "L", dtype=np.float64 if dt == 0 else np.float32,
                        sigma=float(sigma), eigen_failed=bool(rc),
                        factor=z["factors"][z["offsets"][i]:z["offsets"][i + 1]]))
    return out


CASES = _cases()
IDS = [f"{c['n']}-{c['uplo']}-{'d' if c['dtype'] == np.float64 else 's'}-{c['sigma']}" for c in CASES]


def _inputs(oracle, n, seed, dtype):
    a = np.asfortranarray(oracle.gen_gram(n, seed=seed).astype(dtype))
    v = oracle.normal(seed + 100, n).astype(dtype)
    return a, v


def _tri(uplo):
    return np.tril if uplo == "L" else np.triu


def _pack(f, uplo):
    n = f.shape[0]
    idx = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    return f[idx]


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_rank_update_matches_eigen(oracle, c):
    a, v = _inputs(oracle, c["n"], c["seed"], c["dtype"])
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, c["uplo"]) == 0
    ret = oracle.rank_update(f, v, c["sigma"], c["uplo"])
    assert (ret >= 0) == c["eigen_failed"]
    tol = 1e-12 if c["dtype"] == np.float64 else 1e-4
    got = _pack(f, c["uplo"]).astype(np.float64)
    assert np.linalg.norm(got - c["factor"]) <= tol * np.linalg.norm(c["factor"])
    if not c["eigen_failed"]:
        L = _tri(c["uplo"])(f).astype(np.float64)
        L = L if c["uplo"] == "L" else L.T
        want = a.astype(np.float64) + c["sigma"] * np.outer(v, v)
        assert np.linalg.norm(L @ L.T - want) <= (1e-13 if c["dtype"] == np.float64 else 1e-5) * np.linalg.norm(want)


def test_rank_update_argument_errors():
    L = G.lib()
    a = np.eye(4, order="F")
    v = np.ones(4)
    info = ctypes.c_int64(0)
    assert L.gbllt_drank_update(7, b"L", 4, a.ctypes.data, 4, v.ctypes.data, 1.0, ctypes.byref(info)) == -1
    assert L.gbllt_drank_update(G.COL_MAJOR, b"Q", 4, a.ctypes.data, 4, v.ctypes.data, 1.0, ctypes.byref(info)) == -2
    assert L.gbllt_drank_update(G.COL_MAJOR, b"L", -1, a.ctypes.data, 4, v.ctypes.data, 1.0, ctypes.byref(info)) == -3
    assert L.gbllt_drank_update(G.COL_MAJOR, b"L", 4, a.ctypes.data, 3, v.ctypes.data, 1.0, ctypes.byref(info)) == -5
    assert L.gbllt_drank_update(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, None, 1.0, ctypes.byref(info)) == -6
    assert L.gbllt_drank_update(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, v.ctypes.data, float("nan"),
                                ctypes.byref(info)) == -7
    assert L.gbllt_drank_update(G.COL_MAJOR, b"L", 4, a.ctypes.data, 4, v.ctypes.data, 1.0, None) == -8
    assert L.gbllt_drank_update_dev(b"L", 4, 1, 4, None, 1.0, 1, None) == -5
    assert L.gbllt_drank_update(G.COL_MAJOR, b"L", 0, None, 1, None, 1.0, ctypes.byref(info)) == 0 and info.value == 0


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_rank_update_matches_oracle(oracle, c):
    a, v = _inputs(oracle, c["n"], c["seed"], c["dtype"])
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, c["uplo"]) == 0
    ref = np.array(f, order="F", copy=True)
    ret = oracle.rank_update(ref, v, c["sigma"], c["uplo"])
    g = np.array(f, order="F", copy=True)
    info = G.rank_update(g, v, c["sigma"], c["uplo"])
    assert info == (0 if ret < 0 else ret + 1)
    if ret < 0:
        tol = 1e-12 if c["dtype"] == np.float64 else 1e-4
        tri = _tri(c["uplo"])
        assert np.linalg.norm(tri(g) - tri(ref)) <= tol * np.linalg.norm(tri(ref))
        other = np.triu(np.ones(g.shape, bool), 1) if c["uplo"] == "L" else np.tril(np.ones(g.shape, bool), -1)
        assert np.array_equal(g[other], f[other])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 63, 64, 65, 129, 700, 2049])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("sigma", [2.0, 1e-3, -1e-4])
def test_gpu_rank_update_dev_sizes(oracle, n, uplo, sigma):
    torch = pytest.importorskip("torch")
    a = np.asfortranarray(oracle.gen_gram(n, seed=n + 1))
    v = oracle.normal(n + 2, n) / np.sqrt(n)
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, uplo) == 0
    ref = np.array(f, order="F", copy=True)
    assert oracle.rank_update(ref, v, sigma, uplo) == -1
    dl = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()   # row-major f^T = column-major f
    dv = torch.from_numpy(v.copy()).cuda()
    di = torch.full((1,), -7, dtype=torch.int64, device="cuda")
    G.rank_update_dev(dl, n, n, dv, sigma, di, uplo)
    torch.cuda.synchronize()
    assert int(di.item()) == 0
    g = np.asfortranarray(dl.cpu().numpy().T)
    tri = _tri(uplo)
    assert np.linalg.norm(tri(g) - tri(ref)) <= 1e-12 * np.linalg.norm(tri(ref))
    L = tri(g) if uplo == "L" else tri(g).T
    want = a + sigma * np.outer(v, v)
    assert np.linalg.norm(L @ L.T - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.gpu
def test_gpu_rank_downdate_failing_column(oracle):
    n = 300
    a = np.asfortranarray(oracle.gen_gram(n, seed=77))
    v = np.zeros(n)
    v[200] = 3.0  # A - v v^T loses positivity at column 200 exactly
    f = np.array(a, order="F", copy=True)
    assert oracle.potrf(f, "L") == 0
    ref = np.array(f, order="F", copy=True)
    ret = oracle.rank_update(ref, v, -1.0, "L")
    assert ret == 200
    g = np.array(f, order="F", copy=True)
    assert G.rank_update(g, v, -1.0, "L") == 201
