"""Generate tests/golden/llt_golden.npz from Eigen's own LLT.

Run where the reference sources are present (it builds oracle/_ref/libeigen_ref.so from the
Eigen headers in place, see oracle/Makefile):

    python tests/golden/make_golden.py

Inputs are regenerated from seeds by the oracle's Philox generator; the fixture stores, per
case, the seeds, checksums of the input, Eigen's factor (packed triangle), Eigen's solution for
a seeded right-hand side, and the failing column reported by llt_inplace::blocked.  The calls go
through Eigen's public API: LLT<Matrix,UpLo>(A), .info(), .solve(B), .matrixLLT()
(Eigen/src/Cholesky/LLT.h:104-110, 191-195, 483-498), and llt_inplace<T,UpLo>::blocked
(LLT.h:338-399) for the failing column.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "llt_golden.npz"


def eigen_style(n: int, seed: int) -> np.ndarray:
    """symm = a0 a0^T + sum_{3} a1 a1^T with uniform[-1,1] entries (test/cholesky.cpp:69-78)."""
    s = np.zeros((n, n))
    for r in range(4):
        g = (2.0 * O.uniform(seed, n * n, offset=r * n * n) - 1.0).reshape(n, n, order="F")
        s += g @ g.T
    return np.asfortranarray(s)


def make_input(kind: str, n: int, seed: int) -> np.ndarray:
    if kind == "gram":
        return O.gen_gram(n, seed=seed)
    if kind == "eigen":
        return eigen_style(n, seed)
    if kind.startswith("fail"):
        a = O.gen_gram(n, seed=seed)
        k = int(kind[4:])
        a[k, k] = -1.0
        return a
    if kind == "neg":
        return np.asfortranarray(-O.gen_gram(n, seed=seed))
    raise ValueError(kind)


CASES = []
for n in [1, 2, 3, 4, 5, 8, 16, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 200, 257]:
    CASES.append(("gram", n, 1, "d", "L"))
for n in [3, 40, 129]:
    CASES.append(("gram", n, 1, "d", "U"))
for n in [7, 50, 150]:
    CASES.append(("eigen", n, 5, "d", "L"))
    CASES.append(("eigen", n, 5, "d", "U"))
for n in [5, 33, 100, 200]:
    CASES.append(("gram", n, 1, "s", "L"))
CASES.append(("gram", 70, 1, "s", "U"))
for k in [0, 17, 63, 64, 99]:
    CASES.append((f"fail{k}", 100, 1, "d", "L"))
CASES.append(("fail130", 200, 1, "d", "L"))
CASES.append(("fail130", 200, 1, "d", "U"))
CASES.append(("fail40", 64, 1, "s", "L"))
CASES.append(("neg", 50, 1, "d", "L"))


def main() -> None:
    O.build(ref=True)
    R = O.eigen_ref()
    assert R is not None, "Eigen reference library was not built"
    store = {}
    for idx, (kind, n, seed, dt, uplo) in enumerate(CASES):
        dtype = np.float64 if dt == "d" else np.float32
        a64 = make_input(kind, n, seed)
        a = np.asfortranarray(a64.astype(dtype))
        nrhs = 3
        b = np.asfortranarray(O.normal(2, n * nrhs).reshape(nrhs, n).T.astype(dtype))
        # failing column from llt_inplace::blocked on a copy
        c = np.array(a, order="F", copy=True)
        fn = R.ref_dblocked if dt == "d" else R.ref_sblocked
        fail = int(fn(uplo.encode(), n, c.ctypes.data, max(1, n)))
        f = np.array(a, order="F", copy=True)
        x = np.array(b, order="F", copy=True)
        sec = (ctypes.c_double * 2)()
        fn2 = R.ref_dllt if dt == "d" else R.ref_sllt
        info = int(fn2(uplo.encode(), n, nrhs, f.ctypes.data, max(1, n), x.ctypes.data, max(1, n), sec))
        tri = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
        p = f"c{idx:03d}_"
        store[p + "meta"] = np.array([n, seed, nrhs, fail, info], dtype=np.int64)
        store[p + "kind"] = np.array(kind)
        store[p + "dtype"] = np.array(dt)
        store[p + "uplo"] = np.array(uplo)
        store[p + "asum"] = np.array([float(np.sum(a64)), float(np.sum(np.abs(a64)))])
        if fail < 0:
            store[p + "factor"] = f[tri]
            store[p + "x"] = x
    np.savez_compressed(OUT, ncases=np.array(len(CASES)), **store)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(CASES)} cases)")


if __name__ == "__main__":
    main()
