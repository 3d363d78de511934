"""Generate tests/golden/rank_update_golden.npz from Eigen's own LLT::rankUpdate.

Run where the reference sources are present (it builds oracle/_ref/libeigen_ref.so from the
Eigen headers in place, see oracle/Makefile):

    python tests/golden/make_rank_update_golden.py

Per case: A = G G^T/n + I from the oracle's Philox generator (seed), v ~ N(0,1) (seed + 100),
sigma, the triangle and the scalar type; the fixture stores Eigen's factor of A + sigma v v^T
(the `uplo` triangle packed column by column) from LLT<Matrix,UpLo>(A).rankUpdate(v, sigma)
(Eigen/src/Cholesky/LLT.h:469-478 -> llt_rank_update_lower, LLT.h:238-307) and whether Eigen
reported NumericalIssue (a downdate that leaves the matrix indefinite).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "rank_update_golden.npz"

# (n, seed, sigma, uplo, dtype)
CASES = [
    (1, 3, 2.0, "L", "d"), (2, 3, -0.25, "L", "d"), (17, 4, 1.5, "L", "d"), (64, 5, 0.75, "U", "d"),
    (65, 6, -0.05, "L", "d"), (90, 7, 3.0, "U", "d"), (100, 8, -0.01, "U", "d"), (70, 9, -0.3, "L", "d"),
    (33, 10, 0.0, "L", "d"), (50, 11, 2.0, "L", "s"), (80, 12, -0.02, "U", "s"),
]


def inputs(n, seed, dt):
    a = O.gen_gram(n, seed=seed).astype(np.float64 if dt == "d" else np.float32, order="F")
    v = O.normal(seed + 100, n).astype(a.dtype)
    return np.asfortranarray(a), v


def pack(f, uplo):
    n = f.shape[0]
    idx = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    return f[idx]


def main() -> None:
    O.build(ref=True)
    R = O.eigen_ref()
    if R is None:
        raise SystemExit("Eigen's reference LLT could not be built (reference headers missing)")
    meta, facs, offs = [], [], [0]
    for n, seed, sigma, uplo, dt in CASES:
        a, v = inputs(n, seed, dt)
        f = np.array(a, order="F", copy=True)
        fn = R.ref_drank_update if dt == "d" else R.ref_srank_update
        rc = int(fn(uplo.encode(), n, f.ctypes.data, n, v.ctypes.data, sigma))
        assert rc in (0, 1), rc
        p = pack(f, uplo).astype(np.float64)
        facs.append(p)
        offs.append(offs[-1] + p.size)
        meta.append([n, seed, 0 if uplo == "L" else 1, 0 if dt == "d" else 1, rc])
    np.savez(OUT, meta=np.array(meta, dtype=np.int64), sigma=np.array([c[2] for c in CASES]),
             factors=np.concatenate(facs), offsets=np.array(offs, dtype=np.int64))
    print(f"wrote {OUT} ({len(CASES)} cases)")


if __name__ == "__main__":
    main()
