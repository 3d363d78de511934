"""Generate tests/golden/ldlt_golden.npz from Eigen's own LDLT.

Run where the reference sources are present (it builds oracle/_ref/libeigen_ref.so from the
Eigen headers in place, see oracle/Makefile):

    python tests/golden/make_ldlt_golden.py

Two groups of cases, each stored with Eigen's results for LDLT<Matrix,UpLo>(A) (LDLT.h:497-530):
the factor (the UpLo triangle of matrixLDLT(), packed column by column), the transpositions, the
sign (0 PositiveSemiDef, 1 NegativeSemiDef, 2 ZeroSign, 3 Indefinite), the info (0 Success,
1 NumericalIssue) and x = solve(b) for one right-hand side (LDLT.h:573-613):

  - the known-answer matrices of Eigen's own tests, cholesky_bug241 (test/cholesky.cpp:340-355),
    cholesky_definiteness (:358-406) and cholesky_faillure_cases (:408-469), stored as matrices;
  - generated inputs, oracle.gen_sym(kind, n, seed), stored as (kind, n, seed).
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "ldlt_golden.npz"

# test/cholesky.cpp: the 2 x 2 matrices of cholesky_bug241 and cholesky_definiteness, then the
# failure cases of cholesky_faillure_cases (the -8.9999999999999999999 entry is -9 in double).
KNOWN = [
    [[1, 1], [1, 1]],
    [[1, 0], [0, -1]],
    [[1, 2], [2, 1]],
    [[0, 0], [0, 0]],
    [[0, 0], [0, 1]],
    [[-1, 0], [0, 0]],
    [[0, 1], [1, 0]],
    [[-1, -3, 3], [-3, -9, 1], [3, 1, 0]],
    [[1, 2, 3], [2, 4, 1], [3, 1, 0]],
    [[0.1, 0, -0.1, 0, 0, 0, 1, 0],
     [0, 4.24667, 0, 2.00333, 0, 0, 0, 0],
     [-0.1, 0, 0.2, 0, -0.1, 0, 0, 0],
     [0, 2.00333, 0, 8.49333, 0, 2.00333, 0, 0],
     [0, 0, -0.1, 0, 0.1, 0, 0, 1],
     [0, 0, 0, 2.00333, 0, 4.24667, 0, 0],
     [1, 0, 0, 0, 0, 0, 0, 0],
     [0, 0, 0, 0, 1, 0, 0, 0]],
    [[1, 2, 0, 1], [2, 4, 0, 2], [0, 0, 0, 1], [1, 2, 1, 1]],
]

# (kind, n, seed, uplo, dtype)
GENERATED = [
    ("gram", 1, 1, "L", "d"), ("gram", 2, 2, "L", "d"), ("gram", 17, 3, "U", "d"), ("gram", 64, 4, "L", "d"),
    ("gram", 65, 5, "L", "s"), ("gram", 130, 6, "U", "d"), ("gram", 200, 7, "L", "d"),
    ("indef", 3, 8, "L", "d"), ("indef", 64, 9, "U", "d"), ("indef", 65, 10, "L", "d"), ("indef", 129, 11, "L", "s"),
    ("indef", 200, 12, "U", "d"),
    ("wide", 40, 13, "L", "d"), ("wide", 100, 14, "U", "d"),
    ("lagrange", 30, 15, "L", "d"), ("lagrange", 150, 16, "U", "d"),
    ("lowrank", 20, 17, "L", "d"), ("lowrank", 90, 18, "L", "d"),
    ("diag", 1, 19, "L", "d"), ("diag", 9, 20, "L", "d"), ("diag", 70, 21, "U", "d"), ("diag", 33, 22, "L", "s"),
    ("zerocol", 10, 23, "L", "d"), ("zerocol", 129, 24, "U", "d"),
    ("zerodiag", 2, 25, "L", "d"), ("zerodiag", 12, 26, "U", "d"),
]


def pack(f, uplo):
    n = f.shape[0]
    idx = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    return f[idx]


def eigen_ldlt(R, a, uplo, b):
    n = a.shape[0]
    f = np.array(a, order="F", copy=True)
    t = np.zeros(max(n, 1), dtype=np.int32)
    sg = ctypes.c_int32(0)
    fn = R.ref_dldlt if a.dtype == np.float64 else R.ref_sldlt
    rc = int(fn(uplo.encode(), n, f.ctypes.data, n, t.ctypes.data, ctypes.byref(sg)))
    x = np.array(b, copy=True)
    fs = R.ref_dldlt_solve if a.dtype == np.float64 else R.ref_sldlt_solve
    fs(uplo.encode(), n, 1, a.ctypes.data, n, x.ctypes.data, n)
    return f, t[:n], int(sg.value), rc, x


def main() -> None:
    O.build(ref=True)
    R = O.eigen_ref()
    if R is None:
        raise SystemExit("Eigen's reference LDLT could not be built (reference headers missing)")
    meta, facs, trs, xs, known = [], [], [], [], []
    offs, toffs = [0], [0]
    cases = [("known", len(m), i, "L", "d", np.array(m, dtype=np.float64, order="F")) for i, m in enumerate(KNOWN)]
    cases += [(k, n, s, up, dt, O.gen_sym(k, n, s)) for k, n, s, up, dt in GENERATED]
    for kind, n, seed, uplo, dt, a in cases:
        a = np.asfortranarray(a.astype(np.float64 if dt == "d" else np.float32))
        b = O.normal(seed + 7, n).astype(a.dtype)
        f, t, sign, info, x = eigen_ldlt(R, a, uplo, b)
        p = pack(f, uplo).astype(np.float64)
        facs.append(p)
        offs.append(offs[-1] + p.size)
        trs.append(t.astype(np.int32))
        xs.append(x.astype(np.float64))
        toffs.append(toffs[-1] + n)
        if kind == "known":
            known.append(a.astype(np.float64).ravel(order="F"))
        code = -1 if kind == "known" else O.LDLT_KINDS.index(kind)
        meta.append([code, n, seed, 0 if uplo == "L" else 1, 0 if dt == "d" else 1, sign, info])
    np.savez(OUT, meta=np.array(meta, dtype=np.int64), factors=np.concatenate(facs),
             offsets=np.array(offs, dtype=np.int64), transp=np.concatenate(trs), xs=np.concatenate(xs),
             toffsets=np.array(toffs, dtype=np.int64), known=np.concatenate(known))
    print(f"wrote {OUT} ({len(cases)} cases)")


if __name__ == "__main__":
    main()
