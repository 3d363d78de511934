"""Generate tests/golden/blas_golden.npz from Eigen's own BLAS (dsyrk_/ssyrk_, dtrsm_/strsm_).

Run where the reference sources are present: Eigen's BLAS is compiled from its own translation units
(blas/double.cpp, blas/single.cpp, blas/xerbla.cpp) where they lie, into oracle/_ref/libeigen_blas.so
(oracle/Makefile, target `ref`):

    python tests/golden/make_blas_golden.py

SYRK cases (blas/level3_impl.h:355-417): uplo x trans x (n, k) x (alpha, beta) x scalar type; A and C
from the oracle's Philox generator (seeded), C's input triangle poisoned with NaN where beta = 0 (the
reference must not read it).  TRSM cases (blas/level3_impl.h:78-160): every side x uplo x trans x diag,
several (m, n), alpha; A triangular with off-diagonal entries N(0,1)/order and a diagonal in [1, 2]
(signs alternating), so that every solve is well conditioned.  The fixture stores the inputs' seeds
and Eigen's outputs (for SYRK the updated triangle, in numpy's tril/triu index order).
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "blas_golden.npz"

SYRK = []  # (uplo, trans, n, k, alpha, beta, dtype, seed)
seed = 100
for uplo in "LU":
    for trans in "NT":
        ab = [(1.0, 0.0), (-1.0, 1.0), (0.5, -2.0)]
        for i, (n, k) in enumerate([(1, 1), (17, 5), (64, 64), (100, 37), (70, 130)]):
            for alpha, beta in (ab if n < 64 else [ab[i % 3]]):
                SYRK.append((uplo, trans, n, k, alpha, beta, "d", seed))
                seed += 1
for uplo, trans, n, k, alpha, beta in [("L", "N", 65, 33, 1.0, 0.0), ("U", "T", 90, 70, -1.5, 0.25)]:
    SYRK.append((uplo, trans, n, k, alpha, beta, "s", seed))
    seed += 1

TRSM = []  # (side, uplo, trans, diag, m, n, alpha, dtype, seed)
for side in "LR":
    for uplo in "LU":
        for trans in "NT":
            for diag in "NU":
                for m, n, alpha in [(1, 1, 1.0), (33, 7, 1.0), (64, 20, -2.0), (20, 100, 0.5)]:
                    TRSM.append((side, uplo, trans, diag, m, n, alpha, "d", seed))
                    seed += 1
for side, uplo, trans, diag, m, n, alpha in [("L", "L", "N", "N", 70, 9, 1.0), ("R", "U", "T", "U", 40, 66, 2.0)]:
    TRSM.append((side, uplo, trans, diag, m, n, alpha, "s", seed))
    seed += 1


def syrk_inputs(uplo, trans, n, k, beta, dt, seed):
    ar, ac = (n, k) if trans == "N" else (k, n)
    a = np.asfortranarray(O.normal(seed, ar * ac).reshape(ar, ac, order="F").astype(dt))
    c = np.asfortranarray(O.normal(seed + 1, n * n).reshape(n, n, order="F").astype(dt))
    if beta == 0.0:
        tri = np.tril(np.ones((n, n), bool)) if uplo == "L" else np.triu(np.ones((n, n), bool))
        c[tri] = np.nan
    return a, c


def trsm_inputs(side, uplo, m, n, dt, seed):
    na = m if side == "L" else n
    a = O.normal(seed, na * na).reshape(na, na, order="F") / max(na, 1)
    d = 1.0 + O.uniform(seed + 1, na)
    d[1::2] *= -1.0
    a[np.diag_indices(na)] = d
    a = np.tril(a) if uplo == "L" else np.triu(a)
    # the other triangle holds garbage the routine must not read
    other = np.triu(np.ones((na, na), bool), 1) if uplo == "L" else np.tril(np.ones((na, na), bool), -1)
    a[other] = 1e30
    b = O.normal(seed + 2, m * n).reshape(m, n, order="F")
    return np.asfortranarray(a.astype(dt)), np.asfortranarray(b.astype(dt))


def main() -> None:
    O.build(ref=True)
    R = O.eigen_blas_ref()
    if R is None:
        raise SystemExit("Eigen's BLAS could not be built (reference sources missing)")
    I = ctypes.c_int
    out = {}
    syrk_meta, syrk_vals, syrk_off = [], [], [0]
    for uplo, trans, n, k, alpha, beta, dt, sd in SYRK:
        np_dt = np.float64 if dt == "d" else np.float32
        ct = ctypes.c_double if dt == "d" else ctypes.c_float
        a, c = syrk_inputs(uplo, trans, n, k, beta, np_dt, sd)
        fn = R.dsyrk_ if dt == "d" else R.ssyrk_
        fn(ctypes.c_char_p(uplo.encode()), ctypes.c_char_p(trans.encode()), ctypes.byref(I(n)), ctypes.byref(I(k)),
           ctypes.byref(ct(alpha)), a.ctypes.data_as(ctypes.c_void_p), ctypes.byref(I(max(1, a.shape[0]))),
           ctypes.byref(ct(beta)), c.ctypes.data_as(ctypes.c_void_p), ctypes.byref(I(max(1, n))))
        tri = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
        v = c[tri].astype(np.float64)  # the updated triangle, row-index order of numpy's indices
        syrk_vals.append(v)
        syrk_off.append(syrk_off[-1] + v.size)
        syrk_meta.append([0 if uplo == "L" else 1, 0 if trans == "N" else 1, n, k, 0 if dt == "d" else 1, sd])
    trsm_meta, trsm_vals, trsm_off = [], [], [0]
    for side, uplo, trans, diag, m, n, alpha, dt, sd in TRSM:
        np_dt = np.float64 if dt == "d" else np.float32
        ct = ctypes.c_double if dt == "d" else ctypes.c_float
        a, b = trsm_inputs(side, uplo, m, n, np_dt, sd)
        fn = R.dtrsm_ if dt == "d" else R.strsm_
        fn(ctypes.c_char_p(side.encode()), ctypes.c_char_p(uplo.encode()), ctypes.c_char_p(trans.encode()),
           ctypes.c_char_p(diag.encode()), ctypes.byref(I(m)), ctypes.byref(I(n)), ctypes.byref(ct(alpha)),
           a.ctypes.data_as(ctypes.c_void_p), ctypes.byref(I(max(1, a.shape[0]))), b.ctypes.data_as(ctypes.c_void_p),
           ctypes.byref(I(max(1, m))))
        v = b.astype(np.float64).ravel(order="F")
        trsm_vals.append(v)
        trsm_off.append(trsm_off[-1] + v.size)
        trsm_meta.append([0 if side == "L" else 1, 0 if uplo == "L" else 1, 0 if trans == "N" else 1,
                          0 if diag == "N" else 1, m, n, 0 if dt == "d" else 1, sd])
    np.savez(OUT, syrk_meta=np.array(syrk_meta, np.int64), syrk_ab=np.array([(c[4], c[5]) for c in SYRK]),
             syrk_vals=np.concatenate(syrk_vals), syrk_off=np.array(syrk_off, np.int64),
             trsm_meta=np.array(trsm_meta, np.int64), trsm_alpha=np.array([c[6] for c in TRSM]),
             trsm_vals=np.concatenate(trsm_vals), trsm_off=np.array(trsm_off, np.int64))
    print(f"wrote {OUT} ({len(SYRK)} syrk, {len(TRSM)} trsm cases)")


if __name__ == "__main__":
    main()
