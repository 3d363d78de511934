"""Generate tests/golden/rcond_golden.npz from Eigen's own LLT::rcond().

Run where the reference sources are present (it builds oracle/_ref/libeigen_ref.so from the
Eigen headers in place, see oracle/Makefile):

    python tests/golden/make_rcond_golden.py

Per case the fixture stores the kind, order, seed, scalar type and triangle that regenerate the
input with the oracle's Philox generator, and Eigen's LLT<Matrix,UpLo>(A).rcond() -- the 1-norm
kept by LLT::compute (Eigen/src/Cholesky/LLT.h:443-453) combined with
rcond_invmatrix_L1_norm_estimate (Eigen/src/Core/ConditionEstimator.h:56-171).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "rcond_golden.npz"

KINDS = {"gram": 0, "householder": 1, "eigen": 2}


def make_input(kind: str, n: int, seed: int) -> np.ndarray:
    """gram: G G^T/n + I; householder: spectrum log-spaced over [1e-4, 1] (kappa 1e4, seed = v seed);
    eigen: a0 a0^T + 3 more rank-n terms with uniform[-1,1] entries (test/cholesky.cpp:69-78)."""
    if kind == "gram":
        return O.gen_gram(n, seed=seed)
    if kind == "householder":
        return O.gen_householder(n, 1e4, v_seed0=seed)
    if kind == "eigen":
        s = np.zeros((n, n))
        for r in range(4):
            g = (2.0 * O.uniform(seed, n * n, offset=r * n * n) - 1.0).reshape(n, n, order="F")
            s += g @ g.T
        return np.asfortranarray(s)
    raise ValueError(kind)


CASES = []
for n in [1, 2, 3, 17, 64, 65, 130, 300]:
    CASES.append(("gram", n, 2, "d", "L"))
for n in [40, 257]:
    CASES.append(("gram", n, 4, "d", "U"))
for n in [50, 200]:
    CASES.append(("householder", n, 3, "d", "L"))
    CASES.append(("householder", n, 3, "d", "U"))
for n in [20, 90]:
    CASES.append(("eigen", n, 9, "d", "L"))
for n in [33, 150]:
    CASES.append(("gram", n, 6, "s", "L"))
    CASES.append(("eigen", n, 6, "s", "U"))


def main() -> None:
    O.build(ref=True)
    R = O.eigen_ref()
    if R is None:
        raise SystemExit("Eigen's reference LLT could not be built (reference headers missing)")
    meta, vals = [], []
    for kind, n, seed, dt, uplo in CASES:
        a = make_input(kind, n, seed).astype(np.float64 if dt == "d" else np.float32, order="F")
        fn = R.ref_drcond if dt == "d" else R.ref_srcond
        r = float(fn(uplo.encode(), n, a.ctypes.data, n))
        assert r > 0, (kind, n, r)
        meta.append([KINDS[kind], n, seed, 0 if dt == "d" else 1, 0 if uplo == "L" else 1])
        vals.append(r)
    np.savez(OUT, meta=np.array(meta, dtype=np.int64), rcond=np.array(vals))
    print(f"wrote {OUT} ({len(CASES)} cases)")


if __name__ == "__main__":
    main()
