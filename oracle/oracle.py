"""ctypes wrapper of the oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

The oracle is the checker for the GPU path: a plain-C restatement of Eigen's LLT
(Eigen/src/Cholesky/LLT.h:312-399, lapack/cholesky.cpp:14-72) plus the seeded workload
generators.  Only the test suite, the smoke check and the CPU legs of the benchmark use it.

`eigen_ref()` loads Eigen's own LLT compiled from the reference headers (oracle/Makefile,
target `ref`) when that library exists; it exists only where the reference sources were present
at build time.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"
REF_PATH = ORACLE_DIR / "_ref" / "libeigen_ref.so"
BLAS_REF_PATH = ORACLE_DIR / "_ref" / "libeigen_blas.so"  # Eigen's own Fortran BLAS (blas/*.cpp)

_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_dbl = ctypes.c_double
_vp = ctypes.c_void_p
_ch = ctypes.c_char

_SIGS = {
    "oracle_dsym_l1_norm": (_dbl, [_ch, _i64, _vp, _i64]),
    "oracle_ssym_l1_norm": (ctypes.c_float, [_ch, _i64, _vp, _i64]),
    "oracle_drcond": (_dbl, [_ch, _i64, _vp, _i64, _dbl]),
    "oracle_drank_update": (_i64, [_ch, _i64, _vp, _i64, _vp, _dbl]),
    "oracle_srank_update": (_i64, [_ch, _i64, _vp, _i64, _vp, ctypes.c_float]),
    "oracle_srcond": (_dbl, [_ch, _i64, _vp, _i64, _dbl]),
    "oracle_dsyrk": (None, [_ch, _ch, _i64, _i64, _dbl, _vp, _i64, _dbl, _vp, _i64]),
    "oracle_ssyrk": (None, [_ch, _ch, _i64, _i64, ctypes.c_float, _vp, _i64, ctypes.c_float, _vp, _i64]),
    "oracle_dtrsm": (None, [_ch, _ch, _ch, _ch, _i64, _i64, _dbl, _vp, _i64, _vp, _i64]),
    "oracle_strsm": (None, [_ch, _ch, _ch, _ch, _i64, _i64, ctypes.c_float, _vp, _i64, _vp, _i64]),
    "oracle_dldlt": (ctypes.c_int, [_ch, _i64, _vp, _i64, _vp, _vp]),
    "oracle_sldlt": (ctypes.c_int, [_ch, _i64, _vp, _i64, _vp, _vp]),
    "oracle_dldlt_solve": (None, [_ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64]),
    "oracle_sldlt_solve": (None, [_ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64]),
    "oracle_philox4x32_10": (None, [_vp, _vp, _vp]),
    "oracle_normal": (_dbl, [_u64, _u64]),
    "oracle_uniform": (_dbl, [_u64, _u64]),
    "oracle_fill_normal": (None, [_u64, _u64, _i64, _vp]),
    "oracle_fill_uniform": (None, [_u64, _u64, _i64, _vp]),
    "oracle_gen_gram": (None, [_i64, _u64, _u64, _dbl, _vp, _i64]),
    "oracle_spectrum": (None, [_i64, _dbl, _u64, _vp]),
    "oracle_gen_householder": (None, [_i64, ctypes.c_int, _u64, _vp, _vp, _i64]),
    "oracle_batch_sizes": (None, [_i64, _u64, _i64, _i64, _vp]),
    "oracle_gen_rbf": (None, [_i64, _u64, _u64, _dbl, _dbl, _dbl, _vp, _i64]),
    "oracle_dllt_blocked": (_i64, [_i64, _vp, _i64, _i64]),
    "oracle_sllt_blocked": (_i64, [_i64, _vp, _i64, _i64]),
    "oracle_dllt_unblocked": (_i64, [_i64, _vp, _i64, _i64]),
    "oracle_dpotrf": (ctypes.c_int, [_ch, _i64, _vp, _i64, _vp]),
    "oracle_spotrf": (ctypes.c_int, [_ch, _i64, _vp, _i64, _vp]),
    "oracle_dpotrs": (ctypes.c_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64]),
    "oracle_spotrs": (ctypes.c_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64]),
    "oracle_dbackward_error": (_dbl, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64]),
    "oracle_sbackward_error": (_dbl, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64]),
    "oracle_dbatched_posv": (None, [_i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "oracle_sbatched_posv": (None, [_i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "oracle_num_threads": (ctypes.c_int, []),
    "oracle_set_num_threads": (None, [ctypes.c_int]),
}

_lib = None
_ref = None


SRC_RECORD = ORACLE_DIR / "_ref" / "eigen_src.txt"  # where the last `ref` build found the Eigen sources


def eigen_src() -> Path | None:
    """The Eigen source tree: $EIGEN_REF, else the one the last `ref` build used; None if neither."""
    env = os.environ.get("EIGEN_REF")
    if env:
        return Path(env)
    if SRC_RECORD.exists():
        return Path(SRC_RECORD.read_text().strip())
    return None


def build(ref: bool = True, eigen: str | None = None) -> None:
    """Compile liboracle.so; with ref, also Eigen's own LLT and BLAS from the Eigen source tree
    given by `eigen` or $EIGEN_REF, when one is given and holds the sources (nothing else is
    assumed about where they lie).  Same commands as oracle/Makefile, issued directly so that
    `make` is not required.  No FMA contraction: every product and sum is rounded, as in Eigen's
    SSE2 build, on x86-64 and aarch64 alike."""
    src = ORACLE_DIR / "llt_oracle.c"
    deps = [src, ORACLE_DIR / "llt_oracle_body.h"]
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        subprocess.run(["gcc", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall", "-o",
                        str(LIB_PATH), str(src), "-lm"], check=True)
    eigen = eigen or os.environ.get("EIGEN_REF")
    if ref and eigen and Path(eigen, "Eigen").is_dir():
        REF_PATH.parent.mkdir(exist_ok=True)
        SRC_RECORD.write_text(str(Path(eigen).resolve()) + "\n")
        cpp = ORACLE_DIR / "eigen_ref.cpp"
        if not REF_PATH.exists() or REF_PATH.stat().st_mtime < cpp.stat().st_mtime:
            subprocess.run(["g++", "-O3", "-DNDEBUG", "-fopenmp", "-fPIC", "-shared", f"-I{eigen}", "-o",
                            str(REF_PATH), str(cpp)], check=True)
        if not BLAS_REF_PATH.exists():
            subprocess.run(["g++", "-O2", "-fPIC", "-shared", f"-I{eigen}", "-o", str(BLAS_REF_PATH)] +
                           [str(Path(eigen, "blas", f)) for f in ("double.cpp", "single.cpp", "xerbla.cpp")],
                           check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build(ref=False)
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def eigen_ref():
    """Eigen's own LLT (None when it was not built here)."""
    global _ref
    if _ref is None and REF_PATH.exists():
        R = ctypes.CDLL(str(REF_PATH))
        for nm in ("ref_dllt", "ref_sllt"):
            getattr(R, nm).restype = _i64
            getattr(R, nm).argtypes = [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp]
        for nm in ("ref_dblocked", "ref_sblocked"):
            getattr(R, nm).restype = _i64
            getattr(R, nm).argtypes = [_ch, _i64, _vp, _i64]
        for nm in ("ref_drcond", "ref_srcond"):
            getattr(R, nm).restype = _dbl
            getattr(R, nm).argtypes = [_ch, _i64, _vp, _i64]
        R.ref_drank_update.restype = _i64
        R.ref_drank_update.argtypes = [_ch, _i64, _vp, _i64, _vp, _dbl]
        R.ref_srank_update.restype = _i64
        R.ref_srank_update.argtypes = [_ch, _i64, _vp, _i64, _vp, ctypes.c_float]
        for nm in ("ref_dldlt", "ref_sldlt"):
            getattr(R, nm).restype = _i64
            getattr(R, nm).argtypes = [_ch, _i64, _vp, _i64, _vp, _vp]
        for nm in ("ref_dldlt_solve", "ref_sldlt_solve"):
            getattr(R, nm).restype = None
            getattr(R, nm).argtypes = [_ch, _i64, _i64, _vp, _i64, _vp, _i64]
        _ref = R
    return _ref


_blas_ref = None


def eigen_blas_ref():
    """Eigen's own BLAS library (dsyrk_, dtrsm_, ...), None when it was not built here."""
    global _blas_ref
    if _blas_ref is None and BLAS_REF_PATH.exists():
        _blas_ref = ctypes.CDLL(str(BLAS_REF_PATH))
    return _blas_ref


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


# ---- generators --------------------------------------------------------------------------------

def philox(ctr, key) -> list[int]:
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().oracle_philox4x32_10(c, k, o)
    return list(o)


def normal(seed: int, count: int, offset: int = 0) -> np.ndarray:
    out = np.empty(count, dtype=np.float64)
    lib().oracle_fill_normal(seed, offset, count, _p(out))
    return out


def uniform(seed: int, count: int, offset: int = 0) -> np.ndarray:
    out = np.empty(count, dtype=np.float64)
    lib().oracle_fill_uniform(seed, offset, count, _p(out))
    return out


def gen_gram(n: int, seed: int = 1, offset: int = 0, shift: float = 1.0) -> np.ndarray:
    """A = G G^T / n + shift I (Fortran order)."""
    a = np.empty((n, n), dtype=np.float64, order="F")
    if n:
        lib().oracle_gen_gram(n, seed, offset, shift, _p(a), n)
    return a


def spectrum(n: int, kappa: float, perm_seed: int = 11) -> np.ndarray:
    lam = np.empty(n, dtype=np.float64)
    lib().oracle_spectrum(n, kappa, perm_seed, _p(lam))
    return lam


def gen_householder(n: int, kappa: float, nrefl: int = 8, v_seed0: int = 3, perm_seed: int = 11) -> np.ndarray:
    """A = Q diag(lambda) Q^T, Q = H_1 ... H_nrefl, v_i from seed v_seed0 + i."""
    lam = spectrum(n, kappa, perm_seed)
    a = np.empty((n, n), dtype=np.float64, order="F")
    lib().oracle_gen_householder(n, nrefl, v_seed0, _p(lam), _p(a), n)
    return a


def batch_sizes(count: int, seed: int = 21, lo: int = 4, hi: int = 256) -> np.ndarray:
    out = np.empty(count, dtype=np.int64)
    lib().oracle_batch_sizes(count, seed, lo, hi, _p(out))
    return out


def gen_rbf(m: int, seed: int = 31, offset: int = 0, ell: float = 0.2, sigma2: float = 1.0,
            noise: float = 1e-2) -> np.ndarray:
    a = np.empty((m, m), dtype=np.float64, order="F")
    lib().oracle_gen_rbf(m, seed, offset, ell, sigma2, noise, _p(a), m)
    return a


LDLT_KINDS = ("gram", "indef", "wide", "lagrange", "lowrank", "diag", "zerocol", "zerodiag")


def gen_sym(kind: str, n: int, seed: int) -> np.ndarray:
    """Symmetric inputs for the LDL^T path (Fortran order, double):
    gram      G G^T/n + I (positive definite);
    indef     (G + G^T)/(2n) + diag(+-(2 + u)): diagonally dominant, indefinite;
    wide      a diag(d) a^T, a uniform[-1,1], d_k uniform[-1,1] * 10^r, r uniform[-4,4] (the
              wide-spectrum matrices of test/cholesky.cpp:248-255, exponent range narrowed);
    lagrange  gram with its trailing n/3 x n/3 block zeroed (test/cholesky.cpp:214-228);
    lowrank   a a^T, a n x max(1, n/2) uniform[-1,1] (test/cholesky.cpp:230-245);
    diag      integer diagonal in [-3, 3], zeros included (pivots and signs exact);
    zerocol   gram with row and column n/2 zeroed (an exact zero pivot with a zero column);
    zerodiag  (G + G^T) with a zero diagonal (NumericalIssue unless n <= 1)."""
    if n == 0:
        return np.zeros((0, 0), order="F")
    g = normal(seed, n * n).reshape(n, n, order="F")
    u = uniform(seed + 1, n)
    if kind == "gram":
        return gen_gram(n, seed=seed)
    if kind == "indef":
        d = np.where(u < 0.5, -1.0, 1.0) * (2.0 + uniform(seed + 2, n))
        return np.asfortranarray((g + g.T) / (2.0 * n) + np.diag(d))
    if kind == "wide":
        a = 2.0 * uniform(seed + 3, n * n).reshape(n, n, order="F") - 1.0
        d = (2.0 * u - 1.0) * 10.0 ** (8.0 * uniform(seed + 4, n) - 4.0)
        return np.asfortranarray((a * d) @ a.T)
    if kind == "lagrange":
        a = gen_gram(n, seed=seed)
        c = n // 3
        if c:
            a[n - c:, n - c:] = 0.0
        return a
    if kind == "lowrank":
        r = max(1, n // 2)
        a = 2.0 * uniform(seed + 3, n * r).reshape(n, r, order="F") - 1.0
        return np.asfortranarray(a @ a.T)
    if kind == "diag":
        return np.asfortranarray(np.diag(np.floor(7.0 * u) - 3.0))
    if kind == "zerocol":
        a = gen_gram(n, seed=seed)
        a[n // 2, :] = 0.0
        a[:, n // 2] = 0.0
        return a
    if kind == "zerodiag":
        a = np.asfortranarray(g + g.T)
        np.fill_diagonal(a, 0.0)
        return a
    raise ValueError(kind)


# ---- LLT restatement ---------------------------------------------------------------------------

def blocked(a: np.ndarray, uplo: str = "L") -> int:
    """llt_inplace<T,UpLo>::blocked on a (Fortran order, in place): -1 or the failing column."""
    n = a.shape[0]
    lda = max(1, n)
    rs, cs = (lda, 1) if uplo == "U" else (1, lda)
    fn = lib().oracle_dllt_blocked if a.dtype == np.float64 else lib().oracle_sllt_blocked
    return int(fn(n, _p(a), rs, cs))


def potrf(a: np.ndarray, uplo: str = "L") -> int:
    info = np.zeros(1, dtype=np.int64)
    fn = lib().oracle_dpotrf if a.dtype == np.float64 else lib().oracle_spotrf
    rc = fn(uplo.encode(), a.shape[0], _p(a), max(1, a.shape[0]), _p(info))
    assert rc == 0, rc
    return int(info[0])


def potrs(a: np.ndarray, b: np.ndarray, uplo: str = "L") -> None:
    n = a.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    fn = lib().oracle_dpotrs if a.dtype == np.float64 else lib().oracle_spotrs
    rc = fn(uplo.encode(), n, k, _p(a), max(1, n), _p(b), max(1, n))
    assert rc == 0, rc


def sym_l1_norm(a: np.ndarray, uplo: str = "L") -> float:
    """1-norm of the symmetric matrix stored in the `uplo` triangle (LLT.h:443-453)."""
    n = a.shape[0]
    fn = lib().oracle_dsym_l1_norm if a.dtype == np.float64 else lib().oracle_ssym_l1_norm
    return float(fn(uplo.encode(), n, _p(a), max(1, n)))


def rcond(l: np.ndarray, anorm: float, uplo: str = "L") -> float:
    """Reciprocal condition estimate from a factor (ConditionEstimator.h:56-171 over potrs)."""
    n = l.shape[0]
    fn = lib().oracle_drcond if l.dtype == np.float64 else lib().oracle_srcond
    return float(fn(uplo.encode(), n, _p(l) if n else None, max(1, n), float(anorm)))


def rank_update(l: np.ndarray, v: np.ndarray, sigma: float, uplo: str = "L") -> int:
    """In place: the factor of A + sigma v v^T from the factor l of A (LLT.h:238-307); returns the
    column where a downdate fails, or -1."""
    n = l.shape[0]
    fn = lib().oracle_drank_update if l.dtype == np.float64 else lib().oracle_srank_update
    vv = np.ascontiguousarray(v, dtype=l.dtype)
    return int(fn(uplo.encode(), n, _p(l) if n else None, max(1, n), _p(vv) if n else None, sigma))


def syrk(c: np.ndarray, a: np.ndarray, uplo: str = "L", trans: str = "N", alpha: float = 1.0,
         beta: float = 0.0) -> None:
    """In place on the Fortran-order c: Eigen's BLAS syrk (blas/level3_impl.h:355-417)."""
    n = c.shape[0]
    k = a.shape[1] if trans.upper() == "N" else a.shape[0]
    fn = lib().oracle_dsyrk if c.dtype == np.float64 else lib().oracle_ssyrk
    fn(uplo.encode(), trans.encode(), n, k, alpha, _p(a) if a.size else None, max(1, a.shape[0]), beta,
       _p(c) if n else None, max(1, n))


def trsm(b: np.ndarray, a: np.ndarray, side: str = "L", uplo: str = "L", trans: str = "N", diag: str = "N",
         alpha: float = 1.0) -> None:
    """In place on the Fortran-order b: Eigen's BLAS trsm (blas/level3_impl.h:78-160)."""
    m, n = b.shape
    fn = lib().oracle_dtrsm if b.dtype == np.float64 else lib().oracle_strsm
    fn(side.encode(), uplo.encode(), trans.encode(), diag.encode(), m, n, alpha, _p(a) if a.size else None,
       max(1, a.shape[0]), _p(b) if b.size else None, max(1, m))


SIGN_NAMES = ("PositiveSemiDef", "NegativeSemiDef", "ZeroSign", "Indefinite")


def ldlt(a: np.ndarray, uplo: str = "L") -> tuple[bool, np.ndarray, int]:
    """In place: Eigen's pivoted LDL^T of the symmetric matrix in the `uplo` triangle of a
    (ldlt_inplace<Lower>::unblocked, LDLT.h:297-403).  Returns (success, transpositions, sign)."""
    n = a.shape[0]
    t = np.zeros(max(n, 1), dtype=np.int32)
    sg = ctypes.c_int(0)
    fn = lib().oracle_dldlt if a.dtype == np.float64 else lib().oracle_sldlt
    ok = fn(uplo.encode(), n, _p(a) if n else None, max(1, n), _p(t), ctypes.byref(sg))
    return bool(ok), t[:n], int(sg.value)


def ldlt_solve(f: np.ndarray, transp: np.ndarray, b: np.ndarray, uplo: str = "L") -> None:
    """In place: b <- A^{-1} b from an LDL^T factor (LDLT.h:573-613)."""
    n = f.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    t = np.ascontiguousarray(transp, dtype=np.int32)
    fn = lib().oracle_dldlt_solve if f.dtype == np.float64 else lib().oracle_sldlt_solve
    fn(uplo.encode(), n, k, _p(f) if n else None, max(1, n), _p(t) if n else None, _p(b) if n else None, max(1, n))


def backward_error(a: np.ndarray, x: np.ndarray, b: np.ndarray, uplo: str = "L") -> float:
    """||A X - B||_F / (||A||_F ||X||_F), A symmetric given by its `uplo` triangle."""
    n = a.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    fn = lib().oracle_dbackward_error if a.dtype == np.float64 else lib().oracle_sbackward_error
    x = np.asfortranarray(x, dtype=a.dtype)
    b = np.asfortranarray(b, dtype=a.dtype)
    return float(fn(uplo.encode(), n, k, _p(a), max(1, n), _p(x), max(1, n), _p(b), max(1, n)))


def solve(a: np.ndarray, b: np.ndarray, uplo: str = "L") -> tuple[np.ndarray, np.ndarray, int]:
    """Factor a copy of a and solve: returns (factor, X, info)."""
    f = np.array(a, order="F", copy=True)
    info = potrf(f, uplo)
    x = np.array(b, order="F", copy=True)
    if info == 0:
        potrs(f, x, uplo)
    return f, x, info


def batched_posv(ns: np.ndarray, a_packed: np.ndarray, b_packed: np.ndarray):
    """Factor + solve every system of an uneven batch in place; returns info per system."""
    ns = np.ascontiguousarray(ns, dtype=np.int64)
    aoff = np.zeros(len(ns), dtype=np.int64)
    boff = np.zeros(len(ns), dtype=np.int64)
    if len(ns):
        aoff[1:] = np.cumsum(ns * ns)[:-1]
        boff[1:] = np.cumsum(ns)[:-1]
    info = np.zeros(len(ns), dtype=np.int64)
    fn = lib().oracle_dbatched_posv if a_packed.dtype == np.float64 else lib().oracle_sbatched_posv
    fn(len(ns), _p(ns), _p(aoff), _p(boff), _p(a_packed), _p(b_packed), _p(info))
    return info


def set_threads(t: int) -> None:
    lib().oracle_set_num_threads(int(t))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


# ---- adjoint references (numpy, FP64) ---------------------------------------------------------

def chol_adjoint_ref(L: np.ndarray, Lbar: np.ndarray) -> np.ndarray:
    """Symmetric df/dA from df/dL for A = L L^T: 1/2 L^{-T} (P + P^T) L^{-1}, P = Phi(L^T Lbar),
    Phi = lower triangle with halved diagonal (Murray 2016, arXiv:1602.07527, symbolic form)."""
    from scipy.linalg import solve_triangular
    L = np.tril(L)
    P = np.tril(L.T @ np.tril(Lbar))
    P[np.diag_indices_from(P)] *= 0.5
    S = P + P.T
    Y = solve_triangular(L, S, trans="T", lower=True)          # L^{-T} S
    D = solve_triangular(L, Y.T, trans="T", lower=True).T      # (L^{-T} Y^T)^T = Y L^{-1}
    return 0.25 * (D + D.T)  # 1/2 L^{-T} S L^{-1}, symmetrised against roundoff


def gp_objective_ref(A: np.ndarray, y: np.ndarray):
    """f = logdet A + y^T A^{-1} y and its gradients dA = A^{-1} - a a^T (a = A^{-1} y), dy = 2 a."""
    L = np.linalg.cholesky(A)
    from scipy.linalg import cho_solve
    a = cho_solve((L, True), y)
    f = 2.0 * np.sum(np.log(np.diag(L))) + float(y @ a)
    Ainv = cho_solve((L, True), np.eye(A.shape[0]))
    return f, Ainv - np.outer(a, a), 2.0 * a
