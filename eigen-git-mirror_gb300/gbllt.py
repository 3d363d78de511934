"""ctypes binding of libgbllt.so, the C ABI declared in include/gbllt.h.

This is plumbing for Python callers (the test suite and the benchmark): every call goes
straight to the sm_103a kernels behind the C ABI.  There is no fallback; if the library is not
built, `lib()` raises.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libgbllt.so"
HEADER = PKG_DIR.parent / "include" / "gbllt.h"

SUCCESS = 0
ERR_CUDA = -1001
ERR_ALLOC = -1002
ERR_TIMEOUT = -1003
ERR_NO_DEVICE = -1004
ERR_INTERNAL = -1005
ERR_NOT_CONVERGED = -1006
ERR_SCRATCH_LIMIT = -1007
ROW_MAJOR = 101
COL_MAJOR = 102

_i64 = ctypes.c_int64
_int = ctypes.c_int
_ch = ctypes.c_char
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)

# argtypes of every entry point; the test suite checks this table against include/gbllt.h
SIGNATURES: dict[str, tuple] = {
    "gbllt_version": (_int, []),
    "gbllt_last_error": (ctypes.c_char_p, []),
    "gbllt_release_cached_memory": (_int, []),
    "gbllt_dpotrf": (_int, [_int, _ch, _i64, _vp, _i64, _i64p]),
    "gbllt_spotrf": (_int, [_int, _ch, _i64, _vp, _i64, _i64p]),
    "gbllt_dpotrs": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _i64]),
    "gbllt_spotrs": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _i64]),
    "gbllt_dposv": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _i64, _i64p]),
    "gbllt_sposv": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _i64, _i64p]),
    "gbllt_dpotrf_dev": (_int, [_ch, _i64, _vp, _i64, _vp, _vp]),
    "gbllt_spotrf_dev": (_int, [_ch, _i64, _vp, _i64, _vp, _vp]),
    "gbllt_dpotrs_dev": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_spotrs_dev": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_dposv_mixed_dev": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _vp, _vp]),
    "gbllt_dposv_mixed": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _vp]),
    "gbllt_dposv_mixed_dev_noalloc": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _vp, _vp]),
    "gbllt_batch_plan_create": (_int, [_i64, _vp, _int, ctypes.POINTER(_vp)]),
    "gbllt_batch_plan_destroy": (_int, [_vp]),
    "gbllt_batch_plan_layout": (_int, [_vp, _vp, _vp, _i64p, _i64p]),
    "gbllt_batch_plan_tune": (_int, [_vp, ctypes.c_char_p, _vp]),
    "gbllt_batch_plan_set_variant": (_int, [_vp, _int]),
    "gbllt_batch_plan_variant": (_int, [_vp, ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(_int)]),
    "gbllt_dposv_batched_dev": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbllt_batch_dposv_mixed_dev": (_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbllt_sposv_batched_dev": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbllt_dposv_batched": (_int, [_vp, _vp, _vp, _vp]),
    "gbllt_sposv_batched": (_int, [_vp, _vp, _vp, _vp]),
    "gbllt_dpotrf_adjoint_dev": (_int, [_i64, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_dpotrf_adjoint_mixed_dev": (_int, [_i64, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_dpotrs_adjoint_dev": (_int, [_i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_drank_update": (_int, [_int, _ch, _i64, _vp, _i64, _vp, ctypes.c_double, _i64p]),
    "gbllt_srank_update": (_int, [_int, _ch, _i64, _vp, _i64, _vp, ctypes.c_float, _i64p]),
    "gbllt_drank_update_dev": (_int, [_ch, _i64, _vp, _i64, _vp, ctypes.c_double, _vp, _vp]),
    "gbllt_srank_update_dev": (_int, [_ch, _i64, _vp, _i64, _vp, ctypes.c_float, _vp, _vp]),
    "gbllt_dldlt": (_int, [_int, _ch, _i64, _vp, _i64, _vp, _vp, _i64p]),
    "gbllt_sldlt": (_int, [_int, _ch, _i64, _vp, _i64, _vp, _vp, _i64p]),
    "gbllt_dldlt_dev": (_int, [_ch, _i64, _vp, _i64, _vp, _vp, _i64p, _vp]),
    "gbllt_sldlt_dev": (_int, [_ch, _i64, _vp, _i64, _vp, _vp, _i64p, _vp]),
    "gbllt_dldlt_pivots": (_int, [_i64, _vp, _i64, _vp]),
    "gbllt_sldlt_pivots": (_int, [_i64, _vp, _i64, _vp]),
    "gbllt_dldlt_solve": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gbllt_sldlt_solve": (_int, [_int, _ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gbllt_dldlt_solve_dev": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp]),
    "gbllt_sldlt_solve_dev": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp]),
    "gbllt_dsyrk": (_int, [_int, _ch, _ch, _i64, _i64, ctypes.c_double, _vp, _i64, ctypes.c_double, _vp, _i64]),
    "gbllt_ssyrk": (_int, [_int, _ch, _ch, _i64, _i64, ctypes.c_float, _vp, _i64, ctypes.c_float, _vp, _i64]),
    "gbllt_dsyrk_dev": (_int, [_ch, _ch, _i64, _i64, ctypes.c_double, _vp, _i64, ctypes.c_double, _vp, _i64, _vp]),
    "gbllt_ssyrk_dev": (_int, [_ch, _ch, _i64, _i64, ctypes.c_float, _vp, _i64, ctypes.c_float, _vp, _i64, _vp]),
    "gbllt_dtrsm": (_int, [_int, _ch, _ch, _ch, _ch, _i64, _i64, ctypes.c_double, _vp, _i64, _vp, _i64]),
    "gbllt_strsm": (_int, [_int, _ch, _ch, _ch, _ch, _i64, _i64, ctypes.c_float, _vp, _i64, _vp, _i64]),
    "gbllt_dtrsm_dev": (_int, [_ch, _ch, _ch, _ch, _i64, _i64, ctypes.c_double, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_strsm_dev": (_int, [_ch, _ch, _ch, _ch, _i64, _i64, ctypes.c_float, _vp, _i64, _vp, _i64, _vp]),
    "gbllt_dsyresid_dev": (_int, [_ch, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _int, _vp]),
    "gbllt_dlansy_l1_dev": (_int, [_ch, _i64, _vp, _i64, _vp, _vp]),
    "gbllt_slansy_l1_dev": (_int, [_ch, _i64, _vp, _i64, _vp, _vp]),
    "gbllt_dpocon_dev": (_int, [_ch, _i64, _vp, _i64, ctypes.c_double, _dp, _vp]),
    "gbllt_spocon_dev": (_int, [_ch, _i64, _vp, _i64, ctypes.c_float, _fp, _vp]),
    "gbllt_dpocon": (_int, [_int, _ch, _i64, _vp, _i64, ctypes.c_double, _dp]),
    "gbllt_spocon": (_int, [_int, _ch, _i64, _vp, _i64, ctypes.c_float, _fp]),
    "gbllt_profile_enable": (_int, [_int]),
    "gbllt_profile_read": (_int, [_vp, _int, ctypes.POINTER(_int)]),
    "gbllt_profile_trace": (_int, [_vp, _int, ctypes.POINTER(_int)]),
    "gbllt_selftest_wait_timeout": (_int, [_i64, ctypes.POINTER(_int)]),
    "gbllt_selftest_f64_to_f32": (_int, [_vp, _vp, _vp, _i64, _vp]),
}

_lib = None


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 40), ("launches", ctypes.c_int64), ("ms", ctypes.c_double),
                ("flops", ctypes.c_double), ("bytes", ctypes.c_double)]


PREC = {"fp32": 0, "tf32": 1, "tf32x3": 2, "bf16": 3, "bf16x3": 4, "bf16x6": 5}


class BatchMixedReport(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("converged", ctypes.c_int64), ("fallback", ctypes.c_int64),
                ("max_backward_error", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {"steps": int(self.steps), "converged": int(self.converged), "fallback": int(self.fallback),
                "max_backward_error": float(self.max_backward_error)}


BATCH_NOT_CONVERGED = -1


class LaunchRecord(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 40), ("stream", ctypes.c_uint64), ("start_ms", ctypes.c_double),
                ("end_ms", ctypes.c_double), ("flops", ctypes.c_double), ("bytes", ctypes.c_double)]


class MixedOpts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("max_steps", ctypes.c_int), ("tol", ctypes.c_double),
                ("fallback_fp64", ctypes.c_int), ("panel", ctypes.c_int), ("reserve_sms", ctypes.c_int),
                ("residual", ctypes.c_int)]


class MixedReport(ctypes.Structure):
    _fields_ = [("info", ctypes.c_int64), ("steps", ctypes.c_int), ("converged", ctypes.c_int),
                ("used_fallback", ctypes.c_int), ("backward_error", ctypes.c_double),
                ("factor_ms", ctypes.c_double), ("refine_ms", ctypes.c_double),
                ("history", ctypes.c_double * 16)]

    def as_dict(self) -> dict:
        return {"info": int(self.info), "steps": int(self.steps), "converged": bool(self.converged),
                "used_fallback": bool(self.used_fallback), "backward_error": float(self.backward_error),
                "factor_ms": float(self.factor_ms), "refine_ms": float(self.refine_ms),
                "history": [float(self.history[i]) for i in range(min(int(self.steps), 16))]}


RESIDUAL = {"auto": 0, "fp64": 1, "tensor": 2}


def mixed_opts(precision: str = "tf32x3", max_steps: int = 10, tol: float = 1e-14, fallback: bool = True,
               panel: int = 0, reserve_sms: int = 0, residual: str = "auto") -> MixedOpts:
    """gbllt_mixed_opts; panel 0 and reserve_sms 0 take the library defaults (panel 256 below
    n = 16384, 384 from there on, for bf16x3 512 from 16384 and 640 from 32768; 32 reserved SMs for the
    first panels, more as the trailing matrix shrinks)."""
    return MixedOpts(PREC[precision], max_steps, tol, 1 if fallback else 0, panel, reserve_sms,
                     RESIDUAL[residual])


class GblltError(RuntimeError):
    def __init__(self, fn: str, rc: int):
        msg = ""
        if _lib is not None:
            try:
                msg = _lib.gbllt_last_error().decode()
            except Exception:  # pragma: no cover
                pass
        super().__init__(f"{fn} returned {rc} {msg}".strip())
        self.rc = rc


def lib() -> ctypes.CDLL:
    """Load libgbllt.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


BATCH_VARIANTS = 16  # GBLLT_BATCH_VARIANTS of include/gbllt.h

LAPACK_PATH = PKG_DIR / "lib" / "libgbllt_lapack.so"
_lapack = None
_I = ctypes.POINTER(ctypes.c_int)
_C = ctypes.c_char_p
_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
LAPACK_SIGNATURES = {
    "dpotrf_": (ctypes.c_int, [_C, _I, _D, _I, _I]),
    "spotrf_": (ctypes.c_int, [_C, _I, _F, _I, _I]),
    "dpotrs_": (ctypes.c_int, [_C, _I, _I, _D, _I, _D, _I, _I]),
    "spotrs_": (ctypes.c_int, [_C, _I, _I, _F, _I, _F, _I, _I]),
    "dsyrk_": (ctypes.c_int, [_C, _C, _I, _I, _D, _D, _I, _D, _D, _I]),
    "ssyrk_": (ctypes.c_int, [_C, _C, _I, _I, _F, _F, _I, _F, _F, _I]),
    "dtrsm_": (ctypes.c_int, [_C, _C, _C, _C, _I, _I, _D, _D, _I, _D, _I]),
    "strsm_": (ctypes.c_int, [_C, _C, _C, _C, _I, _I, _F, _F, _I, _F, _I]),
}


def lapack() -> ctypes.CDLL:
    """Load libgbllt_lapack.so, the Fortran-ABI dpotrf_/dpotrs_/spotrf_/spotrs_ routines."""
    global _lapack
    if _lapack is None:
        lib()  # the shim resolves its gbllt_* calls against libgbllt.so
        if not LAPACK_PATH.exists():
            raise RuntimeError(f"{LAPACK_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(str(LAPACK_PATH))
        for name, (res, args) in LAPACK_SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lapack = L
    return _lapack


def _cptr(a: np.ndarray, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _ci(v: int):
    return ctypes.byref(ctypes.c_int(v))


def blas_syrk(c: np.ndarray, a: np.ndarray, uplo: str = "L", trans: str = "N", alpha: float = 1.0, beta: float = 0.0,
              n: int | None = None, k: int | None = None, lda: int | None = None, ldc: int | None = None) -> int:
    """dsyrk_ / ssyrk_ of libgbllt_lapack.so on Fortran-order arrays; returns the routine's int."""
    dbl = c.dtype == np.float64
    ct = ctypes.c_double if dbl else ctypes.c_float
    fn = lapack().dsyrk_ if dbl else lapack().ssyrk_
    n = c.shape[0] if n is None else n
    k = (a.shape[1] if trans.upper() == "N" else a.shape[0]) if k is None else k
    lda = max(1, a.shape[0]) if lda is None else lda
    ldc = max(1, c.shape[0]) if ldc is None else ldc
    return fn(ctypes.c_char_p(uplo.encode()), ctypes.c_char_p(trans.encode()), _ci(n), _ci(k),
              ctypes.byref(ct(alpha)), _cptr(a, ct), _ci(lda), ctypes.byref(ct(beta)), _cptr(c, ct), _ci(ldc))


def blas_trsm(b: np.ndarray, a: np.ndarray, side: str = "L", uplo: str = "L", trans: str = "N", diag: str = "N",
              alpha: float = 1.0, m: int | None = None, n: int | None = None, lda: int | None = None,
              ldb: int | None = None) -> int:
    """dtrsm_ / strsm_ of libgbllt_lapack.so on Fortran-order arrays; returns the routine's int."""
    dbl = b.dtype == np.float64
    ct = ctypes.c_double if dbl else ctypes.c_float
    fn = lapack().dtrsm_ if dbl else lapack().strsm_
    m = b.shape[0] if m is None else m
    n = b.shape[1] if n is None else n
    lda = max(1, a.shape[0]) if lda is None else lda
    ldb = max(1, b.shape[0]) if ldb is None else ldb
    return fn(ctypes.c_char_p(side.encode()), ctypes.c_char_p(uplo.encode()), ctypes.c_char_p(trans.encode()),
              ctypes.c_char_p(diag.encode()), _ci(m), _ci(n), ctypes.byref(ct(alpha)), _cptr(a, ct), _ci(lda),
              _cptr(b, ct), _ci(ldb))


def lapack_potrf(a: np.ndarray, uplo: str = "L", lda: int | None = None, n: int | None = None) -> int:
    """?potrf_ through the Fortran ABI on a Fortran-order array; returns info."""
    L = lapack()
    dbl = a.dtype == np.float64
    fn = L.dpotrf_ if dbl else L.spotrf_
    n_ = ctypes.c_int(a.shape[0] if n is None else n)
    lda_ = ctypes.c_int(a.shape[0] if lda is None else lda)
    info = ctypes.c_int(0)
    fn(uplo.encode(), ctypes.byref(n_), _cptr(a, ctypes.c_double if dbl else ctypes.c_float), ctypes.byref(lda_),
       ctypes.byref(info))
    return info.value


def lapack_potrs(a: np.ndarray, b: np.ndarray, uplo: str = "L", nrhs: int | None = None, ldb: int | None = None,
                 n: int | None = None, lda: int | None = None) -> int:
    """?potrs_ through the Fortran ABI (b overwritten with the solution); returns info."""
    L = lapack()
    dbl = a.dtype == np.float64
    ct = ctypes.c_double if dbl else ctypes.c_float
    fn = L.dpotrs_ if dbl else L.spotrs_
    n_ = ctypes.c_int(a.shape[0] if n is None else n)
    k_ = ctypes.c_int((b.shape[1] if b.ndim == 2 else 1) if nrhs is None else nrhs)
    lda_ = ctypes.c_int(a.shape[0] if lda is None else lda)
    ldb_ = ctypes.c_int(b.shape[0] if ldb is None else ldb)
    info = ctypes.c_int(0)
    fn(uplo.encode(), ctypes.byref(n_), ctypes.byref(k_), _cptr(a, ct), ctypes.byref(lda_), _cptr(b, ct),
       ctypes.byref(ldb_), ctypes.byref(info))
    return info.value


def header_functions() -> list[str]:
    """Names of all functions declared in include/gbllt.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbllt_\w+)\s*\(", text)))


def check(fn: str, rc: int) -> None:
    if rc != SUCCESS:
        raise GblltError(fn, rc)


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())  # torch tensor


def _uplo(u: str) -> bytes:
    return u.encode()[:1]


# ---- host-pointer API (numpy, Fortran order) -------------------------------------------------

def potrf(a: np.ndarray, uplo: str = "L") -> int:
    """Factor a (n x n, float64/float32, Fortran order) in place; returns LAPACK info."""
    assert a.flags.f_contiguous and a.ndim == 2 and a.shape[0] == a.shape[1]
    info = _i64(0)
    fn = "gbllt_dpotrf" if a.dtype == np.float64 else "gbllt_spotrf"
    check(fn, getattr(lib(), fn)(COL_MAJOR, _uplo(uplo), a.shape[0], _ptr(a), max(1, a.shape[0]), ctypes.byref(info)))
    return int(info.value)


def potrs(a: np.ndarray, b: np.ndarray, uplo: str = "L") -> None:
    """Solve in place in b (n x k or n, Fortran order) from the factor in a."""
    n = a.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    fn = "gbllt_dpotrs" if a.dtype == np.float64 else "gbllt_spotrs"
    check(fn, getattr(lib(), fn)(COL_MAJOR, _uplo(uplo), n, k, _ptr(a), max(1, n), _ptr(b), max(1, n)))


def posv(a: np.ndarray, b: np.ndarray, uplo: str = "L") -> int:
    n = a.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    info = _i64(0)
    fn = "gbllt_dposv" if a.dtype == np.float64 else "gbllt_sposv"
    check(fn, getattr(lib(), fn)(COL_MAJOR, _uplo(uplo), n, k, _ptr(a), max(1, n), _ptr(b), max(1, n),
                                 ctypes.byref(info)))
    return int(info.value)


# ---- device-pointer API (torch tensors on cuda, column-major = transposed row-major storage) ----

def potrf_dev(a_cm, n: int, lda: int, info_dev, uplo: str = "L", stream: int = 0) -> None:
    import torch
    fn = "gbllt_dpotrf_dev" if a_cm.dtype == torch.float64 else "gbllt_spotrf_dev"
    check(fn, getattr(lib(), fn)(_uplo(uplo), n, _ptr(a_cm), lda, _ptr(info_dev), stream))


def potrs_dev(a_cm, n: int, lda: int, b_cm, nrhs: int, ldb: int, uplo: str = "L", stream: int = 0) -> None:
    import torch
    fn = "gbllt_dpotrs_dev" if a_cm.dtype == torch.float64 else "gbllt_spotrs_dev"
    check(fn, getattr(lib(), fn)(_uplo(uplo), n, nrhs, _ptr(a_cm), lda, _ptr(b_cm), ldb, stream))


def posv_mixed_dev(a_cm, n: int, lda: int, b_cm, ldb: int, x_cm, ldx: int, nrhs: int, opts: MixedOpts | None = None,
                   uplo: str = "L", stream: int = 0, raise_on_error: bool = True) -> tuple[int, dict]:
    """Mixed-precision solve with FP64 refinement on device buffers; returns (rc, report)."""
    rep = MixedReport()
    rc = lib().gbllt_dposv_mixed_dev(_uplo(uplo), n, nrhs, _ptr(a_cm), lda, _ptr(b_cm), ldb, _ptr(x_cm), ldx,
                                     ctypes.byref(opts) if opts is not None else None, ctypes.byref(rep), stream)
    if raise_on_error and rc not in (SUCCESS, ERR_NOT_CONVERGED):
        check("gbllt_dposv_mixed_dev", rc)
    return rc, rep.as_dict()


def posv_mixed(a: np.ndarray, b: np.ndarray, opts: MixedOpts | None = None, uplo: str = "L") -> tuple[np.ndarray, int, dict]:
    """Host-pointer mixed-precision solve (Fortran-order float64 arrays); returns (x, rc, report)."""
    n = a.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    x = np.zeros_like(b, order="F")
    rep = MixedReport()
    rc = lib().gbllt_dposv_mixed(COL_MAJOR, _uplo(uplo), n, k, _ptr(a), max(1, n), _ptr(b), max(1, n), _ptr(x),
                                 max(1, n), ctypes.byref(opts) if opts is not None else None, ctypes.byref(rep))
    if rc not in (SUCCESS, ERR_NOT_CONVERGED):
        check("gbllt_dposv_mixed", rc)
    return x, rc, rep.as_dict()


def potrf_adjoint_dev(l_cm, n: int, ldl: int, lbar_cm, ldlb: int, stream: int = 0, mixed: bool = False) -> None:
    """In place: lbar (df/dL, lower) becomes df/dA (lower triangle of the symmetric gradient); mixed:
    the panel products at 28 bits (gbllt_dpotrf_adjoint_mixed_dev)."""
    fn = "gbllt_dpotrf_adjoint_mixed_dev" if mixed else "gbllt_dpotrf_adjoint_dev"
    check(fn, getattr(lib(), fn)(n, _ptr(l_cm), ldl, _ptr(lbar_cm), ldlb, stream))


def potrs_adjoint_dev(l_cm, n: int, ldl: int, x_cm, ldx: int, xbar_cm, ldxb: int, bbar_cm, ldbb: int, nrhs: int,
                      abar_cm=None, ldab: int = 1, stream: int = 0) -> None:
    check("gbllt_dpotrs_adjoint_dev",
          lib().gbllt_dpotrs_adjoint_dev(n, nrhs, _ptr(l_cm), ldl, _ptr(x_cm), ldx, _ptr(xbar_cm), ldxb, _ptr(bbar_cm),
                                         ldbb, _ptr(abar_cm) if abar_cm is not None else None, max(ldab, 1), stream))


class BatchPlan:
    """A batched-solve plan (gbllt_batch_plan): sizes, packed offsets and the tuned kernel variant."""

    def __init__(self, sizes, dtype=np.float64):
        self.sizes = np.ascontiguousarray(np.asarray(sizes, dtype=np.int64))
        self.elem = 8 if np.dtype(dtype) == np.float64 else 4
        h = _vp()
        check("gbllt_batch_plan_create", lib().gbllt_batch_plan_create(len(self.sizes), self.sizes.ctypes.data,
                                                                       self.elem, ctypes.byref(h)))
        self.handle = h
        n = len(self.sizes)
        self.aoff = np.zeros(n, dtype=np.int64)
        self.boff = np.zeros(n, dtype=np.int64)
        ae, be = _i64(0), _i64(0)
        check("gbllt_batch_plan_layout", lib().gbllt_batch_plan_layout(h, self.aoff.ctypes.data, self.boff.ctypes.data,
                                                                       ctypes.byref(ae), ctypes.byref(be)))
        self.a_elems, self.b_elems = int(ae.value), int(be.value)

    def tune(self, cache_path: str | None = None, stream: int = 0) -> int:
        v = lib().gbllt_batch_plan_tune(self.handle, cache_path.encode() if cache_path else None, stream)
        if v < 0:
            check("gbllt_batch_plan_tune", v)
        return v

    def set_variant(self, v: int) -> None:
        check("gbllt_batch_plan_set_variant", lib().gbllt_batch_plan_set_variant(self.handle, v))

    def variant(self) -> dict:
        p, t, m = _int(0), _int(0), _int(0)
        v = lib().gbllt_batch_plan_variant(self.handle, ctypes.byref(p), ctypes.byref(t), ctypes.byref(m))
        return {"variant": v, "panel": p.value, "threads": t.value, "smem_max_n": m.value}

    def solve_dev(self, a, b, info, stream: int = 0) -> None:
        fn = "gbllt_dposv_batched_dev" if self.elem == 8 else "gbllt_sposv_batched_dev"
        check(fn, getattr(lib(), fn)(self.handle, _ptr(a), _ptr(b), _ptr(info), stream))

    def solve_mixed_dev(self, a, b, x, info, opts: "MixedOpts | None" = None, stream: int = 0) -> dict:
        """gbllt_batch_dposv_mixed_dev: FP64 systems solved with FP32 factors and FP64 refinement;
        a and b are read only, x receives the solutions.  Returns the report."""
        rep = BatchMixedReport()
        check("gbllt_batch_dposv_mixed_dev",
              lib().gbllt_batch_dposv_mixed_dev(self.handle, _ptr(a), _ptr(b), _ptr(x), _ptr(info),
                                                ctypes.byref(opts) if opts is not None else None,
                                                ctypes.byref(rep), stream))
        return rep.as_dict()

    def solve(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        info = np.zeros(len(self.sizes), dtype=np.int64)
        fn = "gbllt_dposv_batched" if self.elem == 8 else "gbllt_sposv_batched"
        check(fn, getattr(lib(), fn)(self.handle, _ptr(a), _ptr(b), info.ctypes.data))
        return info

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                lib().gbllt_batch_plan_destroy(self.handle)
                self.handle = None
        except Exception:  # pragma: no cover
            pass


# ---- diagnostics -------------------------------------------------------------------------------

def profile_enable(on: bool = True) -> None:
    check("gbllt_profile_enable", lib().gbllt_profile_enable(1 if on else 0))


def rank_update(l: np.ndarray, v: np.ndarray, sigma: float, uplo: str = "L") -> int:
    """In place on a Fortran-order factor: the factor of A + sigma v v^T; returns the LAPACK-style info."""
    dbl = l.dtype == np.float64
    fn = lib().gbllt_drank_update if dbl else lib().gbllt_srank_update
    n = l.shape[0]
    vv = np.ascontiguousarray(v, dtype=l.dtype)
    info = ctypes.c_int64(0)
    check("gbllt_?rank_update", fn(COL_MAJOR, uplo.encode(), n, l.ctypes.data if n else None, max(n, 1),
                                    vv.ctypes.data if n else None, sigma, ctypes.byref(info)))
    return info.value


def rank_update_dev(d_l, n: int, ldl: int, d_v, sigma: float, d_info, uplo: str = "L", stream=None,
                    dtype=np.float64) -> None:
    """Device-pointer form (torch tensors); the info is written to the device scalar d_info."""
    fn = lib().gbllt_drank_update_dev if dtype == np.float64 else lib().gbllt_srank_update_dev
    check("gbllt_?rank_update_dev", fn(uplo.encode(), n, _ptr(d_l), ldl, _ptr(d_v), sigma, _ptr(d_info), stream))


SIGN_NAMES = ("PositiveSemiDef", "NegativeSemiDef", "ZeroSign", "Indefinite")


def ldlt(a: np.ndarray, uplo: str = "L") -> tuple[int, np.ndarray, int]:
    """Pivoted LDL^T in place on a Fortran-order array (LDLT::compute); returns (info, transpositions,
    sign): info 0 = Success, 1 = NumericalIssue; sign indexes SIGN_NAMES."""
    dbl = a.dtype == np.float64
    fn = lib().gbllt_dldlt if dbl else lib().gbllt_sldlt
    n = a.shape[0]
    t = np.zeros(max(n, 1), dtype=np.int32)
    sign = ctypes.c_int32(0)
    info = ctypes.c_int64(0)
    check("gbllt_?ldlt", fn(COL_MAJOR, uplo.encode(), n, a.ctypes.data if n else None, max(n, 1), t.ctypes.data,
                            ctypes.byref(sign), ctypes.byref(info)))
    return int(info.value), t[:n], int(sign.value)


def ldlt_pivots(diag: np.ndarray) -> np.ndarray:
    """The transpositions LDLT::compute chooses for this diagonal (host computation)."""
    d = np.ascontiguousarray(diag)
    fn = lib().gbllt_dldlt_pivots if d.dtype == np.float64 else lib().gbllt_sldlt_pivots
    n = d.shape[0]
    t = np.zeros(max(n, 1), dtype=np.int32)
    check("gbllt_?ldlt_pivots", fn(n, d.ctypes.data if n else None, 1, t.ctypes.data))
    return t[:n]


def ldlt_solve(f: np.ndarray, transp: np.ndarray, b: np.ndarray, uplo: str = "L") -> None:
    """In place in b (n or n x k, Fortran order): A^{-1} b from the LDL^T factor and transpositions."""
    dbl = f.dtype == np.float64
    fn = lib().gbllt_dldlt_solve if dbl else lib().gbllt_sldlt_solve
    n = f.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    t = np.ascontiguousarray(transp, dtype=np.int32)
    check("gbllt_?ldlt_solve", fn(COL_MAJOR, uplo.encode(), n, k, f.ctypes.data if n else None, max(n, 1),
                                  t.ctypes.data if n else None, b.ctypes.data if n else None, max(n, 1)))


def ldlt_dev(d_a, n: int, lda: int, uplo: str = "L", stream=None, dtype=np.float64) -> tuple[int, np.ndarray, int]:
    """Device-pointer form (torch tensor, column-major); returns (info, transpositions, sign)."""
    fn = lib().gbllt_dldlt_dev if dtype == np.float64 else lib().gbllt_sldlt_dev
    t = np.zeros(max(n, 1), dtype=np.int32)
    sign = ctypes.c_int32(0)
    info = ctypes.c_int64(0)
    check("gbllt_?ldlt_dev", fn(uplo.encode(), n, _ptr(d_a), lda, t.ctypes.data, ctypes.byref(sign),
                                ctypes.byref(info), stream))
    return int(info.value), t[:n], int(sign.value)


def ldlt_solve_dev(d_a, n: int, lda: int, transp: np.ndarray, d_b, nrhs: int, ldb: int, uplo: str = "L",
                   stream=None, dtype=np.float64) -> None:
    fn = lib().gbllt_dldlt_solve_dev if dtype == np.float64 else lib().gbllt_sldlt_solve_dev
    t = np.ascontiguousarray(transp, dtype=np.int32)
    check("gbllt_?ldlt_solve_dev", fn(uplo.encode(), n, nrhs, _ptr(d_a), lda, t.ctypes.data, _ptr(d_b), ldb, stream))


def syrk(c: np.ndarray, a: np.ndarray, uplo: str = "L", trans: str = "N", alpha: float = 1.0,
         beta: float = 0.0) -> None:
    """In place on the Fortran-order c (n x n): the `uplo` triangle <- alpha op(a) op(a)^T + beta c."""
    dbl = c.dtype == np.float64
    fn = lib().gbllt_dsyrk if dbl else lib().gbllt_ssyrk
    n = c.shape[0]
    k = a.shape[1] if trans.upper() == "N" else a.shape[0]
    lda = max(1, a.shape[0])
    check("gbllt_?syrk", fn(COL_MAJOR, uplo.encode(), trans.encode(), n, k, alpha, a.ctypes.data if a.size else None,
                            lda, beta, c.ctypes.data if n else None, max(1, n)))


def trsm(b: np.ndarray, a: np.ndarray, side: str = "L", uplo: str = "L", trans: str = "N", diag: str = "N",
         alpha: float = 1.0) -> None:
    """In place on the Fortran-order b (m x n): alpha op(a)^{-1} b (side 'L') or alpha b op(a)^{-1}."""
    dbl = b.dtype == np.float64
    fn = lib().gbllt_dtrsm if dbl else lib().gbllt_strsm
    m, n = b.shape
    check("gbllt_?trsm", fn(COL_MAJOR, side.encode(), uplo.encode(), trans.encode(), diag.encode(), m, n, alpha,
                            a.ctypes.data if a.size else None, max(1, a.shape[0]), b.ctypes.data if b.size else None,
                            max(1, m)))


def pocon(l: np.ndarray, anorm: float, uplo: str = "L") -> float:
    """Reciprocal condition estimate from a host factor (Fortran-order float64/float32 array)."""
    dbl = l.dtype == np.float64
    out = ctypes.c_double(0.0) if dbl else ctypes.c_float(0.0)
    fn = lib().gbllt_dpocon if dbl else lib().gbllt_spocon
    n = l.shape[0]
    check("gbllt_?pocon", fn(COL_MAJOR, uplo.encode(), n, l.ctypes.data if n else None, max(n, 1), anorm,
                            ctypes.byref(out)))
    return out.value


def pocon_dev(d_l, n: int, ldl: int, anorm: float, uplo: str = "L", stream=None, dtype=np.float64) -> float:
    """Device-pointer form: d_l is a device tensor holding the factor."""
    dbl = dtype == np.float64
    out = ctypes.c_double(0.0) if dbl else ctypes.c_float(0.0)
    fn = lib().gbllt_dpocon_dev if dbl else lib().gbllt_spocon_dev
    check("gbllt_?pocon_dev", fn(uplo.encode(), n, _ptr(d_l), ldl, anorm, ctypes.byref(out), stream))
    return out.value


def lansy_l1_dev(d_a, n: int, lda: int, d_norm, uplo: str = "L", stream=None, dtype=np.float64) -> None:
    """1-norm of the symmetric matrix stored in one triangle of d_a, written to the device scalar d_norm."""
    fn = lib().gbllt_dlansy_l1_dev if dtype == np.float64 else lib().gbllt_slansy_l1_dev
    check("gbllt_?lansy_l1_dev", fn(uplo.encode(), n, _ptr(d_a), lda, _ptr(d_norm), stream))


def selftest_wait_timeout(wait_us: int = 20000) -> tuple[int, int]:
    """Run the bounded-wait self-test; returns (return code, the code the waits reported)."""
    obs = _int(0)
    rc = lib().gbllt_selftest_wait_timeout(wait_us, ctypes.byref(obs))
    return int(rc), int(obs.value)


def profile_read() -> dict[str, dict]:
    """Per-kernel-class launches, device ms and algorithmic flops / bytes since profile_enable."""
    cap = 64
    arr = (KernelStat * cap)()
    cnt = _int(0)
    check("gbllt_profile_read", lib().gbllt_profile_read(ctypes.cast(arr, _vp), cap, ctypes.byref(cnt)))
    out = {}
    for i in range(min(cnt.value, cap)):
        s = arr[i]
        out[s.name.decode()] = dict(launches=int(s.launches), ms=float(s.ms), flops=float(s.flops),
                                    bytes=float(s.bytes))
    return out


def profile_trace(cap: int = 1 << 20) -> list[dict]:
    """Every launch recorded since profile_enable, in launch order: kernel class, stream, device
    start / end (ms after the first recorded launch), algorithmic flops and bytes."""
    cnt = _int(0)
    check("gbllt_profile_trace", lib().gbllt_profile_trace(None, 0, ctypes.byref(cnt)))
    n = min(cnt.value, cap)
    arr = (LaunchRecord * max(n, 1))()
    check("gbllt_profile_trace", lib().gbllt_profile_trace(ctypes.cast(arr, _vp), n, ctypes.byref(cnt)))
    return [dict(name=arr[i].name.decode(), stream=int(arr[i].stream), start_ms=float(arr[i].start_ms),
                 end_ms=float(arr[i].end_ms), flops=float(arr[i].flops), bytes=float(arr[i].bytes))
            for i in range(n)]
