"""Build libgbllt.so (the sm_103a CUDA kernels + C ABI) in-tree.

Every translation unit under csrc/ is compiled by nvcc for sm_103a only, in parallel, and the
objects are linked into lib/libgbllt.so.  Nothing is installed into site-packages; callers load
the library from this directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libgbllt.so"
LAPACK_LIB = PKG / "lib" / "libgbllt_lapack.so"  # Fortran-ABI dpotrf_/dpotrs_/spotrf_/spotrs_ shim
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    if obj.exists() and obj.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    return obj


def build_lapack_shim(force: bool = False) -> Path:
    """libgbllt_lapack.so: the Fortran-ABI Cholesky routines (C, gcc) linked against libgbllt.so."""
    src = CSRC / "lapack_shim.c"
    deps = [src, LIB, INCLUDE / "gbllt.h", INCLUDE / "gbllt_lapack.h"]
    if not force and LAPACK_LIB.exists() and LAPACK_LIB.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return LAPACK_LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    cmd = [cc, "-O2", "-fPIC", "-shared", "-fvisibility=hidden", "-I", str(INCLUDE), str(src), "-o", str(LAPACK_LIB),
           "-L", str(LIB.parent), "-lgbllt", "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"LAPACK shim build failed:\n{res.stdout}\n{res.stderr}")
    return LAPACK_LIB


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if force or not LIB.exists() or LIB.stat().st_mtime <= max(o.stat().st_mtime for o in objs):
        # libcuda is not linked: driver entry points (tensor-map encoding) are fetched at run time
        # through cudaGetDriverEntryPoint, so the library also loads on a machine without a driver.
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    build_lapack_shim(force)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
