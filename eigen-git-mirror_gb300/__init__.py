"""GB300-native (sm_103a) backend for Eigen's dense Cholesky path, LLT::compute / LLT::solve.

The product is libgbllt.so (CUDA kernels behind the C ABI in include/gbllt.h) and the Eigen
backend header include/eigen_gb300/LLT_GB300.h.  This Python package only builds the library
and exposes a ctypes binding for the test suite and the benchmark.
"""
from . import gbllt  # noqa: F401
from .build import build  # noqa: F401
