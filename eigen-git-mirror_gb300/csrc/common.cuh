// Shared definitions for the GB300 dense Cholesky (LLT) kernels and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "../../include/gbllt.h"

namespace gbllt {

// Status word shared by every launch of one factorisation: -1 while all pivots so far were
// positive, else the 0-based global column of the first non-positive pivot.  Kernels read it on
// entry and return early once it is set, so a failed factorisation costs no further work and
// the host reads one word at the end (the same information LLT::compute keeps in m_info,
// Eigen/src/Cholesky/LLT.h:457).
struct DevStatus {
  long long fail_col;   // -1 = ok
  int timeout;          // a bounded wait ran out (never expected; reported as GBLLT_ERR_TIMEOUT)
  int pad;
};

#define GB_CUDA_TRY(expr)                                                        \
  do {                                                                           \
    cudaError_t err__ = (expr);                                                  \
    if (err__ != cudaSuccess) {                                                  \
      gbllt::set_last_error(err__, #expr, __FILE__, __LINE__);                   \
      return GBLLT_ERR_CUDA;                                                     \
    }                                                                            \
  } while (0)

void set_last_error(cudaError_t e, const char* what, const char* file, int line);
void set_error_message(const char* msg);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Every device allocation of the library goes through these (stream-ordered, or plain for the
// long-lived plan buffers).  With GBLLT_INJECT_ALLOC_FAILURE=1 in the environment they fail with
// cudaErrorMemoryAllocation without calling CUDA: host-side fault injection, so that the
// allocation-failure paths can be tested without exhausting a shared GPU's memory.
cudaError_t dev_malloc_async(void** p, size_t bytes, cudaStream_t s);
cudaError_t dev_malloc(void** p, size_t bytes);

// Per-thread, per-device library stream for the synchronous host-pointer entry points.
cudaStream_t lib_stream();

// Lower-triangle tile enumeration: tile t -> (ti, tj) with 0 <= tj <= ti.
__device__ __forceinline__ void lower_tile_coords(long long t, int& ti, int& tj) {
  long long i = (long long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  while (i * (i + 1) / 2 > t) --i;
  ti = (int)i;
  tj = (int)(t - i * (i + 1) / 2);
}

// FP32 rounded to TF32 (13 zero low bits), to nearest with ties away: one part of the split
// operands of the tensor-core updates.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

}  // namespace gbllt
