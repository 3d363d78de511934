// Batched factor + solve of many small SPD systems of uneven sizes in one persistent launch.
//
// Each system s is an independent LLT<MatrixX?>(A_s).solve(b_s) (Eigen/src/Cholesky/LLT.h:430-498):
// A_s is n_s x n_s column-major at a + aoff[s] (lower triangle read and overwritten with L_s),
// b_s holds n_s values at b + boff[s] and is overwritten with x_s; info[s] is the LAPACK info.
//
// Launch structure: a persistent grid (a multiple of the SM count) pulls systems from a device
// work queue ordered largest-first, so the long systems start early and the short ones fill the
// tail.  A system whose matrix fits in shared memory is staged there (lower triangle, odd leading
// dimension), otherwise it is worked on in place in global memory (L2-resident at these sizes).
// Per system, the blocked right-looking algorithm of llt_inplace::blocked (LLT.h:338-368) runs
// with NBP-wide panels, in one of two forms the autotuner chooses between:
//   algo 0: the panel is factored one column at a time by all threads (the role of unblocked(),
//           LLT.h:312-336, with the same `x <= 0` pivot test), then all threads apply the trailing
//           update with 4 x 4 register tiles;
//   algo 1 (factor_blk): warp 0 factors the panel's diagonal block, each thread solves whole rows
//           below it, and the trailing update reads the panel from a shared-memory copy (lower
//           tiles only, column-major tile order).
// The solve is blocked by 32 rows in both: each diagonal block is staged in shared memory and
// substituted by warp 0 with shuffles, all warps apply the off-diagonal blocks (GEMV forward,
// warp-shuffle dot products backward).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "internal.h"

namespace gbllt {

namespace {

constexpr int kMaxBatchN = 1024;  // largest system order the batched path accepts

template <typename T>
struct BatchArgs {
  T* a;
  T* b;
  int64_t* info;
  const int* order;     // system indices, largest first
  const int* n;         // orders
  const int64_t* aoff;  // element offsets of each A
  const int64_t* boff;  // element offsets of each b
  int count;
  int* counter;         // work-queue ticket, zeroed before each launch
  int smem_max_n;       // systems with n <= smem_max_n are staged in shared memory
  int psld;             // algo 1: leading dimension of the shared panel copy (round_up(max n, 4))
};

// The two sweeps of the solve (LLT.h:483-498) on the factored system, in blocks of 32 rows.  Each
// 32 x 32 diagonal block is first staged in shared memory (Dg, coalesced loads by all threads); warp 0
// then substitutes inside it with the block's right-hand sides in registers (lane = row), one
// warp shuffle per step and the pivots' reciprocals precomputed, so the sequential part touches
// neither global memory nor a CTA barrier.  All warps apply the off-diagonal blocks (a GEMV
// forward, warp-shuffle dot products backward).
constexpr int kDgLd = 33;  // Dg[r * kDgLd + c] = L(j0 + r, j0 + c), r >= c

template <typename T, int THREADS>
__device__ void solve_sweeps(const T* M, int ld, int n, T* bv, T* Dg) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto load_diag = [&](int j0, int jb) {
    for (int idx = tid; idx < jb * jb; idx += THREADS) {
      const int r = idx % jb, c = idx / jb;
      if (r >= c) Dg[r * kDgLd + c] = M[(j0 + r) + (long long)(j0 + c) * ld];
    }
  };
  // L y = b
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int jb = min(32, n - j0);
    load_diag(j0, jb);
    __syncthreads();
    if (warp == 0) {
      T b = lane < jb ? bv[j0 + lane] : T(0);
      const T rinv = lane < jb ? T(1) / Dg[lane * kDgLd + lane] : T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (j < jb) {
          const T yj = __shfl_sync(0xffffffffu, b * rinv, j);
          if (lane > j && lane < jb) b = fma(-Dg[lane * kDgLd + j], yj, b);
          if (lane == j) b = yj;
        }
      }
      if (lane < jb) bv[j0 + lane] = b;
    }
    __syncthreads();
    for (int i = j0 + jb + tid; i < n; i += THREADS) {
      T s = T(0);
#pragma unroll 8
      for (int p = j0; p < j0 + jb; ++p) s = fma(M[i + (long long)p * ld], bv[p], s);
      bv[i] -= s;
    }
    __syncthreads();
  }
  // L^T x = y
  for (int j0 = ((n - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int jb = min(32, n - j0);
    load_diag(j0, jb);
    for (int c = j0 + warp; c < j0 + jb; c += THREADS / 32) {
      T s = T(0);
      for (int r = j0 + jb + lane; r < n; r += 32) s = fma(M[r + (long long)c * ld], bv[r], s);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
      if (lane == 0) bv[c] -= s;
    }
    __syncthreads();
    if (warp == 0) {
      T b = lane < jb ? bv[j0 + lane] : T(0);
      const T rinv = lane < jb ? T(1) / Dg[lane * kDgLd + lane] : T(0);
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        if (j < jb) {
          const T xj = __shfl_sync(0xffffffffu, b * rinv, j);
          if (lane < j) b = fma(-Dg[j * kDgLd + lane], xj, b);
          if (lane == j) b = xj;
        }
      }
      if (lane < jb) bv[j0 + lane] = b;
    }
    __syncthreads();
  }
}

// Factor + solve one system held in M (leading dimension ld), right-hand side in bv (shared).
// Returns -1 on success or the failing column.  All threads of the CTA call it.
template <typename T, int NBP, int THREADS>
__device__ int factor_solve(T* M, int ld, int n, T* bv, T* Dg, int* s_fail, T* s_inv) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) *s_fail = -1;
  __syncthreads();
  for (int k0 = 0; k0 < n; k0 += NBP) {
    const int kb = min(NBP, n - k0);
    // ---- panel: columns k0 .. k0+kb, rows k0 .. n, by all threads, one column at a time
    for (int j = k0; j < k0 + kb; ++j) {
      if (tid == 0) {
        const T d = M[j + (long long)j * ld];
        if (d <= T(0)) {
          *s_fail = j;
        } else {
          const T r = sqrt(d);
          M[j + (long long)j * ld] = r;
          *s_inv = T(1) / r;  // one division per column; the column is scaled by multiplication
        }
      }
      __syncthreads();
      if (*s_fail >= 0) return *s_fail;
      const T inv = *s_inv;
      for (int i = j + 1 + tid; i < n; i += THREADS) M[i + (long long)j * ld] *= inv;
      __syncthreads();
      // remaining panel columns: one warp per column, lanes over rows
      for (int l = j + 1 + warp; l < k0 + kb; l += THREADS / 32) {
        const T mlj = M[l + (long long)j * ld];
        for (int i = l + lane; i < n; i += 32) M[i + (long long)l * ld] -= M[i + (long long)j * ld] * mlj;
      }
      __syncthreads();
    }
    // ---- trailing update: rows / columns r0 .. n, lower 4 x 4 tiles
    const int r0 = k0 + kb;
    const int m = n - r0;
    if (m > 0) {
      const int mt = (m + 3) >> 2;
      for (int idx = tid; idx < mt * mt; idx += THREADS) {
        const int ti = idx % mt, tj = idx / mt;
        if (ti < tj) continue;
        const int i0 = r0 + 4 * ti, j0 = r0 + 4 * tj;
        T acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
        for (int p = k0; p < r0; ++p) {
          const T* col = M + (long long)p * ld;
          T ar[4], ac[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) ar[u] = i0 + u < n ? col[i0 + u] : T(0);
#pragma unroll
          for (int v = 0; v < 4; ++v) ac[v] = j0 + v < n ? col[j0 + v] : T(0);
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fma(ar[u], ac[v], acc[u][v]);
        }
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int i = i0 + u, j = j0 + v;
            if (i < n && j < n && i >= j) M[i + (long long)j * ld] -= acc[u][v];
          }
      }
    }
    __syncthreads();
  }
  solve_sweeps<T, THREADS>(M, ld, n, bv, Dg);
  return -1;
}

// Four consecutive values from 16-byte aligned (float) / 32-byte aligned (double) shared memory.
__device__ __forceinline__ void load4(const float* p, float* o) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void load4(const double* p, double* o) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  const double2 b = *reinterpret_cast<const double2*>(p + 2);
  o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}

// Panel-blocked factorisation (the kernel variants with algo = 1).  Per NBP-wide panel at k0:
//   1. warp 0 factors the kb x kb diagonal block in shared memory (Ds), one column per step with
//      the rows spread over the lanes and only warp-level synchronisation: unblocked() of
//      LLT.h:312-336 with its `x <= 0` test, so the failing column is the same;
//   2. every thread solves whole rows below the block against it (L21 = A21 L11^{-T}, the row's
//      kb values in registers, no synchronisation inside), storing them to M and to the
//      shared panel copy Ps (Ps[p * psld + r] = L(r0 + r, k0 + p));
//   3. the trailing update A22 -= L21 L21^T reads L21 from Ps only: 4 x 4 register tiles over the
//      lower tiles in column-major order, so the lanes of a warp share the tile column (its 4
//      panel values are a shared-memory broadcast) and cover consecutive rows of M (coalesced).
// Four CTA barriers per panel instead of three per column.
template <typename T, int NBP, int THREADS>
__device__ int factor_blk(T* M, int ld, int n, T* Ds, T* Dinv, T* Ps, int psld, int* s_fail) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int DLD = NBP + 1;
  if (tid == 0) *s_fail = -1;
  for (int k0 = 0; k0 < n; k0 += NBP) {
    const int kb = min(NBP, n - k0);
    for (int idx = tid; idx < kb * kb; idx += THREADS) {
      const int r = idx % kb, c = idx / kb;
      if (r >= c) Ds[r * DLD + c] = M[(k0 + r) + (long long)(k0 + c) * ld];
    }
    __syncthreads();
    if (warp == 0) {
      for (int j = 0; j < kb; ++j) {
        const T d = Ds[j * DLD + j];
        if (d <= T(0)) {  // the `x <= 0` test of LLT.h:328 (a NaN pivot passes it)
          if (lane == 0) *s_fail = k0 + j;
          break;
        }
        const T rt = sqrt(d), inv = T(1) / rt;
        const int i = j + 1 + lane;
        T lij = T(0);
        if (i < kb) {
          lij = Ds[i * DLD + j] * inv;
          Ds[i * DLD + j] = lij;
        }
        __syncwarp();
        if (i < kb)
          for (int l = j + 1; l <= i; ++l) Ds[i * DLD + l] -= lij * Ds[l * DLD + j];
        if (lane == 0) {
          Ds[j * DLD + j] = rt;
          Dinv[j] = inv;
        }
        __syncwarp();
      }
    }
    __syncthreads();
    if (*s_fail >= 0) return *s_fail;
    // the factored diagonal block back to M; rows below: L21 = A21 L11^{-T}, one thread per row
    for (int idx = tid; idx < kb * kb; idx += THREADS) {
      const int r = idx % kb, c = idx / kb;
      if (r >= c) M[(k0 + r) + (long long)(k0 + c) * ld] = Ds[r * DLD + c];
    }
    const int r0 = k0 + kb;
    const int m = n - r0;
    for (int r = tid; r < m; r += THREADS) {
      T x[NBP];
#pragma unroll
      for (int c = 0; c < NBP; ++c) x[c] = c < kb ? M[(r0 + r) + (long long)(k0 + c) * ld] : T(0);
#pragma unroll
      for (int c = 0; c < NBP; ++c) {
        if (c < kb) {
          T v = x[c];
#pragma unroll
          for (int q = 0; q < c; ++q) v = fma(-x[q], Ds[c * DLD + q], v);
          x[c] = v * Dinv[c];
        }
      }
#pragma unroll
      for (int c = 0; c < NBP; ++c)
        if (c < kb) {
          M[(r0 + r) + (long long)(k0 + c) * ld] = x[c];
          Ps[c * psld + r] = x[c];
        }
    }
    __syncthreads();
    if (m > 0) {
      // lower 4 x 4 tiles of the m x m trailing matrix, column-major: tile t -> (tile column tj,
      // offset o = ti - tj), advanced incrementally by THREADS
      const int mt = (m + 3) >> 2;
      const int ntile = mt * (mt + 1) / 2;
      int tj = 0, o = tid;
      while (tj < mt && o >= mt - tj) { o -= mt - tj; ++tj; }
      for (int t = tid; t < ntile; t += THREADS) {
        const int ti = tj + o;
        const int i0 = 4 * ti, j0 = 4 * tj;
        // the tile of A22 is fetched before the product, so its (L2) latency overlaps the FMAs
        T acc[4][4];
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int i = i0 + u, j = j0 + v;
            acc[u][v] = (i < m && j < m && i >= j) ? M[(r0 + i) + (long long)(r0 + j) * ld] : T(0);
          }
        for (int p = 0; p < kb; ++p) {
          const T* pr = Ps + p * psld;
          T ar[4], ac[4];
          load4(pr + i0, ar);
          load4(pr + j0, ac);
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fma(-ar[u], ac[v], acc[u][v]);
        }
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int i = i0 + u, j = j0 + v;
            if (i < m && j < m && i >= j) M[(r0 + i) + (long long)(r0 + j) * ld] = acc[u][v];
          }
        o += THREADS;
        while (tj < mt && o >= mt - tj) { o -= mt - tj; ++tj; }
      }
    }
    __syncthreads();
  }
  return -1;
}

// Shared-memory carve-up of the kernels: [bv: kMaxBatchN][Dg: 32 x 33][Ds: NBP(NBP+1)][Dinv: NBP]
// [Ps: NBP psld][staged matrix], Ds/Dinv/Ps only for algo 1; every part starts on a multiple of 4
// elements (32 x 33 = 1056).
template <typename T>
__host__ __device__ constexpr size_t blk_elems(int nbp, int psld) {
  return (size_t)nbp * (nbp + 1) + (size_t)nbp + (size_t)nbp * psld;
}

template <typename T, int NBP, int THREADS, int ALGO, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) batched_posv_kernel(BatchArgs<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* bv = reinterpret_cast<T*>(smem_raw);          // kMaxBatchN values
  T* Dg = bv + kMaxBatchN;                         // the solve's 32 x 32 diagonal block
  T* Ds = Dg + 32 * kDgLd;                         // algo 1: diagonal block, its inverse pivots, panel
  T* Dinv = Ds + NBP * (NBP + 1);
  T* Ps = Dinv + NBP;
  T* sm = ALGO == 1 ? Ds + blk_elems<T>(NBP, p.psld) : Ds;  // staged matrix
  __shared__ int s_ticket, s_fail;
  __shared__ T s_inv;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_ticket = atomicAdd(p.counter, 1);
    __syncthreads();
    const int t = s_ticket;
    __syncthreads();
    if (t >= p.count) break;
    const int sys = p.order[t];
    const int n = p.n[sys];
    T* A = p.a + p.aoff[sys];
    T* B = p.b + p.boff[sys];
    const bool staged = n <= p.smem_max_n;
    const int ld = staged ? (n | 1) : n;
    T* M = staged ? sm : A;
    if (staged)
      for (int idx = tid; idx < n * n; idx += THREADS) {
        const int i = idx % n, j = idx / n;
        if (i >= j) M[i + j * ld] = A[(long long)j * n + i];
      }
    for (int i = tid; i < n; i += THREADS) bv[i] = B[i];
    __syncthreads();
    int fail = -1;
    if (n > 0) {
      if (ALGO == 0) {
        fail = factor_solve<T, NBP, THREADS>(M, ld, n, bv, Dg, &s_fail, &s_inv);
      } else {
        fail = factor_blk<T, NBP, THREADS>(M, ld, n, Ds, Dinv, Ps, p.psld, &s_fail);
        if (fail < 0) solve_sweeps<T, THREADS>(M, ld, n, bv, Dg);
      }
    }
    if (staged)
      for (int idx = tid; idx < n * n; idx += THREADS) {
        const int i = idx % n, j = idx / n;
        if (i >= j) A[(long long)j * n + i] = M[i + j * ld];
      }
    if (fail < 0)
      for (int i = tid; i < n; i += THREADS) B[i] = bv[i];
    if (tid == 0) p.info[sys] = fail < 0 ? 0 : (int64_t)fail + 1;
    __syncthreads();
  }
}

// ---- variants and launch ---------------------------------------------------------------------

// Kernel variants the autotuner sweeps: algorithm (0: column at a time, 1: panel-blocked) x panel
// width x threads per CTA x the largest order staged in shared memory (-1 = as large as fits in one
// CTA's shared memory; smaller caps leave room for more CTAs per SM, the larger systems then running
// in place in global memory, L2-resident).
// The last two variants ask the compiler for 8 (4) resident CTAs of 128 (256) threads, i.e. at
// most 64 registers per thread, trading registers for warps that hide latency.
struct Variant {
  int algo, nbp, threads, smem_cap, min_blocks;
};
constexpr Variant kVariants[] = {
    {0, 16, 128, -1, 1}, {0, 32, 128, -1, 1}, {0, 16, 256, -1, 1}, {0, 32, 256, -1, 1},
    {0, 16, 128, 96, 1}, {0, 16, 256, 96, 1}, {0, 16, 128, 0, 1},  {0, 16, 256, 0, 1},
    {1, 16, 128, 0, 1},  {1, 16, 256, 0, 1},  {1, 32, 128, 0, 1},  {1, 32, 256, 0, 1},
    {1, 16, 128, -1, 1}, {1, 16, 256, 96, 1}, {1, 16, 128, 0, 8},  {1, 16, 256, 0, 4}};
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
static_assert(kNumVariants == GBLLT_BATCH_VARIANTS, "gbllt.h states the number of batched kernel variants");

template <typename T>
using BatchKernel = void (*)(BatchArgs<T>);

// kernel of each variant, in the order of kVariants
template <typename T>
BatchKernel<T> kernel_of(int v) {
  static const BatchKernel<T> table[] = {
      batched_posv_kernel<T, 16, 128, 0, 1>, batched_posv_kernel<T, 32, 128, 0, 1>,
      batched_posv_kernel<T, 16, 256, 0, 1>, batched_posv_kernel<T, 32, 256, 0, 1>,
      batched_posv_kernel<T, 16, 128, 0, 1>, batched_posv_kernel<T, 16, 256, 0, 1>,
      batched_posv_kernel<T, 16, 128, 0, 1>, batched_posv_kernel<T, 16, 256, 0, 1>,
      batched_posv_kernel<T, 16, 128, 1, 1>, batched_posv_kernel<T, 16, 256, 1, 1>,
      batched_posv_kernel<T, 32, 128, 1, 1>, batched_posv_kernel<T, 32, 256, 1, 1>,
      batched_posv_kernel<T, 16, 128, 1, 1>, batched_posv_kernel<T, 16, 256, 1, 1>,
      batched_posv_kernel<T, 16, 128, 1, 8>, batched_posv_kernel<T, 16, 256, 1, 4>};
  static_assert(sizeof(table) / sizeof(table[0]) == kNumVariants, "one kernel per variant");
  return table[v];
}

// Dynamic shared memory of a variant: b, the algo-1 panel buffers, and the staged matrix.
template <typename T>
size_t smem_bytes(int variant, int smem_max_n, int psld) {
  const Variant v = kVariants[variant];
  size_t e = (size_t)kMaxBatchN + 32 * kDgLd + (v.algo == 1 ? blk_elems<T>(v.nbp, psld) : 0);
  if (smem_max_n > 0) e += (size_t)(smem_max_n | 1) * smem_max_n;
  return e * sizeof(T);
}

template <typename T>
int launch_batched(int variant, const BatchArgs<T>& args, int grid, size_t smem, cudaStream_t s) {
  const BatchKernel<T> kern = kernel_of<T>(variant);
  GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, kVariants[variant].threads, smem, s>>>(args);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int occupancy(int variant, size_t smem) {
  int blocks = 0;
  const BatchKernel<T> f = kernel_of<T>(variant);
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, f, kVariants[variant].threads, smem);
  return blocks;
}

// Synthetic SPD systems with the plan's sizes (A = I * n + 1/(1 + |i - j|), b = 1) for timing.
template <typename T>
__global__ void fill_tuning_kernel(T* a, T* b, const int* n, const int64_t* aoff, const int64_t* boff, int count) {
  const int s = blockIdx.x;
  if (s >= count) return;
  const int m = n[s];
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    const int i = idx % m, j = idx / m;
    a[aoff[s] + idx] = (i == j ? T(m) : T(0)) + T(1) / T(1 + abs(i - j));
  }
  for (int i = threadIdx.x; i < m; i += blockDim.x) b[boff[s] + i] = T(1);
}

}  // namespace

// ---- plans ------------------------------------------------------------------------------------

struct BatchPlan {
  int64_t count = 0;
  int elem = 8;  // 8 = double, 4 = float
  int64_t a_elems = 0, b_elems = 0;
  int max_n = 0;
  std::vector<int> h_n;
  std::vector<int64_t> h_aoff, h_boff;
  // device arrays (one allocation)
  void* dev = nullptr;
  int* d_order = nullptr;
  int* d_n = nullptr;
  int64_t* d_aoff = nullptr;
  int64_t* d_boff = nullptr;
  int* d_counter = nullptr;
  int device = 0;
  int variant = 3;
  int smem_max_n = 0;
  int psld = 4;  // algo-1 panel copy: round_up(max_n, 4)
  int grid = 0;
  size_t smem = 0;
  double tuned_ms[kNumVariants] = {};
  // the FP32 plan of the same sizes that the mixed-precision solve factors with (made and tuned on
  // its first call)
  BatchPlan* f32 = nullptr;
  // cached graph
  cudaGraphExec_t exec = nullptr;
  void* g_a = nullptr;
  void* g_b = nullptr;
  void* g_info = nullptr;
  std::mutex mu;
};

namespace {

template <typename T>
void configure(BatchPlan* p) {
  int dev = 0, sms = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // stage in shared memory every system whose matrix fits (leaving room for b and the panel
  // buffers), up to the variant's cap
  p->psld = std::max(4, (p->max_n + 3) / 4 * 4);
  int nmax = std::min(p->max_n, kMaxBatchN);
  while (nmax > 0 && smem_bytes<T>(p->variant, nmax, p->psld) > (size_t)optin) --nmax;
  const int cap = kVariants[p->variant].smem_cap;
  if (cap >= 0 && nmax > cap) nmax = cap;
  p->smem_max_n = nmax;
  p->smem = smem_bytes<T>(p->variant, nmax, p->psld);
  const int occ = std::max(1, occupancy<T>(p->variant, p->smem));
  p->grid = sms * occ;
}

// Algorithmic work of one batch: sum n^3/3 + 2 n^2 flops; bytes: read A-lower + b, write L + x.
void batch_work(const BatchPlan* p, double* fl, double* by) {
  *fl = 0;
  *by = 0;
  for (int v : p->h_n) {
    *fl += (double)v * v * v / 3.0 + 2.0 * v * v;
    *by += ((double)v * (v + 1) + 2.0 * v) * p->elem;
  }
}

template <typename T>
int run_plan(BatchPlan* p, T* a, T* b, int64_t* info, cudaStream_t s, bool prof) {
  BatchArgs<T> args{a, b, info, p->d_order, p->d_n, p->d_aoff, p->d_boff, (int)p->count, p->d_counter,
                    p->smem_max_n, p->psld};
  GB_CUDA_TRY(cudaMemsetAsync(p->d_counter, 0, sizeof(int), s));
  static const std::string kname = std::string("batched_posv_") + tname<T>();
  double fl = 0, by = 0;
  if (prof) batch_work(p, &fl, &by);
  ProfScope ps(prof ? kname.c_str() : nullptr, s, fl, by);
  return launch_batched<T>(p->variant, args, p->grid, p->smem, s);
}

}  // namespace

int batch_plan_create(int64_t count, const int64_t* n, int elem, BatchPlan** out) {
  if (count < 0) return -1;
  if (!n && count > 0) return -2;
  if (elem != 4 && elem != 8) return -3;
  if (!out) return -4;
  for (int64_t s = 0; s < count; ++s)
    if (n[s] < 0 || n[s] > kMaxBatchN) return -2;
  int rc = ensure_device();
  if (rc) return rc;
  BatchPlan* p = new BatchPlan();
  p->count = count;
  p->elem = elem;
  p->h_n.resize(count);
  p->h_aoff.resize(count);
  p->h_boff.resize(count);
  int64_t ao = 0, bo = 0;
  for (int64_t s = 0; s < count; ++s) {
    p->h_n[s] = (int)n[s];
    p->h_aoff[s] = ao;
    p->h_boff[s] = bo;
    ao += n[s] * n[s];
    bo += n[s];
    p->max_n = std::max(p->max_n, (int)n[s]);
  }
  p->a_elems = ao;
  p->b_elems = bo;
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return p->h_n[x] > p->h_n[y]; });
  cudaGetDevice(&p->device);
  const size_t bytes = (size_t)count * (4 + 4 + 8 + 8) + 256 * 4;
  if (dev_malloc((void**)&p->dev, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return GBLLT_ERR_ALLOC;
  }
  char* base = (char*)p->dev;
  p->d_aoff = (int64_t*)base;
  p->d_boff = p->d_aoff + count;
  p->d_order = (int*)(p->d_boff + count);
  p->d_n = p->d_order + count;
  p->d_counter = (int*)(((uintptr_t)(p->d_n + count) + 255) & ~(uintptr_t)255);
  cudaMemcpy(p->d_aoff, p->h_aoff.data(), count * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(p->d_boff, p->h_boff.data(), count * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(p->d_order, order.data(), count * 4, cudaMemcpyHostToDevice);
  if (cudaMemcpy(p->d_n, p->h_n.data(), count * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(p->dev);
    delete p;
    return GBLLT_ERR_CUDA;
  }
  if (elem == 8) configure<double>(p);
  else configure<float>(p);
  *out = p;
  return GBLLT_SUCCESS;
}

void batch_plan_destroy(BatchPlan* p) {
  if (!p) return;
  batch_plan_destroy(p->f32);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->dev) cudaFree(p->dev);
  delete p;
}

// Autotuner: times every kernel variant on synthetic SPD systems of the plan's sizes (3 runs
// each, CUDA events) and keeps the fastest.  Returns the chosen variant.
int batch_plan_tune(BatchPlan* p, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(p->mu);
  const size_t es = p->elem;
  void* buf = nullptr;
  const size_t bytes = (size_t)p->a_elems * es + (size_t)p->b_elems * es + (size_t)p->count * 8 + 512;
  if (dev_malloc((void**)&buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    return GBLLT_ERR_ALLOC;
  }
  char* a = (char*)buf;
  char* b = a + (((size_t)p->a_elems * es + 255) & ~(size_t)255);
  int64_t* info = (int64_t*)(b + (((size_t)p->b_elems * es + 255) & ~(size_t)255));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = p->variant;
  double best_ms = 1e30;
  int rc = GBLLT_SUCCESS;
  for (int v = 0; v < kNumVariants && !rc; ++v) {
    p->variant = v;
    if (p->elem == 8) configure<double>(p);
    else configure<float>(p);
    double tot = 0;
    for (int r = 0; r < 4 && !rc; ++r) {
      if (p->elem == 8) fill_tuning_kernel<double><<<(unsigned)std::max<int64_t>(p->count, 1), 256, 0, s>>>(
          (double*)a, (double*)b, p->d_n, p->d_aoff, p->d_boff, (int)p->count);
      else fill_tuning_kernel<float><<<(unsigned)std::max<int64_t>(p->count, 1), 256, 0, s>>>(
          (float*)a, (float*)b, p->d_n, p->d_aoff, p->d_boff, (int)p->count);
      cudaEventRecord(e0, s);
      rc = p->elem == 8 ? run_plan<double>(p, (double*)a, (double*)b, info, s, false)
                        : run_plan<float>(p, (float*)a, (float*)b, info, s, false);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0) tot += ms;  // first run warms up
    }
    p->tuned_ms[v] = tot / 3;
    if (tot / 3 < best_ms) {
      best_ms = tot / 3;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (rc) return rc;
  p->variant = best;
  if (p->elem == 8) configure<double>(p);
  else configure<float>(p);
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return best;
}

int batch_plan_set_variant(BatchPlan* p, int v) {
  if (v < 0 || v >= kNumVariants) return -2;
  std::lock_guard<std::mutex> lk(p->mu);
  p->variant = v;
  if (p->elem == 8) configure<double>(p);
  else configure<float>(p);
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return GBLLT_SUCCESS;
}

// Launch through a CUDA graph (memset of the queue ticket + the persistent kernel), captured once
// per (plan, buffers) on a private stream and replayed on the caller's stream.
template <typename T>
int batch_run(BatchPlan* p, T* a, T* b, int64_t* info, bool use_graph, cudaStream_t s) {
  if ((int)sizeof(T) != p->elem) return -1;
  if (p->count == 0) return GBLLT_SUCCESS;
  std::lock_guard<std::mutex> lk(p->mu);
  if (!use_graph) return run_plan<T>(p, a, b, info, s, true);
  if (!p->exec || p->g_a != a || p->g_b != b || p->g_info != info) {
    if (p->exec) {
      cudaGraphExecDestroy(p->exec);
      p->exec = nullptr;
    }
    cudaStream_t cs;
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    GB_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    int rc = run_plan<T>(p, a, b, info, cs, false);
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    GB_CUDA_TRY(e);
    e = cudaGraphInstantiate(&p->exec, g, 0);
    cudaGraphDestroy(g);
    GB_CUDA_TRY(e);
    p->g_a = a;
    p->g_b = b;
    p->g_info = info;
  }
  static const std::string kname = std::string("batched_posv_") + tname<T>();
  double fl = 0, by = 0;
  batch_work(p, &fl, &by);
  ProfScope ps(kname.c_str(), s, fl, by);
  GB_CUDA_TRY(cudaGraphLaunch(p->exec, s));
  return GBLLT_SUCCESS;
}

template int batch_run<double>(BatchPlan*, double*, double*, int64_t*, bool, cudaStream_t);
template int batch_run<float>(BatchPlan*, float*, float*, int64_t*, bool, cudaStream_t);

// ---- batched mixed precision: FP32 factorisation, FP64 refinement --------------------------------
//
// Each FP64 system is rounded to FP32 and factored, with its first solve, by the FP32 batched kernel
// (dsposv's scheme per system, as gbllt_dposv_mixed_dev does for one large system).  The refinement
// then runs one launch per step for the whole batch, CTAs pulling systems from the largest-first
// queue: r = b - A x in FP64 from A's lower triangle, the normwise backward error
// ||r||_F / (||A||_F ||x||_F) against tol, and while it is above, x += L^{-T} L^{-1} r with the FP32
// factor (r scaled by its largest entry before the rounding).  A system leaves the queue's work once
// it converged, its FP32 factorisation failed, or the last step checked it.

namespace {

enum : int { kMxActive = 0, kMxDone = 1, kMxFailed = 2, kMxStalled = 3 };

// The lower triangle of every system rounded to FP32 (same packed layout), and b; also ||A||_F^2 of
// each system from the rounded entries (the backward-error test needs it to a few digits only, and
// FP32 keeps it off the FP64 pipe).  A warp per column.
__global__ void __launch_bounds__(256) round_lower_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                          float* __restrict__ af, float* __restrict__ bf,
                                                          double* __restrict__ anorm2, const int* __restrict__ nv,
                                                          const int64_t* __restrict__ aoff,
                                                          const int64_t* __restrict__ boff, int count) {
  __shared__ float red[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int s = blockIdx.x; s < count; s += gridDim.x) {
    const int n = nv[s];
    const double* A = a + aoff[s];
    float* F = af + aoff[s];
    float q = 0.f;
    for (int j = warp; j < n; j += 8)
      for (int i = j + lane; i < n; i += 32) {
        const float v = (float)A[(long long)j * n + i];
        F[(long long)j * n + i] = v;
        q = fmaf(i == j ? v : 2.f * v, v, q);
      }
    for (int i = threadIdx.x; i < n; i += 256) bf[boff[s] + i] = (float)b[boff[s] + i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) q += __shfl_down_sync(0xffffffffu, q, off);
    if (lane == 0) red[warp] = q;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int w = 0; w < 8; ++w) t += red[w];
      anorm2[s] = (double)t;
    }
    __syncthreads();
  }
}

struct RefineArgs {
  const double* a;       // FP64 systems (lower triangles read)
  const double* b;
  double* x;             // iterates, laid out like b
  const float* lf;       // FP32 factors (lower), laid out like a
  const float* xf;       // FP32 first solutions, laid out like b
  const int64_t* info32; // FP32 factorisation info
  int64_t* info;
  int* state;            // kMx* per system
  const double* anorm2;  // ||A||_F^2 per system
  const int* order;
  const int* n;
  const int64_t* aoff;
  const int64_t* boff;
  int count;
  float* rsc;            // residuals scaled by their largest entry, FP32, laid out like b
  double* rmax;          // that scale per system
  int* counter;          // queue ticket of the residual launch, zeroed before each step
  int* counter2;         // queue ticket of the correction launch, zeroed before each step
  int* active;           // systems left for a correction by this step
  int* done;             // systems converged so far
  unsigned long long* maxbe;  // the largest backward error at the systems' last checks (bit pattern)
  int step, last;
  double tol;
};

constexpr int kRefRows = 64;   // rows of a staged tile of A (one per thread)
constexpr int kTileLd = 33;    // its row pitch in doubles (odd: column reads across rows avoid bank conflicts)

template <int THREADS>
__global__ void __launch_bounds__(THREADS) refine_batch_kernel(RefineArgs p) {
  constexpr int NW = THREADS / 32;
  static_assert(THREADS == kRefRows, "one thread per row of a staged tile");
  __shared__ double xs[kMaxBatchN];
  __shared__ double rs[kMaxBatchN];
  __shared__ double tile[kRefRows * kTileLd];
  __shared__ double part[NW][32];
  __shared__ double red[3][NW];
  __shared__ int s_ticket;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (;;) {
    if (tid == 0) s_ticket = atomicAdd(p.counter, 1);
    __syncthreads();
    const int t = s_ticket;
    __syncthreads();
    if (t >= p.count) break;
    const int sys = p.order[t];
    const int n = p.n[sys];
    int st = p.state[sys];
    if (p.step == 0) {
      st = p.info32[sys] != 0 ? kMxFailed : kMxActive;
      if (tid == 0) {
        p.state[sys] = st;
        if (st == kMxFailed) p.info[sys] = p.info32[sys];
      }
    }
    if (st != kMxActive) continue;  // uniform over the CTA
    const double* A = p.a + p.aoff[sys];
    const double* B = p.b + p.boff[sys];
    double* X = p.x + p.boff[sys];
    for (int i = tid; i < n; i += THREADS) {
      xs[i] = p.step == 0 ? (double)p.xf[p.boff[sys] + i] : X[i];
      rs[i] = B[i];
    }
    __syncthreads();
    // r = b - A x with A's lower triangle read once per step, coalesced: the triangle goes through
    // shared memory in tiles of kRefRows rows x 32 columns (column by column, kRefRows consecutive
    // doubles each).  From a tile at rows R0.., columns J0..: thread t adds row R0 + t's products with
    // x(J0..) to r (its own row), and lane c of warp w the products of column J0 + c over the warp's
    // rows with x(R0..) to a partial sum of r(J0 + c) (its own column): every FP64 instruction with all
    // lanes busy, no shuffles; the warps' partials are added once per tile.
    for (int J0 = 0; J0 < n; J0 += 32) {
      const int jb = n - J0 < 32 ? n - J0 : 32;
      for (int R0 = J0; R0 < n; R0 += kRefRows) {
        const int rb = n - R0 < kRefRows ? n - R0 : kRefRows;
        for (int c = 0; c < jb; ++c)
          for (int r = tid; r < rb; r += THREADS) tile[r * kTileLd + c] = A[(long long)(J0 + c) * n + R0 + r];
        __syncthreads();
        {  // rows: r(i) -= sum_{j <= i} A(i, j) x(j) over this tile's columns
          const int r = tid;
          if (r < rb) {
            const int i = R0 + r;
            double acc = 0.0;
#pragma unroll 8
            for (int c = 0; c < 32; ++c)
              if (c < jb && J0 + c <= i) acc = fma(tile[r * kTileLd + c], xs[J0 + c], acc);
            rs[i] -= acc;
          }
        }
        {  // columns: r(j) -= sum_{i > j} A(i, j) x(i), lane = column, this warp's rows
          double acc = 0.0;
          const int j = J0 + lane;
#pragma unroll 8
          for (int rr = 0; rr < kRefRows / NW; ++rr) {
            const int r = warp * (kRefRows / NW) + rr;
            if (r < rb && lane < jb && R0 + r > j) acc = fma(tile[r * kTileLd + lane], xs[R0 + r], acc);
          }
          part[warp][lane] = acc;
        }
        __syncthreads();
        if (tid < jb) {
          double sum = 0.0;
#pragma unroll
          for (int w = 0; w < NW; ++w) sum += part[w][tid];
          rs[J0 + tid] -= sum;
        }
        __syncthreads();
      }
    }
    double rr = 0.0, xx = 0.0, rm = 0.0;
    for (int i = tid; i < n; i += THREADS) {
      rr = fma(rs[i], rs[i], rr);
      xx = fma(xs[i], xs[i], xx);
      rm = fmax(rm, fabs(rs[i]));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      rr += __shfl_down_sync(0xffffffffu, rr, off);
      xx += __shfl_down_sync(0xffffffffu, xx, off);
      rm = fmax(rm, __shfl_down_sync(0xffffffffu, rm, off));
    }
    if (lane == 0) {
      red[0][warp] = rr;
      red[1][warp] = xx;
      red[2][warp] = rm;
    }
    __syncthreads();
    rr = xx = rm = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      rr += red[0][w];
      xx += red[1][w];
      rm = fmax(rm, red[2][w]);
    }
    const double a2 = p.anorm2[sys];
    const double be = rr == 0.0 ? 0.0 : sqrt(rr) / (sqrt(a2) * sqrt(xx));
    const bool ok = be <= p.tol;  // false for NaN
    if (p.step == 0)
      for (int i = tid; i < n; i += THREADS) X[i] = xs[i];
    if (ok || p.step == p.last) {
      if (tid == 0) {
        p.state[sys] = ok ? kMxDone : kMxStalled;
        p.info[sys] = ok ? 0 : GBLLT_BATCH_NOT_CONVERGED;
        if (ok) atomicAdd(p.done, 1);
        atomicMax(p.maxbe, (unsigned long long)__double_as_longlong(be));
      }
      __syncthreads();  // xs, rs are reused by the next system
      continue;
    }
    // left for the correction launch: r scaled by its largest entry, rounded to FP32
    const double rinv = 1.0 / rm;
    for (int i = tid; i < n; i += THREADS) p.rsc[p.boff[sys] + i] = (float)(rs[i] * rinv);
    if (tid == 0) {
      p.rmax[sys] = rm;
      atomicAdd(p.active, 1);
    }
    __syncthreads();
  }
}

// The correction of every system the residual launch left active: x += L^{-T} L^{-1} r with the FP32
// factor (the solve's 32-row blocks want more threads than the residual's tiles).
template <int THREADS>
__global__ void __launch_bounds__(THREADS) correct_batch_kernel(RefineArgs p) {
  __shared__ __align__(16) float rf[kMaxBatchN];
  __shared__ __align__(16) float Dg[32 * kDgLd];
  __shared__ int s_ticket;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_ticket = atomicAdd(p.counter2, 1);
    __syncthreads();
    const int t = s_ticket;
    __syncthreads();
    if (t >= p.count) break;
    const int sys = p.order[t];
    if (p.state[sys] != kMxActive) continue;  // uniform over the CTA
    const int n = p.n[sys];
    double* X = p.x + p.boff[sys];
    for (int i = tid; i < n; i += THREADS) rf[i] = p.rsc[p.boff[sys] + i];
    __syncthreads();
    solve_sweeps<float, THREADS>(p.lf + p.aoff[sys], n, n, rf, Dg);
    const double rm = p.rmax[sys];
    for (int i = tid; i < n; i += THREADS) X[i] = fma(rm, (double)rf[i], X[i]);
    __syncthreads();
  }
}

// Systems left to the FP64 fallback (FP32 factorisation failed or tol not reached).
__global__ void list_unsolved_kernel(const int* __restrict__ state, int count, int* __restrict__ list,
                                     int* __restrict__ nlist) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x)
    if (state[s] == kMxFailed || state[s] == kMxStalled) list[atomicAdd(nlist, 1)] = s;
}

// Copy system list[k] (A and b) of a packed batch to system k of another.  A CTA per system.
__global__ void __launch_bounds__(256) gather_systems_kernel(const int* __restrict__ list, int nlist,
                                                             const int* __restrict__ nv,
                                                             const int64_t* __restrict__ aoff,
                                                             const int64_t* __restrict__ boff, const double* __restrict__ a,
                                                             const double* __restrict__ b, const int64_t* __restrict__ aoff2,
                                                             const int64_t* __restrict__ boff2, double* __restrict__ a2,
                                                             double* __restrict__ b2) {
  for (int k = blockIdx.x; k < nlist; k += gridDim.x) {
    const int s = list[k], n = nv[s];
    for (long long e = threadIdx.x; e < (long long)n * n; e += 256) a2[aoff2[k] + e] = a[aoff[s] + e];
    for (int i = threadIdx.x; i < n; i += 256) b2[boff2[k] + i] = b[boff[s] + i];
  }
}

// The other way: the solution and info of system k of the small batch to system list[k] of the large
// one (the solution only where that system's factorisation succeeded).
__global__ void __launch_bounds__(256) scatter_solutions_kernel(const int* __restrict__ list, int nlist,
                                                                const int* __restrict__ nv,
                                                                const int64_t* __restrict__ boff,
                                                                const int64_t* __restrict__ boff2,
                                                                const double* __restrict__ x2,
                                                                const int64_t* __restrict__ info2,
                                                                double* __restrict__ x, int64_t* __restrict__ info) {
  for (int k = blockIdx.x; k < nlist; k += gridDim.x) {
    const int s = list[k], n = nv[s];
    if (info2[k] == 0)
      for (int i = threadIdx.x; i < n; i += 256) x[boff[s] + i] = x2[boff2[k] + i];
    if (threadIdx.x == 0) info[s] = info2[k];
  }
}

constexpr int kRefineThreads = kRefRows;
constexpr int kCorrectThreads = 128;

}  // namespace

int batch_posv_mixed(BatchPlan* p, const double* a, const double* b, double* x, int64_t* info,
                     const gbllt_mixed_opts& o, gbllt_batch_mixed_report* rep, cudaStream_t s) {
  gbllt_batch_mixed_report r;
  memset(&r, 0, sizeof r);
  if (rep) *rep = r;
  if (p->count == 0) return GBLLT_SUCCESS;
  const int count = (int)p->count;
  // the FP32 plan of the same sizes, tuned once
  {
    std::lock_guard<std::mutex> lk(p->mu);
    if (!p->f32) {
      std::vector<int64_t> sizes(p->h_n.begin(), p->h_n.end());
      BatchPlan* f = nullptr;
      int rc = batch_plan_create(p->count, sizes.data(), 4, &f);
      if (rc) return rc;
      if ((rc = batch_plan_tune(f, s)) < 0) {
        batch_plan_destroy(f);
        return rc;
      }
      p->f32 = f;
    }
  }
  BatchPlan* f = p->f32;
  // workspace: FP32 factors and first solutions, per-system state, counters
  auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t o_af = 0, o_bf = o_af + up((size_t)p->a_elems * 4), o_i32 = o_bf + up((size_t)p->b_elems * 4),
               o_st = o_i32 + up((size_t)count * 8), o_an = o_st + up((size_t)count * 4),
               o_list = o_an + up((size_t)count * 8), o_rsc = o_list + up((size_t)count * 4),
               o_rm = o_rsc + up((size_t)p->b_elems * 4), o_cnt = o_rm + up((size_t)count * 8), total = o_cnt + 256;
  char* ws = nullptr;
  if (dev_malloc_async((void**)&ws, total, s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("gbllt_batch_dposv_mixed_dev: allocation of the workspace failed");
    return GBLLT_ERR_ALLOC;
  }
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } ws_free{ws, s};
  float* af = (float*)(ws + o_af);
  float* bf = (float*)(ws + o_bf);
  int64_t* info32 = (int64_t*)(ws + o_i32);
  int* state = (int*)(ws + o_st);
  double* anorm2 = (double*)(ws + o_an);
  int* list = (int*)(ws + o_list);
  float* rsc = (float*)(ws + o_rsc);
  double* rmax = (double*)(ws + o_rm);
  // [0] residual ticket, [1] active, [2] correction ticket, [3] done, [4] unsolved; [6..7] max backward error
  int* cnt = (int*)(ws + o_cnt);
  unsigned long long* maxbe = (unsigned long long*)(cnt + 6);
  GB_CUDA_TRY(cudaMemsetAsync(cnt, 0, 64, s));
  {
    static const std::string kr = "batched_round_f32";
    double by = 0;
    for (int v : p->h_n) by += (double)v * (v + 1) / 2.0 * 12.0 + (double)v * 12.0;
    ProfScope ps(kr.c_str(), s, 0.0, by);
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    round_lower_kernel<<<(unsigned)std::max(1, std::min(count, 8 * std::max(sms, 1))), 256, 0, s>>>(
        a, b, af, bf, anorm2, p->d_n, p->d_aoff, p->d_boff, count);
    GB_CUDA_TRY(cudaGetLastError());
  }
  {
    std::lock_guard<std::mutex> lk(f->mu);
    int rc = run_plan<float>(f, af, bf, info32, s, true);
    if (rc) return rc;
  }
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)std::max(1, std::min(count, 8 * std::max(sms, 1)));
  RefineArgs ra{a,     b,          x,      af,        bf,        info32, info,    state,   anorm2,
                p->d_order, p->d_n, p->d_aoff, p->d_boff, count, rsc, rmax, cnt, cnt + 2, cnt + 1,
                cnt + 3, maxbe, 0,      o.max_steps, o.tol};
  static const std::string kf = "batched_refine_f64";
  double fl = 0, by = 0;
  for (int v : p->h_n) {
    fl += 2.0 * v * v;  // the FP64 residual
    by += (double)v * (v + 1) / 2.0 * 8.0 + (double)v * 28.0;
  }
  static const std::string kc = "batched_correct_f32";
  double flc = 0, byc = 0;
  for (int v : p->h_n) {
    flc += 2.0 * v * v;
    byc += (double)v * (v + 1) / 2.0 * 4.0 + (double)v * 20.0;
  }
  for (int step = 0; step <= o.max_steps; ++step) {
    ra.step = step;
    GB_CUDA_TRY(cudaMemsetAsync(cnt, 0, 12, s));  // the two tickets and the active count
    {
      ProfScope ps(kf.c_str(), s, fl, by);
      refine_batch_kernel<kRefineThreads><<<grid, kRefineThreads, 0, s>>>(ra);
      GB_CUDA_TRY(cudaGetLastError());
    }
    {
      ProfScope ps(kc.c_str(), s, flc, byc);
      correct_batch_kernel<kCorrectThreads><<<grid, kCorrectThreads, 0, s>>>(ra);
      GB_CUDA_TRY(cudaGetLastError());
    }
    int act = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&act, cnt + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (act == 0) break;
    r.steps = step + 1;
  }
  int host_cnt[5] = {0, 0, 0, 0, 0};
  unsigned long long hbe = 0;
  // the systems left to the FP64 fallback
  list_unsolved_kernel<<<(unsigned)std::max(1, std::min((count + 255) / 256, 1024)), 256, 0, s>>>(state, count, list,
                                                                                                   cnt + 4);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpyAsync(host_cnt, cnt, 20, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&hbe, maxbe, 8, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  r.converged = host_cnt[3];
  double mbe = 0;
  memcpy(&mbe, &hbe, 8);
  r.max_backward_error = mbe;
  const int nf = host_cnt[4];
  if (nf > 0 && o.fallback_fp64) {
    // the unsolved systems, in index order, as a batch of their own solved by the FP64 kernel
    std::vector<int> h_list(nf);
    GB_CUDA_TRY(cudaMemcpy(h_list.data(), list, (size_t)nf * 4, cudaMemcpyDeviceToHost));
    std::sort(h_list.begin(), h_list.end());
    GB_CUDA_TRY(cudaMemcpyAsync(list, h_list.data(), (size_t)nf * 4, cudaMemcpyHostToDevice, s));
    std::vector<int64_t> sizes(nf);
    for (int k = 0; k < nf; ++k) sizes[k] = p->h_n[h_list[k]];
    BatchPlan* t = nullptr;
    int rc = batch_plan_create(nf, sizes.data(), 8, &t);
    if (rc) return rc;
    struct PlanFree {
      BatchPlan* t;
      ~PlanFree() { batch_plan_destroy(t); }
    } t_free{t};
    t->variant = p->variant;
    configure<double>(t);
    char* tw = nullptr;
    const size_t ta = up((size_t)t->a_elems * 8), tb = up((size_t)t->b_elems * 8);
    if (dev_malloc_async((void**)&tw, ta + tb + (size_t)nf * 8, s) != cudaSuccess) {
      cudaGetLastError();
      set_error_message("gbllt_batch_dposv_mixed_dev: allocation of the fallback's workspace failed");
      return GBLLT_ERR_ALLOC;
    }
    struct Free2 {
      void* p;
      cudaStream_t s;
      ~Free2() { cudaFreeAsync(p, s); }
    } tw_free{tw, s};
    double* ta_p = (double*)tw;
    double* tb_p = (double*)(tw + ta);
    int64_t* tinfo = (int64_t*)(tw + ta + tb);
    const unsigned g2 = (unsigned)std::min(nf, 4096);
    gather_systems_kernel<<<g2, 256, 0, s>>>(list, nf, p->d_n, p->d_aoff, p->d_boff, a, b, t->d_aoff, t->d_boff, ta_p,
                                             tb_p);
    GB_CUDA_TRY(cudaGetLastError());
    if ((rc = run_plan<double>(t, ta_p, tb_p, tinfo, s, true))) return rc;
    scatter_solutions_kernel<<<g2, 256, 0, s>>>(list, nf, p->d_n, p->d_boff, t->d_boff, tb_p, tinfo, x, info);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    r.fallback = nf;
  }
  if (rep) *rep = r;
  return GBLLT_SUCCESS;
}

}  // namespace gbllt

// ---- tuning cache: a JSON object, one entry per line, keyed by dtype, count and a hash of the sizes
namespace gbllt {
namespace {

std::string plan_signature(const BatchPlan* p) {
  uint64_t h = 1469598103934665603ull;  // FNV-1a over the sizes
  for (int v : p->h_n) {
    h ^= (uint64_t)(uint32_t)v;
    h *= 1099511628211ull;
  }
  char buf[96];
  snprintf(buf, sizeof buf, "%s-%lld-%016llx", p->elem == 8 ? "f64" : "f32", (long long)p->count,
           (unsigned long long)h);
  return buf;
}

std::vector<std::pair<std::string, std::string>> read_cache(const char* path) {
  std::vector<std::pair<std::string, std::string>> entries;
  FILE* f = fopen(path, "r");
  if (!f) return entries;
  char line[1024];
  while (fgets(line, sizeof line, f)) {
    const char* q0 = strchr(line, '"');
    if (!q0) continue;
    const char* q1 = strchr(q0 + 1, '"');
    const char* br = q1 ? strchr(q1, '{') : nullptr;
    const char* be = br ? strrchr(br, '}') : nullptr;
    if (!q1 || !br || !be) continue;
    entries.emplace_back(std::string(q0 + 1, q1), std::string(br, be + 1));
  }
  fclose(f);
  return entries;
}

int cached_variant(const char* path, const std::string& sig) {
  for (auto& e : read_cache(path))
    if (e.first == sig) {
      const char* v = strstr(e.second.c_str(), "\"variant\":");
      if (v) return atoi(v + 10);
    }
  return -1;
}

void write_cache(const char* path, const std::string& sig, const BatchPlan* p) {
  auto entries = read_cache(path);
  std::string body = "{\"variant\": " + std::to_string(p->variant) +
                     ", \"algo\": " + std::to_string(kVariants[p->variant].algo) +
                     ", \"panel\": " + std::to_string(kVariants[p->variant].nbp) +
                     ", \"threads\": " + std::to_string(kVariants[p->variant].threads) +
                     ", \"smem_max_n\": " + std::to_string(p->smem_max_n) + ", \"ms\": [";
  for (int v = 0; v < kNumVariants; ++v) {
    char num[32];
    snprintf(num, sizeof num, "%s%.4f", v ? ", " : "", p->tuned_ms[v]);
    body += num;
  }
  body += "]}";
  bool found = false;
  for (auto& e : entries)
    if (e.first == sig) {
      e.second = body;
      found = true;
    }
  if (!found) entries.emplace_back(sig, body);
  FILE* f = fopen(path, "w");
  if (!f) return;
  fprintf(f, "{\n");
  for (size_t i = 0; i < entries.size(); ++i)
    fprintf(f, "\"%s\": %s%s\n", entries[i].first.c_str(), entries[i].second.c_str(), i + 1 < entries.size() ? "," : "");
  fprintf(f, "}\n");
  fclose(f);
}

}  // namespace
}  // namespace gbllt

using namespace gbllt;

extern "C" {

int gbllt_batch_plan_create(int64_t count, const int64_t* n, int elem_bytes, gbllt_batch_plan** plan) {
  BatchPlan* p = nullptr;
  int rc = batch_plan_create(count, n, elem_bytes, &p);
  if (rc == GBLLT_SUCCESS) *plan = (gbllt_batch_plan*)p;
  return rc;
}

int gbllt_batch_plan_destroy(gbllt_batch_plan* plan) {
  batch_plan_destroy((BatchPlan*)plan);
  return GBLLT_SUCCESS;
}

int gbllt_batch_plan_layout(const gbllt_batch_plan* plan, int64_t* aoff, int64_t* boff, int64_t* a_elems,
                            int64_t* b_elems) {
  if (!plan) return -1;
  const BatchPlan* p = (const BatchPlan*)plan;
  if (aoff) memcpy(aoff, p->h_aoff.data(), p->count * sizeof(int64_t));
  if (boff) memcpy(boff, p->h_boff.data(), p->count * sizeof(int64_t));
  if (a_elems) *a_elems = p->a_elems;
  if (b_elems) *b_elems = p->b_elems;
  return GBLLT_SUCCESS;
}

int gbllt_batch_plan_tune(gbllt_batch_plan* plan, const char* cache_path, void* stream) {
  if (!plan) return -1;
  BatchPlan* p = (BatchPlan*)plan;
  const std::string sig = plan_signature(p);
  if (cache_path) {
    const int v = cached_variant(cache_path, sig);
    if (v >= 0 && v < kNumVariants) {
      batch_plan_set_variant(p, v);
      return v;
    }
  }
  const int v = batch_plan_tune(p, (cudaStream_t)stream);
  if (v >= 0 && cache_path) write_cache(cache_path, sig, p);
  return v;
}

int gbllt_batch_plan_set_variant(gbllt_batch_plan* plan, int variant) {
  if (!plan) return -1;
  return batch_plan_set_variant((BatchPlan*)plan, variant);
}

int gbllt_batch_plan_variant(const gbllt_batch_plan* plan, int* panel, int* threads, int* smem_max_n) {
  if (!plan) return -1;
  const BatchPlan* p = (const BatchPlan*)plan;
  if (panel) *panel = kVariants[p->variant].nbp;
  if (threads) *threads = kVariants[p->variant].threads;
  if (smem_max_n) *smem_max_n = p->smem_max_n;
  return p->variant;
}

int gbllt_dposv_batched_dev(gbllt_batch_plan* plan, double* d_a, double* d_b, int64_t* d_info, void* stream) {
  if (!plan) return -1;
  if (((BatchPlan*)plan)->elem != 8) return -1;
  if (!d_a || !d_b) return -2;
  if (!d_info) return -4;
  return batch_run<double>((BatchPlan*)plan, d_a, d_b, d_info, true, (cudaStream_t)stream);
}

int gbllt_sposv_batched_dev(gbllt_batch_plan* plan, float* d_a, float* d_b, int64_t* d_info, void* stream) {
  if (!plan) return -1;
  if (((BatchPlan*)plan)->elem != 4) return -1;
  if (!d_a || !d_b) return -2;
  if (!d_info) return -4;
  return batch_run<float>((BatchPlan*)plan, d_a, d_b, d_info, true, (cudaStream_t)stream);
}

static int host_batched(gbllt_batch_plan* plan, void* a, void* b, int64_t* info, int elem) {
  if (!plan) return -1;
  BatchPlan* p = (BatchPlan*)plan;
  if (p->elem != elem) return -1;
  if ((!a || !b) && p->count > 0) return -2;
  if (!info && p->count > 0) return -4;
  if (p->count == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  cudaStream_t s = lib_stream();
  const size_t ab = (size_t)p->a_elems * elem, bb = (size_t)p->b_elems * elem, ib = (size_t)p->count * 8;
  char* d = nullptr;
  if (dev_malloc_async((void**)&d, ab + bb + ib + 512, s) != cudaSuccess) {
    cudaGetLastError();
    return GBLLT_ERR_ALLOC;
  }
  char* da = d;
  char* db = d + ((ab + 255) & ~(size_t)255);
  int64_t* di = (int64_t*)(db + ((bb + 255) & ~(size_t)255));
  cudaMemcpyAsync(da, a, ab, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(db, b, bb, cudaMemcpyHostToDevice, s);
  rc = elem == 8 ? batch_run<double>(p, (double*)da, (double*)db, di, false, s)
                 : batch_run<float>(p, (float*)da, (float*)db, di, false, s);
  if (!rc) {
    cudaMemcpyAsync(a, da, ab, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(b, db, bb, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(info, di, ib, cudaMemcpyDeviceToHost, s);
  }
  cudaFreeAsync(d, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (!rc && e != cudaSuccess) {
    set_last_error(e, "batched solve", __FILE__, __LINE__);
    return GBLLT_ERR_CUDA;
  }
  return rc;
}

int gbllt_dposv_batched(gbllt_batch_plan* plan, double* a, double* b, int64_t* info) {
  return host_batched(plan, a, b, info, 8);
}

int gbllt_sposv_batched(gbllt_batch_plan* plan, float* a, float* b, int64_t* info) {
  return host_batched(plan, a, b, info, 4);
}

int gbllt_batch_dposv_mixed_dev(gbllt_batch_plan* plan, const double* d_a, const double* d_b, double* d_x,
                                int64_t* d_info, const gbllt_mixed_opts* opts, gbllt_batch_mixed_report* report,
                                void* stream) {
  if (!plan) return -1;
  BatchPlan* p = (BatchPlan*)plan;
  if (p->elem != 8) return -1;
  if (p->count > 0 && (!d_a || !d_b)) return -2;
  if (p->count > 0 && !d_x) return -4;
  if (p->count > 0 && !d_info) return -5;
  gbllt_mixed_opts o;
  if (resolve_mixed_opts(opts, &o, 0)) return -6;
  int rc = ensure_device();
  if (rc) return rc;
  return batch_posv_mixed(p, d_a, d_b, d_x, d_info, o, report, (cudaStream_t)stream);
}

}  // extern "C"
