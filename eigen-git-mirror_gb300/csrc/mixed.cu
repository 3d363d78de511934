// Mixed-precision LLT solve with FP64 iterative refinement.
//
// Eigen's LLT<MatrixXd> (Eigen/src/Cholesky/LLT.h:430-498) factors and solves entirely in FP64.
// On GB300 the FP64 pipe delivers ~1 TFLOP/s while the tensor cores deliver ~1 PFLOP/s (TF32) and
// ~2 PFLOP/s (BF16), so this path:
//   1. scales A symmetrically by powers of two (D A D, D = 2^-floor(e_i / 2) for a_ii = f 2^e_i, so the
//      diagonal lies in [0.5, 2): exact scaling, as LAPACK's xPOEQUB) and rounds the scaled lower
//      triangle to an FP32 working matrix;
//   2. factors it with the blocked right-looking algorithm of llt_inplace::blocked (LLT.h:338-368)
//      in two levels: panels of width `panel` are factored in 64-column steps (the diagonal block and
//      its inverse in FP32 by one CTA, the panel solve as the product with that inverse on the tensor
//      cores, its result split into tensor-core operands for the in-panel update on tcgen05), and the
//      trailing SYRK of each panel
//      -- almost all of the n^3/3 flops -- runs on tcgen05 tensor cores in TF32 or BF16 (optionally
//      as split-precision products) with FP32 accumulation, one panel ahead on a second stream;
//   3. refines in FP64: r = b - A x (reading only the stored triangle of A; on the FP64 pipe, or for
//      four or more right-hand sides on the tensor cores with FP64-exact error-free slicing,
//      ozaki.cu), solve with the FP32 factor, x += d, until ||r||_F / (||A||_F ||x||_F) <= tol
//      (LAPACK dsposv-style refinement, with the FP64 GPU factorisation as fallback).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "tc_gemm.h"

namespace gbllt {

namespace {

constexpr int TS = 32;  // conversion tile

// x rounded to the nearest float, ties to even (IEEE 754), in integer arithmetic on x's bits where
// the result is a normal float; zeros, subnormal results, overflow beyond the rounding and
// non-finite values take the hardware conversion.  On GB300 the FP64-to-FP32 conversion runs on the
// narrow FP64 pipe: the working copy's conversion was bound by it (84 % busy, DRAM 22 %).
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7FF) - 1023 + 127;  // the float's biased exponent
  if (ef >= 1 && ef <= 254) {
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;  // 52 fraction bits
    const unsigned int keep = (unsigned int)(m >> 29);    // the top 23
    const unsigned int rest = (unsigned int)(m & 0x1FFFFFFFu);
    const unsigned int up = (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) ? 1u : 0u;
    // a carry out of the fraction raises the exponent (254 + 1 = infinity, as rounding requires)
    const unsigned int bits = (((unsigned int)ef << 23) | keep) + up;
    return __uint_as_float(bits | ((unsigned int)(b >> 32) & 0x80000000u));
  }
  return __double2float_rn(x);
}

// v * 2^p rounded to float: an exponent add on v's bits where v and the product are normal doubles
// (exact), else ldexp; then f64_to_f32_rn.  Neither step uses the FP64 pipe on the common path.
__device__ __forceinline__ float scale_pow2_to_f32(double v, int p) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e > 0 && e < 0x7FF && e + p > 0 && e + p < 0x7FF) return f64_to_f32_rn(__longlong_as_double(b + ((long long)p << 52)));
  return f64_to_f32_rn(ldexp(v, p));
}

// The exponent p of a scale d = 2^p (a normal power of two).
__device__ __forceinline__ int pow2_exponent(double d) { return (int)((__double_as_longlong(d) >> 52) & 0x7FF) - 1023; }

// Af(i, j) = d_i * A(i, j) * d_j for i >= j, as float (d powers of two: exact scaling, one rounding),
// A given by its upper triangle: element (i, j), i >= j, lives at a[i * lda + j], so each 32 x 32 tile
// is transposed through shared memory.
__global__ void __launch_bounds__(256) convert_scaled_upper_kernel(const double* __restrict__ a, long long lda,
                                                                   long long n, const double* __restrict__ d,
                                                                   float* __restrict__ af, long long ldf) {
  __shared__ double t[TS][TS + 1];
  int ti, tj;
  lower_tile_coords(blockIdx.x, ti, tj);
  const long long i0 = (long long)ti * TS, j0 = (long long)tj * TS;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int c = ty; c < TS; c += 8) {
    const long long col = i0 + c, row = j0 + tx;  // a[col * lda + row] = A(row, col) = A(col, row)
    if (col < n && row < n && col >= row) t[c][tx] = a[col * lda + row];
  }
  __syncthreads();
  for (int c = ty; c < TS; c += 8) {
    const long long i = i0 + tx, j = j0 + c;
    if (i < n && j < n && i >= j) af[j * ldf + i] = scale_pow2_to_f32(t[tx][c], pow2_exponent(d[i]) + pow2_exponent(d[j]));
  }
}

// The same conversion for a lower-stored A, a column at a time: CTA b takes columns b, b + gridDim.x,
// ... and its threads stream down each column from the diagonal (coalesced reads and writes, four
// rows per thread in flight).  One CTA per 32 x 32 tile, as above, spent more time starting tiles
// than moving bytes (about 1 TB/s at n = 32768); the product is the same, so is the result.

// Self-test of f64_to_f32_rn: out[i] = f64_to_f32_rn(in[i]) and ref[i] = the hardware conversion.
__global__ void f64_to_f32_selftest_kernel(const double* __restrict__ in, float* __restrict__ out,
                                           float* __restrict__ ref, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[i] = f64_to_f32_rn(in[i]);
    ref[i] = __double2float_rn(in[i]);
  }
}
__global__ void __launch_bounds__(256) convert_scaled_lower_kernel(const double* __restrict__ a, long long lda,
                                                                   long long n, const double* __restrict__ d,
                                                                   float* __restrict__ af, long long ldf) {
  for (long long j = blockIdx.x; j < n; j += gridDim.x) {
    const int pj = pow2_exponent(d[j]);
    const double* col = a + j * lda;
    float* out = af + j * ldf;
    long long i = j + threadIdx.x;
    for (; i + 3 * 256 < n; i += 4 * 256) {
      double v[4], di[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        v[u] = col[i + u * 256];
        di[u] = d[i + u * 256];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) out[i + u * 256] = scale_pow2_to_f32(v[u], pow2_exponent(di[u]) + pj);
    }
    for (; i < n; i += 256) out[i] = scale_pow2_to_f32(col[i], pow2_exponent(d[i]) + pj);
  }
}

template <bool UP>
__global__ void diag_scale_kernel(const double* __restrict__ a, long long lda, long long n, double* __restrict__ d) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    // d_i = 2^-floor(e / 2) for a_ii = f 2^e, f in [0.5, 1): d_i^2 a_ii in [0.5, 2) (the power-of-two
    // equilibration of LAPACK's xPOEQUB; the refinement converged in the same steps as with
    // 1 / sqrt(a_ii), and the scaling of A, R and X is exact)
    const double v = a[i * lda + i];
    int e = 0;
    if (v > 0.0) frexp(v, &e);
    d[i] = v > 0.0 ? ldexp(1.0, -(e >> 1)) : 1.0;
  }
}

// Tensor-core operands are K-major copies of panel values split into NP successive roundings:
// part0 = round(v), part1 = round(v - part0), part2 = round(v - part0 - part1).  KIND 0 = bf16,
// 1 = tf32 (to_tf32).

// K-major copies of the block Af(r0 .. r0+rows, c0 .. c0+bs) in NP parts, stored at
// out[k][r * ldk + p] for p < bs (zero for bs <= p < ldk).
template <int KIND>
__global__ void __launch_bounds__(256) split_panel_kernel(const float* __restrict__ af, long long ldf, long long r0,
                                                          long long c0, long long rows, int bs, int np,
                                                          void* __restrict__ p0, void* __restrict__ p1,
                                                          void* __restrict__ p2, long long ldk) {
  __shared__ float t[TS][TS + 1];
  const long long rb = (long long)blockIdx.x * TS;
  const int pb = blockIdx.y * TS;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int c = ty; c < TS; c += 8) {  // read along rows (contiguous)
    const long long r = rb + tx;
    const int p = pb + c;
    t[c][tx] = (r < rows && p < bs) ? af[(c0 + p) * ldf + r0 + r] : 0.f;
  }
  __syncthreads();
  void* outs[3] = {p0, p1, p2};
  for (int c = ty; c < TS; c += 8) {  // write along p (contiguous)
    const long long r = rb + c;
    const int p = pb + tx;
    if (r < rows && p < (int)ldk) {
      float v = p < bs ? t[tx][c] : 0.f;
      for (int k = 0; k < np; ++k) {
        if (KIND == 0) {
          const __nv_bfloat16 h = __float2bfloat16_rn(v);
          ((__nv_bfloat16*)outs[k])[r * ldk + p] = h;
          v -= __bfloat162float(h);
        } else {
          const float h = to_tf32(v);
          ((float*)outs[k])[r * ldk + p] = h;
          v -= h;
        }
      }
    }
  }
}

// ---- FP64 residual  R = B - A X  (A symmetric, only the `UP` triangle read) ---------------------

constexpr int RB = 64;   // row block
constexpr int RCH = 16;  // right-hand sides per CTA

template <bool UP>
__device__ __forceinline__ bool stored(long long i, long long j) {
  return UP ? (i <= j) : (i >= j);
}

template <bool UP, int NR>
__global__ void __launch_bounds__(256) symm_partial_kernel(const double* __restrict__ a, long long lda, long long n,
                                                           const double* __restrict__ x, long long ldx, long long nrhs,
                                                           int jpc, double* __restrict__ part) {
  // NR = 16: 4 thread groups x 4 right-hand sides each, every thread sums the full tile depth.
  // NR = 1: one right-hand side; the 4 thread groups each sum a quarter of the tile depth and
  //         the quarters are added in shared memory (no FP64 work on absent columns).
  __shared__ double As[RB][RB + 1];  // As[p][r] = A(I + r, J + p)
  __shared__ double Xs[RB][NR + 1];
  __shared__ double red[4][RB];
  const long long I = (long long)blockIdx.x * RB;
  const long long c0 = (long long)blockIdx.z * NR;
  const int nb = (int)((n + RB - 1) / RB);
  const int jb0 = blockIdx.y * jpc;
  const int jb1 = min(nb, jb0 + jpc);
  const int tid = threadIdx.x, r = tid & 63, cq = tid >> 6;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int jb = jb0; jb < jb1; ++jb) {
    const long long J = (long long)jb * RB;
    // A(I + rr, J + p): stored at a[(J+p)*lda + I+rr] ("direct", contiguous in rr) when in the stored
    // triangle, else at a[(I+rr)*lda + J+p] ("mirrored", contiguous in p).
    const bool all_direct = UP ? (I + RB - 1 <= J) : (I >= J + RB - 1);
    for (int idx = tid; idx < RB * RB; idx += 256) {
      int rr, p;
      if (all_direct) { rr = idx & 63; p = idx >> 6; }
      else            { p = idx & 63; rr = idx >> 6; }
      const long long gi = I + rr, gj = J + p;
      double v = 0.0;
      if (gi < n && gj < n) v = stored<UP>(gi, gj) ? a[gj * lda + gi] : a[gi * lda + gj];
      As[p][rr] = v;
    }
    for (int idx = tid; idx < RB * NR; idx += 256) {
      const int p = idx & 63, c = idx >> 6;
      Xs[p][c] = (J + p < n && c0 + c < nrhs) ? x[(c0 + c) * ldx + J + p] : 0.0;
    }
    __syncthreads();
    if (NR == 1) {
#pragma unroll 4
      for (int p = cq * 16; p < cq * 16 + 16; ++p) acc[0] = fma(As[p][r], Xs[p][0], acc[0]);
    } else {
      for (int p = 0; p < RB; ++p) {
        const double l = As[p][r];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = fma(l, Xs[p][(cq * 4 + q) % NR], acc[q]);
      }
    }
    __syncthreads();
  }
  if (NR == 1) {
    red[cq][r] = acc[0];
    __syncthreads();
    if (cq == 0 && I + r < n && c0 < nrhs)
      part[((long long)blockIdx.y * nrhs + c0) * n + I + r] = (red[0][r] + red[1][r]) + (red[2][r] + red[3][r]);
  } else if (I + r < n) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long c = c0 + cq * 4 + q;
      if (c < nrhs) part[((long long)blockIdx.y * nrhs + c) * n + I + r] = acc[q];
    }
  }
}

__global__ void residual_reduce_kernel(const double* __restrict__ part, int nparts, long long n, long long nrhs,
                                       const double* __restrict__ b, long long ldb, double* __restrict__ r,
                                       long long ldr) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nrhs) return;
  const long long c = idx / n, i = idx % n;
  double s = 0.0;
  for (int k = 0; k < nparts; ++k) s += part[((long long)k * nrhs + c) * n + i];
  r[c * ldr + i] = b[c * ldb + i] - s;
}

// Split-K partition of the FP64 residual: nparts partial sums of jpc row blocks each.
void residual_parts(int64_t n, int64_t nrhs, int* nparts_out, int* jpc_out) {
  const int nb = (int)ceil_div(n, RB), zc = (int)ceil_div(nrhs, RCH);
  int nparts = (int)(1216 / ((int64_t)nb * zc));
  nparts = nparts < 1 ? 1 : (nparts > nb ? nb : nparts);
  const int jpc = (nb + nparts - 1) / nparts;
  *jpc_out = jpc;
  *nparts_out = (nb + jpc - 1) / jpc;
}

// R = B - A X on the FP64 pipe; part holds nparts * n * nrhs doubles.
void symm_residual_fp64(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, const double* x,
                        int64_t ldx, const double* b, int64_t ldb, double* R, int64_t ldr, double* part, int nparts,
                        int jpc, cudaStream_t s) {
  static const std::string kr = "symm_residual_f64";
  ProfScope ps(kr.c_str(), s, 2.0 * n * n * nrhs, (double)n * n * 8.0 + 3.0 * n * nrhs * 8.0);
  const int nb = (int)ceil_div(n, RB), zc = (int)ceil_div(nrhs, RCH);
  if (nrhs == 1) {
    dim3 grid((unsigned)nb, (unsigned)nparts, 1);
    if (upper) symm_partial_kernel<true, 1><<<grid, 256, 0, s>>>(a, lda, n, x, ldx, nrhs, jpc, part);
    else symm_partial_kernel<false, 1><<<grid, 256, 0, s>>>(a, lda, n, x, ldx, nrhs, jpc, part);
  } else {
    dim3 grid((unsigned)nb, (unsigned)nparts, (unsigned)zc);
    if (upper) symm_partial_kernel<true, RCH><<<grid, 256, 0, s>>>(a, lda, n, x, ldx, nrhs, jpc, part);
    else symm_partial_kernel<false, RCH><<<grid, 256, 0, s>>>(a, lda, n, x, ldx, nrhs, jpc, part);
  }
  residual_reduce_kernel<<<(unsigned)ceil_div(n * nrhs, 256), 256, 0, s>>>(part, nparts, n, nrhs, b, ldb, R, ldr);
}

// ---- deterministic sums of squares ------------------------------------------------------------

// mode 0: column-major m x k block (ld);  mode 1/2: symmetric matrix from its lower/upper triangle.
// The work is cut into tasks of SUMSQ_ROWS rows of one column; block b takes the tasks b,
// b + gridDim.x, ... and thread t the rows t, t + 256, ... of each: a fixed order, so the sum does not
// depend on timing, and one index division per task instead of one per element (with a division per
// element the pass over A took milliseconds and crowded the first panel of the factorisation that
// runs beside it).
constexpr long long SUMSQ_ROWS = 2048;
__global__ void __launch_bounds__(256) sumsq_kernel(const double* __restrict__ a, long long ld, long long m, long long k,
                                                    int mode, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  const long long per_col = (m + SUMSQ_ROWS - 1) / SUMSQ_ROWS;
  for (long long t = blockIdx.x; t < k * per_col; t += gridDim.x) {
    const long long j = t / per_col, c = t - j * per_col;
    long long i0 = c * SUMSQ_ROWS, i1 = i0 + SUMSQ_ROWS < m ? i0 + SUMSQ_ROWS : m;
    // the triangle that is not stored is never read (it may hold anything, NaN included)
    if (mode == 1 && i0 < j) i0 = j;
    if (mode == 2 && i1 > j + 1) i1 = j + 1;
    const double* col = a + j * ld;
    for (long long i = i0 + threadIdx.x; i < i1; i += 256) {
      const double v = col[i];
      s += (mode == 0 || i == j ? 1.0 : 2.0) * v * v;
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_parts_kernel(const double* __restrict__ part, int np, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += 256) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Rf = float(d_i * R(i, c) / scale) with scale = sqrt(*ss) (the Frobenius norm of R)
__global__ void residual_to_f32_kernel(const double* __restrict__ r, long long ldr, long long n, long long nrhs,
                                       const double* __restrict__ d, const double* __restrict__ ss,
                                       float* __restrict__ rf, long long ldrf) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nrhs) return;
  const long long c = idx / n, i = idx % n;
  const double sc = sqrt(*ss);
  const double inv = sc > 0.0 ? 1.0 / sc : 0.0;
  rf[c * ldrf + i] = (float)(d[i] * r[c * ldr + i] * inv);
}

// X(i, c) += d_i * Rf(i, c) * scale
__global__ void update_x_kernel(const float* __restrict__ rf, long long ldrf, long long n, long long nrhs,
                                const double* __restrict__ d, const double* __restrict__ ss, double* __restrict__ x,
                                long long ldx, int first) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nrhs) return;
  const long long c = idx / n, i = idx % n;
  const double v = d[i] * (double)rf[c * ldrf + i] * sqrt(*ss);
  x[c * ldx + i] = first ? v : x[c * ldx + i] + v;
}

__global__ void copy_cols_kernel(const double* __restrict__ src, long long lds, long long n, long long nrhs,
                                 double* __restrict__ dst, long long ldd) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nrhs) return;
  const long long c = idx / n, i = idx % n;
  dst[c * ldd + i] = src[c * lds + i];
}

inline unsigned grid1(long long total, int bs = 256) { return (unsigned)((total + bs - 1) / bs); }
inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

struct Arena {
  char* base = nullptr;
  size_t off = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* p = (T*)(base + off);
    off += count * sizeof(T);
    return p;
  }
};

}  // namespace

// Factor the scaled FP32 working matrix af (n x n lower, ldf) with tensor-core trailing updates.
int split_parts(int prec) {
  switch (prec) {
    case GBLLT_PREC_TF32: case GBLLT_PREC_BF16: return 1;
    case GBLLT_PREC_TF32X3: case GBLLT_PREC_BF16X3: return 2;
    case GBLLT_PREC_BF16X6: return 3;
    default: return 0;
  }
}

// SMs left to the panel factorisation while the look-ahead update of the previous panel runs.  With
// the library default (reserve_sms = 0) the reservation follows the panels: the update of panel k
// does about rs^2 panel flops beside the chain of panel k+1 (about rs panel^2 flops, plus a latency
// floor), so the chain's share grows as rs shrinks: SMs / (1 + kReserveRatio rs / panel), between
// kDefaultReserveSms (the first panels; BF16x6, 64 RHS: 32 against 24 saved 0.5-1.7 ms at n = 32768,
// 40 and 48 were slower) and half the SMs.
constexpr int kDefaultReserveSms = 32;
constexpr double kReserveRatio = 0.08;

// Factor the scaled FP32 working matrix af (n x n lower, ldf) with tensor-core trailing updates.
// With a side stream (and the events and second operand set that go with it), one panel of
// lookahead: panel k's trailing update is split into the strip of panel k+1's columns (main stream,
// first) and the rest (side stream), so panel k+1's factorisation overlaps the large update.
//   ev[0/1]: panel k's operands are split (side waits before its update)
//   ev[2/3]: side update k finished (main waits before touching those columns / operand buffers)
// In-panel updates (the remaining columns of the current panel by each 64-column step) also run
// on tcgen05: the step's 64 columns are split into ipparts (K-major, 64 wide) and applied to the
// lower part of the panel's remaining columns.  While the look-ahead update occupies the other
// SMs, these launches are capped to the reserved SMs.
// With an aux stream, the next step's diagonal block is left out of the in-panel update and is
// factored right after the panel solve on the same stream, with this step's contribution applied by
// the diagonal kernel itself, while the rest of the in-panel update runs on aux:
//   ev[4]: the step's panel solve finished (aux waits before the in-panel update)
//   ev[5]: the in-panel update finished (main waits before the next panel solve)
int potrf_mixed_f32(int64_t n, float* af, int64_t ldf, int prec, int panel, int reserve_sms, void* const* parts,
                    void* const* parts2, void* const* ipparts, float* linv, int64_t ldk, DevStatus* st, int* d_err,
                    cudaStream_t s, cudaStream_t side, cudaEvent_t* ev, cudaStream_t aux) {
  static const std::string ksplit = "split_panel";
  const int kind = (prec == GBLLT_PREC_BF16 || prec == GBLLT_PREC_BF16X3 || prec == GBLLT_PREC_BF16X6) ? kTcBF16
                                                                                                       : kTcTF32;
  const int np = split_parts(prec);
  const bool lookahead = side != nullptr && prec != GBLLT_PREC_FP32;
  const int nseg = np == 1 ? 1 : np == 2 ? 3 : 6;
  const uint32_t code = np == 1 ? kSegX1 : np == 2 ? kSegX3 : kSegX6;
  const bool adaptive = reserve_sms == 0;
  int sms = 0;
  if (adaptive) {
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  // SMs reserved for the chain of a panel with rs_chain rows below it
  auto reserve_for = [&](int64_t rs_chain) -> int {
    if (!adaptive) return reserve_sms;
    int v = (int)(sms / (1.0 + kReserveRatio * (double)rs_chain / panel));
    if (v > sms / 2) v = sms / 2;
    return v < kDefaultReserveSms ? kDefaultReserveSms : v;
  };
  int cur_res = adaptive ? kDefaultReserveSms : reserve_sms;  // the reservation of the update in flight
  int iter = 0;
  bool side_pending = false;
  bool diag_ready = false;  // the current step's diagonal block is already factored (previous step)
  bool u_pending = false;   // the previous step's in-panel update runs on aux
  for (int64_t k0 = 0; k0 < n; k0 += panel, ++iter) {
    const int bs = (int)(n - k0 < panel ? n - k0 : panel);
    const int64_t rs = n - k0 - bs;
    // panel: 64-column steps; the in-panel update only touches the panel's remaining columns
    for (int64_t j0 = k0; j0 < k0 + bs; j0 += kNB) {
      const int jb = (int)(k0 + bs - j0 < kNB ? k0 + bs - j0 : kNB);
      const int64_t below = n - j0 - jb;
      const int64_t cols_left = k0 + bs - (j0 + jb);
      // the split precisions solve the panel on the tensor cores with the block's inverse
      float* const li = prec == GBLLT_PREC_FP32 ? nullptr : linv;
      if (diag_ready) diag_ready = false;
      else launch_potrf_diag_f32s(af, ldf, j0, jb, st, s, 0, 0, li);
      if (prec == GBLLT_PREC_FP32) {
        launch_trsm_panel<float>(af, ldf, j0, jb, below, st, s);
        if (cols_left > 0 || rs > 0) launch_syrk_lower<float>(af, ldf, j0, jb, below, below, st, s);
        continue;
      }
      if (u_pending) {  // this step's panel rows below the block come from the previous in-panel update
        GB_CUDA_TRY(cudaStreamWaitEvent(s, ev[5], 0));
        u_pending = false;
      }
      if (cols_left == 0) {
        launch_trsm_panel_tc(af, ldf, j0, jb, below, st, li, 0, 0, nullptr, s);
        continue;
      }
      // the solve writes the step's split operand too (K-major, 64 wide)
      launch_trsm_panel_tc(af, ldf, j0, jb, below, st, li, kind == kTcBF16 ? 0 : 1, np, ipparts, s);
      int64_t skip = 0;  // rows of the next diagonal block, left out of the in-panel update
      cudaStream_t us = s;
      if (aux) {
        // the next diagonal block follows the solve on this stream (applying this step's contribution
        // itself) while the rest of the in-panel update runs on aux
        skip = cols_left < kNB ? cols_left : kNB;
        GB_CUDA_TRY(cudaEventRecord(ev[4], s));
        launch_potrf_diag_f32s(af, ldf, j0 + jb, (int)skip, st, s, j0, jb, li);
        diag_ready = true;
        GB_CUDA_TRY(cudaStreamWaitEvent(aux, ev[4], 0));
        us = aux;
      }
      TcOperand ipa{{ipparts[0], ipparts[1], ipparts[2]}, below, kNB, kNB, skip};
      TcOperand ipb{{ipparts[0], ipparts[1], ipparts[2]}, below, kNB, kNB, 0};
      // capped to the reserved SMs, one left to the diagonal block
      int cap = (lookahead && side_pending && cur_res > 0) ? cur_res : 0;
      if (cap > 1 && aux) --cap;
      const int rc = tc_update(ipa, ipb, kind, nseg, code, af + (j0 + jb) * ldf + (j0 + jb + skip), ldf,
                               below - skip, cols_left, kTcLowerRect, d_err, us, 0, cap, (int)skip);
      if (rc) return rc;
      if (aux) {
        GB_CUDA_TRY(cudaEventRecord(ev[5], aux));
        u_pending = true;
      }
    }
    if (u_pending) {
      GB_CUDA_TRY(cudaStreamWaitEvent(s, ev[5], 0));
      u_pending = false;
    }
    if (rs > 0 && prec != GBLLT_PREC_FP32) {
      void* const* pp = (lookahead && (iter & 1)) ? parts2 : parts;
      // the operand buffers about to be overwritten were last read by the side update two panels ago
      // (waited for here), and the columns of the next panel were last written by the previous side
      // update (waited for before the strip below, so that the split overlaps that update)
      if (lookahead && iter >= 2) GB_CUDA_TRY(cudaStreamWaitEvent(s, ev[2 + (iter & 1)], 0));
      {
        ProfScope ps(ksplit.c_str(), s, 0.0, (double)rs * bs * 4.0 + (double)rs * ldk * (kind == kTcBF16 ? 2 : 4) * np);
        dim3 grid((unsigned)ceil_div(rs, TS), (unsigned)ceil_div(ldk, TS));
        if (kind == kTcBF16)
          split_panel_kernel<0><<<grid, 256, 0, s>>>(af, ldf, k0 + bs, k0, rs, bs, np, pp[0], pp[1], pp[2], ldk);
        else
          split_panel_kernel<1><<<grid, 256, 0, s>>>(af, ldf, k0 + bs, k0, rs, bs, np, pp[0], pp[1], pp[2], ldk);
      }
      if (lookahead && side_pending) GB_CUDA_TRY(cudaStreamWaitEvent(s, ev[2 + ((iter + 1) & 1)], 0));
      TcOperand op{{pp[0], pp[1], pp[2]}, rs, bs, ldk, 0};
      float* c0 = af + (k0 + bs) * ldf + (k0 + bs);
      int rc;
      if (!lookahead || rs <= panel) {
        rc = tc_update(op, op, kind, nseg, code, c0, ldf, rs, rs, kTcLowerTri, d_err, s);
        if (rc) return rc;
      } else {
        const int64_t nb = panel;  // the next panel's width
        // strip: columns of the next panel, all rows below (row >= column inside its top block)
        rc = tc_update(op, op, kind, nseg, code, c0, ldf, rs, nb, kTcLowerRect, d_err, s);
        if (rc) return rc;
        GB_CUDA_TRY(cudaEventRecord(ev[iter & 1], s));
        // the rest of the trailing matrix on the side stream
        GB_CUDA_TRY(cudaStreamWaitEvent(side, ev[iter & 1], 0));
        TcOperand op2{{pp[0], pp[1], pp[2]}, rs, bs, ldk, nb};
        cur_res = reserve_for(rs - nb);
        rc = tc_update(op2, op2, kind, nseg, code, c0 + nb * ldf + nb, ldf, rs - nb, rs - nb, kTcLowerTri, d_err,
                       side, cur_res > 0 ? cur_res : 0);
        if (rc) return rc;
        GB_CUDA_TRY(cudaEventRecord(ev[2 + (iter & 1)], side));
        side_pending = true;
      }
    }
  }
  if (lookahead && side_pending) {
    GB_CUDA_TRY(cudaStreamWaitEvent(s, ev[2], 0));
    GB_CUDA_TRY(cudaStreamWaitEvent(s, ev[3], 0));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

// Default outer panel width.  A wider panel makes each trailing update deeper (fewer passes of C
// through HBM per flop) at the price of a longer panel factorisation.  Solve times to 1e-14 (64 RHS,
// kappa = 1e6):
//   BF16x6, n = 32768: 114 ms at 384, 111 ms at 512, 121 ms at 640 and 768 (a fifth refinement step:
//     the deeper updates' FP32 accumulation in TMEM costs the factor accuracy); n = 24576: 60.5 ms at
//     384, 66 ms at 512 (five steps);
//   BF16x3 (five steps at every width; its error is the two-part split's): n = 32768: 110.2 / 107.5 /
//     106.6 / 106.1 ms at 384 / 512 / 640 / 768; n = 24576: 62.0 / 61.1 / 60.8 ms at 384 / 512 / 640;
//     n = 16384: 31.4 / 31.1 / 31.4 ms at 384 / 512 / 640.
int default_panel(int64_t n, int precision) {
  if (precision == GBLLT_PREC_BF16X3) return n >= 32768 ? 640 : n >= 16384 ? 512 : 256;
  return n >= 16384 ? 384 : 256;
}

int resolve_mixed_opts(const gbllt_mixed_opts* in, gbllt_mixed_opts* o, int64_t n) {
  memset(o, 0, sizeof *o);
  o->precision = GBLLT_PREC_TF32X3;
  o->max_steps = 10;
  o->tol = 1e-14;
  o->fallback_fp64 = 1;
  if (in) {
    *o = *in;
    if (o->max_steps <= 0) o->max_steps = 10;
    if (o->max_steps > 16) o->max_steps = 16;
    if (!(o->tol > 0)) o->tol = 1e-14;
  }
  if (o->panel <= 0) o->panel = default_panel(n, o->precision);
  if (o->precision < GBLLT_PREC_FP32 || o->precision > GBLLT_PREC_BF16X6) return -1;
  if (o->residual != GBLLT_RESIDUAL_AUTO && o->residual != GBLLT_RESIDUAL_TENSOR &&
      o->residual != GBLLT_RESIDUAL_FP64)
    return -1;
  if (o->panel % kNB != 0) return -1;
  return 0;
}

MixedLayout mixed_layout(int64_t n, int64_t nrhs, const gbllt_mixed_opts& o, bool lookahead) {
  MixedLayout L;
  L.ldf = round_up(n, 32);
  L.ldk = round_up(o.panel, 64);
  L.nb = (int)ceil_div(n, RB);
  L.zc = (int)ceil_div(nrhs, RCH);
  residual_parts(n, nrhs, &L.nparts, &L.jpc);
  L.nsq = 512;
  L.es_k = (o.precision == GBLLT_PREC_BF16 || o.precision == GBLLT_PREC_BF16X3 || o.precision == GBLLT_PREC_BF16X6)
               ? 2 : 4;
  L.bytes = (size_t)L.ldf * n * 4 + (size_t)n * 8 + (size_t)n * nrhs * (8 + 4) + (size_t)L.nparts * n * nrhs * 8 +
            (size_t)L.nsq * 8 + 64 + (size_t)split_parts(o.precision) * (lookahead ? 2 : 1) * n * L.ldk * L.es_k +
            (size_t)split_parts(o.precision) * (n * kNB * L.es_k + 256) + kNB * kNB * 4 + 256 +
            sizeof(DevStatus) + 16 * 256 + potrs_ws_bytes(n, 8);
  L.fallback_bytes = (size_t)n * n * 8 + 256;
  return L;
}

int posv_mixed_core(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, const double* b, int64_t ldb,
                    double* x, int64_t ldx, const gbllt_mixed_opts& o, gbllt_mixed_report* rep, void* ws,
                    size_t ws_bytes, bool may_allocate, cudaStream_t s) {
  gbllt_mixed_report r;
  memset(&r, 0, sizeof r);
  const MixedLayout Ly = mixed_layout(n, nrhs, o, may_allocate);
  if (ws_bytes < Ly.bytes) return GBLLT_ERR_ALLOC;
  const int64_t ldf = Ly.ldf, ldk = Ly.ldk;
  const int nparts = Ly.nparts, jpc = Ly.jpc, nsq = Ly.nsq;
  const size_t es_k = Ly.es_k;
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() {
      if (p) cudaFreeAsync(p, s);
    }
  };
  Arena ar{(char*)ws, 0};
  float* af = ar.take<float>((size_t)ldf * n);
  double* dsc = ar.take<double>(n);
  double* R = ar.take<double>((size_t)n * nrhs);
  float* Rf = ar.take<float>((size_t)n * nrhs);
  double* part = ar.take<double>((size_t)nparts * n * nrhs);
  double* sq = ar.take<double>(nsq);
  double* norms = ar.take<double>(8);  // [0] ||A||^2, [1] ||R||^2, [2] ||X||^2
  void* parts[3] = {nullptr, nullptr, nullptr};
  void* parts2[3] = {nullptr, nullptr, nullptr};  // second operand set for the lookahead schedule
  for (int i = 0; i < split_parts(o.precision); ++i) parts[i] = ar.take<char>((size_t)n * ldk * es_k);
  if (may_allocate)
    for (int i = 0; i < split_parts(o.precision); ++i) parts2[i] = ar.take<char>((size_t)n * ldk * es_k);
  void* ipparts[3] = {nullptr, nullptr, nullptr};  // one 64-column step's operands for the in-panel update
  for (int i = 0; i < split_parts(o.precision); ++i) ipparts[i] = ar.take<char>((size_t)n * kNB * es_k);
  float* linv = ar.take<float>(kNB * kNB);  // the current 64-column step's L11^{-1}
  DevStatus* st = ar.take<DevStatus>(1);
  int* d_err = (int*)&st->timeout;
  void* solve_ws = ar.take<char>(potrs_ws_bytes(n, 8));  // sized for the FP64 fallback solve too
  const size_t used = ar.off;

  // device-time stamps (only where creating events is allowed)
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  if (may_allocate)
    for (auto& e : ev) GB_CUDA_TRY(cudaEventCreate(&e));
  struct EvFree {
    cudaEvent_t* e;
    ~EvFree() {
      for (int i = 0; i < 3; ++i)
        if (e[i]) cudaEventDestroy(e[i]);
    }
  } evguard{ev};
  auto stamp = [&](int i) -> int {
    if (ev[i]) GB_CUDA_TRY(cudaEventRecord(ev[i], s));
    return 0;
  };
  auto elapsed = [&](int i, int j) -> double {
    float ms = 0.f;
    if (ev[i] && ev[j]) cudaEventElapsedTime(&ms, ev[i], ev[j]);
    return ms;
  };

  auto sumsq_on = [&](const double* p, int64_t ld, int64_t m, int64_t k, int mode, double* out, cudaStream_t st_) {
    const int64_t tasks = k * ((m + SUMSQ_ROWS - 1) / SUMSQ_ROWS);
    int blocks = (int)(tasks < nsq ? tasks : nsq);
    blocks = blocks < 1 ? 1 : blocks;
    sumsq_kernel<<<blocks, 256, 0, st_>>>(p, ld, m, k, mode, sq);
    sum_parts_kernel<<<1, 256, 0, st_>>>(sq, blocks, out);
  };
  auto sumsq = [&](const double* p, int64_t ld, int64_t m, int64_t k, int mode, double* out) {
    sumsq_on(p, ld, m, k, mode, out, s);
  };
  // the residual on the tensor cores needs A's slices (n^2 * 16 bytes): only where allocating is allowed
  OzakiResidual oz;
  bool use_oz = may_allocate && (o.residual == GBLLT_RESIDUAL_TENSOR ||
                                 (o.residual == GBLLT_RESIDUAL_AUTO && nrhs >= GBLLT_RESIDUAL_TENSOR_MIN_RHS));
  auto residual = [&]() -> int {  // R = B - A X
    if (use_oz && !oz.buf) {  // A's slices, made once, at the first residual
      const int rc2 = oz.setup(upper, n, nrhs, a, lda, s);
      if (rc2 == GBLLT_ERR_ALLOC) use_oz = false;  // not enough device memory: the FP64 residual
      else if (rc2) return rc2;
    }
    if (use_oz) return oz.residual(x, ldx, b, ldb, R, n, s);
    symm_residual_fp64(upper, n, nrhs, a, lda, x, ldx, b, ldb, R, n, part, nparts, jpc, s);
    return GBLLT_SUCCESS;
  };
  // the tensor-core residual's bounded waits report through its own word
  auto residual_timed_out = [&](bool* out) -> int {
    *out = false;
    if (!use_oz) return GBLLT_SUCCESS;
    int h = 0;
    int rc2 = oz.timeout_flag_into(&h, s);
    if (rc2) return rc2;
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    *out = h != 0;
    return GBLLT_SUCCESS;
  };

  GB_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
  GB_CUDA_TRY(cudaMemsetAsync(&st->fail_col, 0xFF, sizeof(long long), s));
  int rc;
  if ((rc = stamp(0))) return rc;
  // 1. scale and round
  if (upper) diag_scale_kernel<true><<<grid1(n), 256, 0, s>>>(a, lda, n, dsc);
  else diag_scale_kernel<false><<<grid1(n), 256, 0, s>>>(a, lda, n, dsc);
  {
    static const std::string kc = "convert_scaled";
    ProfScope ps(kc.c_str(), s, 2.0 * n * (n + 1) / 2, (double)n * (n + 1) / 2 * 12.0);
    const int64_t nt = ceil_div(n, TS);
    if (upper) {
      convert_scaled_upper_kernel<<<(unsigned)(nt * (nt + 1) / 2), 256, 0, s>>>(a, lda, n, dsc, af, ldf);
    } else {
      int sms = 0, dev = 0;
      GB_CUDA_TRY(cudaGetDevice(&dev));
      GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      const int64_t g = (int64_t)sms * 8;
      convert_scaled_lower_kernel<<<(unsigned)(n < g ? n : g), 256, 0, s>>>(a, lda, n, dsc, af, ldf);
    }
  }
  // 2. low-precision factorisation.  Where creating streams is allowed it runs on three internal
  // streams of the highest priority (chain, look-ahead update, next diagonal block), fenced to the
  // caller's stream by events, while a stream of the lowest priority forms what the refinement needs
  // from A alone (||A||_F and the tensor-core residual's slices of A): its blocks take only the slots
  // the factorisation leaves free.
  struct Streams {
    cudaStream_t caller = nullptr;  // may be 0, the legacy default stream
    bool armed = false;             // caller is set and must wait for the internal streams
    cudaStream_t fs = nullptr, side = nullptr, aux = nullptr, low = nullptr;
    cudaEvent_t lev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t in = nullptr, out = nullptr, pre = nullptr;
    ~Streams() {
      // The caller's stream waits for everything issued on these streams before anything it orders
      // later (the release of the workspace they use): on an early error return the factorisation's
      // or the low-priority stream's kernels may still be running.  Work already issued completes.
      // The internal streams are non-blocking, so even the legacy default stream needs the wait.
      for (cudaStream_t q : {fs, side, aux, low}) {
        if (!q || !armed) continue;
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
          if (cudaEventRecord(e, q) == cudaSuccess) cudaStreamWaitEvent(caller, e, 0);
          cudaEventDestroy(e);
        } else {
          cudaStreamSynchronize(q);  // no event: wait on the host instead
        }
      }
      for (cudaStream_t q : {fs, side, aux, low})
        if (q) cudaStreamDestroy(q);
      for (auto& e : lev)
        if (e) cudaEventDestroy(e);
      for (cudaEvent_t e : {in, out, pre})
        if (e) cudaEventDestroy(e);
    }
  } xs;
  bool pre_ready = false;  // ||A||^2 (and A's slices) are being formed on the low-priority stream
  if (may_allocate) {
    xs.caller = s;
    xs.armed = true;
    // A's slices are reserved on the caller's stream, before the fork below, so that every call makes
    // the same allocations on the same stream in the same order and the pool hands back the same
    // blocks (an allocation on a fresh internal stream does not always reuse them)
    if (use_oz) {
      const int rc2 = oz.reserve(n, nrhs, s);
      if (rc2 == GBLLT_ERR_ALLOC) use_oz = false;  // not enough device memory: the FP64 residual
      else if (rc2) return rc2;
    }
    int least = 0, greatest = 0;
    GB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    GB_CUDA_TRY(cudaStreamCreateWithPriority(&xs.fs, cudaStreamNonBlocking, greatest));
    GB_CUDA_TRY(cudaStreamCreateWithPriority(&xs.side, cudaStreamNonBlocking, greatest));
    GB_CUDA_TRY(cudaStreamCreateWithPriority(&xs.aux, cudaStreamNonBlocking, greatest));
    GB_CUDA_TRY(cudaStreamCreateWithPriority(&xs.low, cudaStreamNonBlocking, least));
    for (auto& e : xs.lev) GB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaEvent_t* e : {&xs.in, &xs.out, &xs.pre}) GB_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    GB_CUDA_TRY(cudaEventRecord(xs.in, s));
    GB_CUDA_TRY(cudaStreamWaitEvent(xs.fs, xs.in, 0));
    GB_CUDA_TRY(cudaStreamWaitEvent(xs.low, xs.in, 0));
    sumsq_on(a, lda, n, n, upper ? 2 : 1, &norms[0], xs.low);
    if (use_oz) {
      const int rc2 = oz.setup(upper, n, nrhs, a, lda, xs.low);
      // A's slices are released in the caller's stream order: xs (declared after oz, so destroyed
      // first) makes the caller's stream wait for the low-priority stream on every exit, while the
      // low-priority stream itself is destroyed by then
      if (oz.buf) oz.stream = s;
      if (rc2 == GBLLT_ERR_ALLOC) use_oz = false;  // not enough device memory: the FP64 residual
      else if (rc2) return rc2;
    }
    GB_CUDA_TRY(cudaEventRecord(xs.pre, xs.low));
    pre_ready = true;
    rc = potrf_mixed_f32(n, af, ldf, o.precision, o.panel, o.reserve_sms, parts, parts2, ipparts, linv, ldk, st, d_err,
                         xs.fs, xs.side, xs.lev, xs.aux);
    if (rc) return rc;
    GB_CUDA_TRY(cudaEventRecord(xs.out, xs.fs));
    GB_CUDA_TRY(cudaStreamWaitEvent(s, xs.out, 0));
  } else {
    rc = potrf_mixed_f32(n, af, ldf, o.precision, o.panel, o.reserve_sms, parts, parts2, ipparts, linv, ldk, st, d_err, s,
                         nullptr, xs.lev, nullptr);
    if (rc) return rc;
  }
  if ((rc = stamp(1))) return rc;
  if (pre_ready) {  // everything after this point (norms, residuals, fallback) may use the low stream's results
    GB_CUDA_TRY(cudaStreamWaitEvent(s, xs.pre, 0));
  }
  DevStatus hst;
  GB_CUDA_TRY(cudaMemcpyAsync(&hst, st, sizeof hst, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (hst.timeout) return GBLLT_ERR_TIMEOUT;
  r.info = hst.fail_col >= 0 ? hst.fail_col + 1 : 0;
  r.factor_ms = elapsed(0, 1);

  bool ok = false;
  if (r.info == 0) {
    // 3. refinement: x_0 = 0, r_0 = b
    if (!pre_ready) sumsq(a, lda, n, n, upper ? 2 : 1, &norms[0]);
    copy_cols_kernel<<<grid1(n * nrhs), 256, 0, s>>>(b, ldb, n, nrhs, R, n);
    sumsq(R, n, n, nrhs, 0, &norms[1]);
    double best = INFINITY;
    for (int step = 0; step < o.max_steps; ++step) {
      residual_to_f32_kernel<<<grid1(n * nrhs), 256, 0, s>>>(R, n, n, nrhs, dsc, &norms[1], Rf, n);
      if ((rc = potrs_ws<float>(false, n, nrhs, af, ldf, Rf, n, solve_ws, s))) return rc;
      update_x_kernel<<<grid1(n * nrhs), 256, 0, s>>>(Rf, n, n, nrhs, dsc, &norms[1], x, ldx, step == 0);
      if ((rc = residual())) return rc;
      sumsq(R, n, n, nrhs, 0, &norms[1]);
      sumsq(x, ldx, n, nrhs, 0, &norms[2]);
      double hn[3];
      int serr = 0;  // the FP32 sweeps' error word: a bounded wait ran out
      GB_CUDA_TRY(cudaMemcpyAsync(hn, norms, sizeof hn, cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaMemcpyAsync(&serr, potrs_ws_error_word(n, sizeof(float), solve_ws), sizeof(int),
                                  cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaStreamSynchronize(s));
      bool tmo = false;
      if ((rc = residual_timed_out(&tmo))) return rc;
      if (tmo || serr) return GBLLT_ERR_TIMEOUT;
      const double be =
          (hn[0] > 0 && hn[2] > 0) ? sqrt(hn[1]) / (sqrt(hn[0]) * sqrt(hn[2])) : (hn[1] > 0 ? INFINITY : 0.0);
      r.steps = step + 1;
      if (step < 16) r.history[step] = be;
      r.backward_error = be;
      if (be <= o.tol) {
        ok = true;
        break;
      }
      if (!(be < 0.5 * best) && step >= 2) break;  // stagnation or divergence
      if (be < best) best = be;
    }
  }
  if ((rc = stamp(2))) return rc;
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  r.refine_ms = elapsed(1, 2);
  r.converged = ok ? 1 : 0;

  double* w = nullptr;
  Free wg{nullptr, s};
  if (!ok && o.fallback_fp64) {
    // plain FP64 GPU factorisation of a copy of A (the LAPACK dsposv fallback)
    if (may_allocate) {
      if (dev_malloc_async((void**)&w, (size_t)n * n * 8, s) != cudaSuccess) {
        cudaGetLastError();
        return GBLLT_ERR_ALLOC;
      }
      wg.p = w;
    } else if (ws_bytes >= ((used + 255) & ~(size_t)255) + (size_t)n * n * 8) {
      w = (double*)((char*)ws + ((used + 255) & ~(size_t)255));
    }
  }
  if (w) {
    GB_CUDA_TRY(copy2d_async(w, n * 8, a, lda * 8, n * 8, n, cudaMemcpyDeviceToDevice, s));
    GB_CUDA_TRY(cudaMemsetAsync(&st->fail_col, 0xFF, sizeof(long long), s));
    if (upper && (rc = transpose_inplace_dev<double>(n, w, n, s))) return rc;
    if ((rc = potrf_lower_dev<double>(n, w, n, st, s, may_allocate))) return rc;
    GB_CUDA_TRY(cudaMemcpyAsync(&hst, st, sizeof hst, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hst.timeout) return GBLLT_ERR_TIMEOUT;
    r.used_fallback = 1;
    if (hst.fail_col >= 0) {
      r.info = hst.fail_col + 1;
    } else {
      r.info = 0;
      copy_cols_kernel<<<grid1(n * nrhs), 256, 0, s>>>(b, ldb, n, nrhs, x, ldx);
      if ((rc = potrs_ws<double>(false, n, nrhs, w, n, x, ldx, solve_ws, s))) return rc;
      if ((rc = residual())) return rc;
      sumsq(R, n, n, nrhs, 0, &norms[1]);
      sumsq(x, ldx, n, nrhs, 0, &norms[2]);
      sumsq(a, lda, n, n, upper ? 2 : 1, &norms[0]);
      double hn[3];
      int serr = 0;
      GB_CUDA_TRY(cudaMemcpyAsync(hn, norms, sizeof hn, cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaMemcpyAsync(&serr, potrs_ws_error_word(n, sizeof(double), solve_ws), sizeof(int),
                                  cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaStreamSynchronize(s));
      if (serr) return GBLLT_ERR_TIMEOUT;
      r.backward_error = sqrt(hn[1]) / (sqrt(hn[0]) * sqrt(hn[2]));
      r.converged = r.backward_error <= o.tol;
      ok = true;
    }
  }
  if (rep) *rep = r;
  GB_CUDA_TRY(cudaGetLastError());
  if (r.info != 0) return GBLLT_SUCCESS;  // caller reads report->info
  return ok ? GBLLT_SUCCESS : GBLLT_ERR_NOT_CONVERGED;
}

int posv_mixed_dev(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, const double* b, int64_t ldb,
                   double* x, int64_t ldx, const gbllt_mixed_opts* opts, gbllt_mixed_report* rep, cudaStream_t s) {
  gbllt_mixed_opts o;
  if (resolve_mixed_opts(opts, &o, n)) return -10;
  const MixedLayout Ly = mixed_layout(n, nrhs, o, true);
  void* raw = nullptr;
  if (dev_malloc_async((void**)&raw, Ly.bytes, s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("gbllt_dposv_mixed: allocation of the workspace failed");
    return GBLLT_ERR_ALLOC;
  }
  const int rc = posv_mixed_core(upper, n, nrhs, a, lda, b, ldb, x, ldx, o, rep, raw, Ly.bytes, true, s);
  cudaFreeAsync(raw, s);
  return rc;
}

}  // namespace gbllt

extern "C" int gbllt_dsyresid_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                  const double* d_x, int64_t ldx, const double* d_b, int64_t ldb, double* d_r,
                                  int64_t ldr, int method, void* stream) {
  using namespace gbllt;
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (n > 0 && !d_a) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (n > 0 && nrhs > 0 && !d_x) return -6;
  if (ldx < (n > 1 ? n : 1)) return -7;
  if (n > 0 && nrhs > 0 && !d_b) return -8;
  if (ldb < (n > 1 ? n : 1)) return -9;
  if (n > 0 && nrhs > 0 && !d_r) return -10;
  if (ldr < (n > 1 ? n : 1)) return -11;
  if (method != GBLLT_RESIDUAL_AUTO && method != GBLLT_RESIDUAL_TENSOR && method != GBLLT_RESIDUAL_FP64) return -12;
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const bool upper = uplo == 'U' || uplo == 'u';
  if (method == GBLLT_RESIDUAL_TENSOR ||
      (method == GBLLT_RESIDUAL_AUTO && nrhs >= GBLLT_RESIDUAL_TENSOR_MIN_RHS)) {
    OzakiResidual oz;
    if ((rc = oz.setup(upper, n, nrhs, d_a, lda, s))) return rc;
    return oz.residual(d_x, ldx, d_b, ldb, d_r, ldr, s);
  }
  int nparts = 1, jpc = 1;
  residual_parts(n, nrhs, &nparts, &jpc);
  void* part = nullptr;
  if (dev_malloc_async(&part, (size_t)nparts * n * nrhs * 8, s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("cudaMallocAsync failed");
    return GBLLT_ERR_ALLOC;
  }
  symm_residual_fp64(upper, n, nrhs, d_a, lda, d_x, ldx, d_b, ldb, d_r, ldr, (double*)part, nparts, jpc, s);
  cudaFreeAsync(part, s);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

extern "C" int gbllt_selftest_f64_to_f32(const double* d_in, float* d_out, float* d_ref, int64_t n, void* stream) {
  using namespace gbllt;
  if (n < 0) return -4;
  if (n > 0 && (!d_in || !d_out || !d_ref)) return -1;
  if (n == 0) return GBLLT_SUCCESS;
  const int rc = ensure_device();
  if (rc) return rc;
  f64_to_f32_selftest_kernel<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(d_in, d_out, d_ref, n);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}
