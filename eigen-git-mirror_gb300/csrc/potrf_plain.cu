// Plain-precision blocked Cholesky on the GPU (double for LLT<MatrixXd>, float for
// LLT<MatrixXf>).
//
// The algorithm is the right-looking blocked factorisation of llt_inplace<Scalar,Lower>::blocked
// (Eigen/src/Cholesky/LLT.h:338-368), mapped onto three kernels per panel of width kNB = 64:
//
//   potrf_diag_kernel   one CTA factors the 64 x 64 diagonal block A11 in shared memory
//                       (the role of llt_inplace::unblocked, LLT.h:312-336; the pivot test is
//                       the same `x <= 0`, LLT.h:329).  Where Eigen divides the column by the
//                       pivot, the kernel multiplies by its reciprocal (one division per column).
//                       FP64 arithmetic uses potrf_diag_f64_kernel, laid out for GB300's narrow
//                       FP64 pipe (balanced lanes, pivots off the critical path);
//   trsm_panel_kernel   A21 <- A21 L11^{-T}: four threads per row of A21, the row held in
//                       registers, L11 from shared memory (the OnTheRight solve that
//                       LLT.h:364 issues, TriangularSolverMatrix.h:188-329).  The mixed-precision
//                       factorisation's FP32 panels use trsm_panel_tc_kernel instead: the product
//                       with L11^{-1} (formed by the FP32 diagonal kernel) on the tensor cores;
//   syrk_lower_kernel   A22 -= A21 A21^T on 64 x 64 tiles of the lower triangle only (the rank
//                       update of LLT.h:365 -> GeneralMatrixMatrixTriangular.h:57-194), each
//                       thread accumulating a 4 x 4 register block over the panel depth.
//
// On GB300 the FP64 pipe (DFMA and DMMA alike) delivers about 1 TFLOP/s for the whole chip,
// i.e. under two FP64 FMAs per clock per SM, so every FP64 kernel here is bound by that pipe
// and not by memory: a 64 x 64 x 64 tile update needs 64 KB of operands for 262144 FMAs.
#include <cuda_bf16.h>

#include "internal.h"
#include "mma_split.cuh"

namespace gbllt {

namespace {

constexpr int NB = kNB;

// FP32 diagonal block of the mixed-precision factorisation, in blocks of four columns (the pivot
// test of LLT.h:329, `x <= 0` fails; L(i, j) = A(i, j) * rsqrt(d), L(j, j) = d * rsqrt(d)).  For each block one warp factors the four columns of the rows below
// with shuffles (lane l holds rows j+l and j+l+32), the finished columns go to shared memory, and
// all 512 threads apply the rank-4 update to the trailing triangle, thread (i = tid % 64,
// g = tid / 64) in row i at columns j+4+g, j+12+g, ...  Two barriers per four columns; the loops are
// not unrolled over the blocks, so the code stays in the instruction cache.
// PRE: the block first receives the update of one more panel step, A11 -= P P^T, where P holds the
// pk columns pk0 .. pk0+pk-1 of the block's rows (the step's panel); the caller leaves the block out
// of that step's own trailing update, so this factorisation does not wait for it.
constexpr int DIAG_THREADS = 512;
// LINV: the kernel also writes X = L11^{-1} (64 x 64, row-major, identity beyond bs) to linv, for the
// tensor-core panel solve, in 16 x 16 blocks: 64 threads invert the four diagonal blocks (thread
// (b, j) substitutes column j of block b, unrolled, L read by broadcast), then the blocks below
// follow by distance from the diagonal, d = 1, 2, 3: T = sum_{k=j}^{i-1} L_ik X_kj, then
// X_ij = -X_ii T, every entry of a level at once.  Seven barriers; a warp substitution over the
// whole block issued ten times the instructions.
template <bool PRE, bool LINV>
__global__ void __launch_bounds__(DIAG_THREADS) potrf_diag_f32s_kernel(float* __restrict__ a, long long lda,
                                                                       long long k0, int bs,
                                                                       DevStatus* __restrict__ st, long long pk0,
                                                                       int pk, float* __restrict__ linv) {
  if (st->fail_col >= 0) return;
  constexpr int G = DIAG_THREADS / NB;  // column groups
  __shared__ float s[NB][NB + 1];         // s[c][r] = A(r, c), lower part; L once column c is done
  __shared__ __align__(16) float Lr[NB][4];  // the current block's four columns of L, by row
  __shared__ int s_fail;
  const int tid = threadIdx.x, i = tid & 63, g = tid >> 6;
  float* blk = a + k0 * lda + k0;
  {
    float v[NB * NB / DIAG_THREADS];  // all loads in flight before the first shared store
#pragma unroll
    for (int u = 0; u < NB * NB / DIAG_THREADS; ++u) {
      const int c = (tid >> 6) + u * G, r = tid & 63;
      v[u] = (r < bs && c < bs && r >= c) ? blk[(long long)c * lda + r] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < NB * NB / DIAG_THREADS; ++u) s[(tid >> 6) + u * G][tid & 63] = v[u];
  }
  constexpr int PP = NB + 4;                   // row pitch: rows stay 16-byte aligned
  __shared__ __align__(16) float pr[NB * PP];  // PRE: pr[r * PP + q] = P(r, q), zero beyond pk; LINV: X
  if constexpr (PRE) {
    const float* pan = a + pk0 * lda + k0;
    {
      float v[NB * NB / DIAG_THREADS];
#pragma unroll
      for (int u = 0; u < NB * NB / DIAG_THREADS; ++u) {
        const int q = (tid >> 6) + u * G, r = tid & 63;
        v[u] = (r < bs && q < pk) ? pan[(long long)q * lda + r] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < NB * NB / DIAG_THREADS; ++u) pr[(tid & 63) * PP + (tid >> 6) + u * G] = v[u];
    }
    __syncthreads();
    // thread (i, g): entries (i, k) for k = g, g + 8, ... <= i, each a dot product over the pk
    // columns, four at a time (row k's reads are the same for the whole warp)
    float acc[NB / G];
#pragma unroll
    for (int m = 0; m < NB / G; ++m) acc[m] = 0.f;
    for (int q = 0; q < NB; q += 4) {
      const float4 pi = *reinterpret_cast<const float4*>(pr + i * PP + q);
#pragma unroll
      for (int m = 0; m < NB / G; ++m) {
        if (g + G * m <= i) {
          const float4 pk4 = *reinterpret_cast<const float4*>(pr + (g + G * m) * PP + q);
          acc[m] = fmaf(pi.x, pk4.x, acc[m]);
          acc[m] = fmaf(pi.y, pk4.y, acc[m]);
          acc[m] = fmaf(pi.z, pk4.z, acc[m]);
          acc[m] = fmaf(pi.w, pk4.w, acc[m]);
        }
      }
    }
#pragma unroll
    for (int m = 0; m < NB / G; ++m)
      if (g + G * m <= i) s[g + G * m][i] -= acc[m];
  }
  if (tid == 0) s_fail = -1;
  __syncthreads();
  int done = bs;  // finished columns
  for (int j = 0; j < bs; j += 4) {
    const int w = bs - j < 4 ? bs - j : 4;  // columns of this block
    // (a) one warp factors columns j .. j+w-1 of rows j .. bs-1: lane l holds rows j+l and j+l+32;
    //     the pivot and L(j+c2, j+c) come from the lane that holds row j+c (j+c2) by shuffle
    if (tid < 32) {
      const int l = tid, r0 = j + l, r1 = j + l + 32;
      float v0[4], v1[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        v0[c] = (c < w && r0 < bs && r0 >= j + c) ? s[j + c][r0] : 0.f;
        v1[c] = (c < w && r1 < bs) ? s[j + c][r1] : 0.f;
      }
      int f = 4;  // first column of the block whose pivot fails the test (4: none)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (c < w && f == 4) {  // uniform over the warp
          const float d = __shfl_sync(0xffffffffu, v0[c], c);
          if (!(d > 0.f)) {
            f = c;
          } else {
            // one MUFU reciprocal square root on the serial path; the refinement that uses this
            // factor absorbs its last-bit differences from the correctly rounded sqrt and division
            const float inv = rsqrtf(d);
            v0[c] = l == c ? d * inv : v0[c] * inv;
            v1[c] *= inv;
#pragma unroll
            for (int c2 = c + 1; c2 < 4; ++c2) {
              const float lc = __shfl_sync(0xffffffffu, v0[c], c2);  // L(j + c2, j + c)
              v0[c2] = fmaf(-v0[c], lc, v0[c2]);
              v1[c2] = fmaf(-v1[c], lc, v1[c2]);
            }
          }
        }
      }
      const int fin = f < w ? f : w;  // finished columns of the block
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (c < fin && r0 < bs && r0 >= j + c) s[j + c][r0] = v0[c];
        if (c < fin && r1 < bs) s[j + c][r1] = v1[c];
      }
      if (r0 >= j + 4 && r0 < bs)
        *reinterpret_cast<float4*>(Lr[r0]) = make_float4(0 < fin ? v0[0] : 0.f, 1 < fin ? v0[1] : 0.f,
                                                         2 < fin ? v0[2] : 0.f, 3 < fin ? v0[3] : 0.f);
      if (r1 < bs)
        *reinterpret_cast<float4*>(Lr[r1]) = make_float4(0 < fin ? v1[0] : 0.f, 1 < fin ? v1[1] : 0.f,
                                                         2 < fin ? v1[2] : 0.f, 3 < fin ? v1[3] : 0.f);
      if (l == 0 && f < w) s_fail = j + f;
    }
    __syncthreads();
    if (s_fail >= 0) {  // block-uniform
      done = s_fail;
      break;
    }
    // (b) rank-4 update of the trailing triangle, rows and columns from j + 4
    const int jn = j + 4;
    if (i >= jn && i < bs) {
      const float4 li = *reinterpret_cast<const float4*>(Lr[i]);
      int k = jn + g;
      for (; k + G <= i; k += 2 * G) {
        const float4 l0 = *reinterpret_cast<const float4*>(Lr[k]);
        const float4 l1 = *reinterpret_cast<const float4*>(Lr[k + G]);
        float a0 = s[k][i], a1 = s[k + G][i];
        a0 = fmaf(-li.x, l0.x, a0); a1 = fmaf(-li.x, l1.x, a1);
        a0 = fmaf(-li.y, l0.y, a0); a1 = fmaf(-li.y, l1.y, a1);
        a0 = fmaf(-li.z, l0.z, a0); a1 = fmaf(-li.z, l1.z, a1);
        a0 = fmaf(-li.w, l0.w, a0); a1 = fmaf(-li.w, l1.w, a1);
        s[k][i] = a0;
        s[k + G][i] = a1;
      }
      if (k <= i) {
        const float4 l0 = *reinterpret_cast<const float4*>(Lr[k]);
        float a0 = s[k][i];
        a0 = fmaf(-li.x, l0.x, a0);
        a0 = fmaf(-li.y, l0.y, a0);
        a0 = fmaf(-li.z, l0.z, a0);
        a0 = fmaf(-li.w, l0.w, a0);
        s[k][i] = a0;
      }
    }
    __syncthreads();
  }
  for (int idx = tid; idx < NB * NB; idx += DIAG_THREADS) {
    const int c = idx >> 6, r = idx & 63;
    if (c < done && r < bs && r >= c) blk[(long long)c * lda + r] = s[c][r];
  }
  if (tid == 0 && done < bs) st->fail_col = k0 + done;
  if constexpr (LINV) {
    static_assert(DIAG_THREADS >= 3 * 256 / 2 && NB == 64, "four 16 x 16 blocks per side");
    if (done < bs) return;  // failed: the panel solve does not run (block-uniform)
    // s holds L (zero above the diagonal and beyond bs); the identity continues past bs
    float* xs = pr;                  // xs[r * PP + c] = X(r, c)
    __shared__ float rinv[NB];       // 1 / L(r, r), 1 beyond bs
    __shared__ float tb[3][16][17];  // T of the blocks of one level
    if (tid < NB) rinv[tid] = tid < bs ? 1.f / s[tid][tid] : 1.f;
    __syncthreads();
    if (tid < NB) {  // diagonal block b, column j: rows i = 0 .. 15 by substitution
      const int b = tid >> 4, j = tid & 15, o = 16 * b;
      float x[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        float acc = i == j ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < i; ++k) acc = fmaf(-s[o + k][o + i], x[k], acc);  // x[k] = 0 for k < j
        x[i] = acc * rinv[o + i];
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) xs[(o + i) * PP + o + j] = x[i];
    }
    __syncthreads();
    for (int d = 1; d < 4; ++d) {
      const int cnt = (4 - d) * 256;  // blocks (j + d, j), j = 0 .. 3 - d
      for (int idx = tid; idx < cnt; idx += DIAG_THREADS) {
        const int jb = idx >> 8, r = (idx >> 4) & 15, c = idx & 15, ib = jb + d;
        float t0 = 0.f, t1 = 0.f;
        for (int q = 16 * jb; q < 16 * ib; q += 2) {
          t0 = fmaf(s[q][16 * ib + r], xs[q * PP + 16 * jb + c], t0);
          t1 = fmaf(s[q + 1][16 * ib + r], xs[(q + 1) * PP + 16 * jb + c], t1);
        }
        tb[jb][r][c] = t0 + t1;
      }
      __syncthreads();
      for (int idx = tid; idx < cnt; idx += DIAG_THREADS) {
        const int jb = idx >> 8, r = (idx >> 4) & 15, c = idx & 15, ib = jb + d;
        float v = 0.f;
#pragma unroll
        for (int m = 0; m < 16; ++m) v = fmaf(xs[(16 * ib + r) * PP + 16 * ib + m], tb[jb][m][c], v);
        xs[(16 * ib + r) * PP + 16 * jb + c] = -v;
      }
      __syncthreads();
    }
    for (int idx = tid; idx < NB * NB; idx += DIAG_THREADS) {
      const int r = idx >> 6, c = idx & 63;
      linv[idx] = (c >> 4) <= (r >> 4) ? xs[r * PP + c] : 0.f;
    }
  }
}

// T = storage type, TC = arithmetic type (the mixed-precision path stores float and factors the
// diagonal block in double).
template <typename T, typename TC>
__global__ void __launch_bounds__(256) potrf_diag_kernel(T* __restrict__ a, long long lda, long long k0, int bs,
                                                         DevStatus* __restrict__ st) {
  if (st->fail_col >= 0) return;  // an earlier panel already failed: nothing more to do
  __shared__ TC s[NB][NB + 1];   // s[j][i] = A11(i, j), lower part only
  __shared__ int fail;
  const int tid = threadIdx.x;
  T* blk = a + k0 * lda + k0;
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int j = idx / NB, i = idx % NB;
    if (i < bs && j < bs && i >= j) s[j][i] = (TC)blk[(long long)j * lda + i];
  }
  if (tid == 0) fail = -1;
  __syncthreads();
  const int tx = tid & 63, ty = tid >> 6;
  __shared__ TC inv_s;
  int j = 0;
  for (; j < bs; ++j) {
    if (tid == 0) {
      const TC d = s[j][j];
      if (d <= TC(0)) fail = j;
      else {
        const TC r = sqrt(d);
        s[j][j] = r;
        inv_s = TC(1) / r;  // one division per column; the column is scaled by multiplication
      }
    }
    __syncthreads();
    if (fail >= 0) break;  // block-uniform
    const TC inv = inv_s;
    if (tid > j && tid < bs) s[j][tid] = s[j][tid] * inv;
    __syncthreads();
    for (int l = j + 1 + ty; l < bs; l += 4) {
      const TC ljl = s[j][l];
      if (tx >= l && tx < bs) s[l][tx] = fma(-s[j][tx], ljl, s[l][tx]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int jj = idx / NB, i = idx % NB;
    if (i < bs && jj < bs && i >= jj) blk[(long long)jj * lda + i] = (T)s[jj][i];
  }
  if (tid == 0 && fail >= 0) st->fail_col = k0 + fail;
}

// 1/sqrt(d) in FP64: the Newton-Raphson iteration for the reciprocal square root,
// y <- y (3 - d y^2) / 2 (quadratic convergence), applied STEPS times to the FP32 estimate
// rsqrtf(d): about 22 correct bits, 44 after one step, the FP64 rounding limit (a few units in the
// last place) after two.  Outside the range where the FP32 estimate is defined, the library's sqrt
// and division are used.
template <int STEPS>
__device__ __forceinline__ double rsqrt_newton(double d) {
  if (d > 1e-36 && d < 1e36) {
    double y = (double)rsqrtf((float)d);
    const double h = 0.5 * d;
#pragma unroll
    for (int i = 0; i < STEPS; ++i) y = y * fma(-h * y, y, 1.5);
    return y;
  }
  return 1.0 / sqrt(d);
}

// The 64 x 64 diagonal block in FP64 arithmetic (storage T: double for the plain path, float for
// the mixed-precision one).  On GB300 an FP64 warp instruction holds its SM sub-partition's FP64
// unit for about 70 clocks whatever the number of active lanes, and a dependent FP64 instruction
// waits that long; the kernel is arranged around both facts:
//   - lane p of each warp owns the row pair (p, 63 - p), whose trailing parts together have
//     63 - 2j elements in column step j, nearly the same for every lane (no idle lanes);
//   - 16 warps, four per sub-partition, warp w updating the columns c = w (mod 16), so each
//     sub-partition always has independent FP64 work to overlap latencies with;
//   - the thread that updates the element (j+1, j+1) does it first and takes the next pivot at
//     once, while the other warps finish the update, so the pivot's dependent chain (one
//     reciprocal square root) overlaps the update instead of following it.
// Per column: warps 0/1 scale rows p / 63 - p by the reciprocal pivot, one barrier, the rank-1
// update, one barrier.  The pivot test is the `x <= 0` of LLT.h:328 (a NaN pivot passes it).  Rows
// and columns beyond bs are padded with the identity, which factors to itself.  With FP32 storage
// one Newton step suffices: its 44 bits exceed by far the 24 the factor is rounded to.
template <typename T>
__global__ void __launch_bounds__(512) potrf_diag_f64_kernel(T* __restrict__ a, long long lda, long long k0, int bs,
                                                             DevStatus* __restrict__ st) {
  constexpr int STEPS = sizeof(T) == 8 ? 2 : 1;
  constexpr int NW = 16;  // warps, and the column residue classes
  if (st->fail_col >= 0) return;
  __shared__ double s[NB][NB + 1];  // s[c][r] = A11(r, c), lower part
  __shared__ double col[NB];        // L(r, j) of the current column j
  __shared__ double piv;            // 1 / L(j, j)
  __shared__ int fail;
  const int tid = threadIdx.x, w = tid >> 5, p = tid & 31;
  T* blk = a + k0 * lda + k0;
  for (int idx = tid; idx < NB * NB; idx += 32 * NW) {
    const int c = idx / NB, r = idx % NB;
    double v = (r == c) ? 1.0 : 0.0;
    if (r < bs && c < bs && r >= c) v = (double)blk[(long long)c * lda + r];
    s[c][r] = v;
  }
  __syncthreads();
  if (tid == 0) {
    fail = -1;
    const double d = s[0][0];
    if (d <= 0.0) {
      fail = 0;
    } else {
      const double y = rsqrt_newton<STEPS>(d);
      s[0][0] = d * y;
      piv = y;
    }
  }
  __syncthreads();
  const int r0 = p, r1 = NB - 1 - p;
  for (int j = 0; j < NB; ++j) {
    if (fail >= 0) break;  // block-uniform: read after a barrier
    if (w < 2) {
      const int r = w == 0 ? r0 : r1;
      if (r > j) {
        const double l = s[j][r] * piv;
        s[j][r] = l;
        col[r] = l;
      }
    }
    __syncthreads();
    const int cfirst = j + 1 + ((w - (j + 1)) & (NW - 1));  // smallest column c > j with c = w (mod 16)
    const int n1 = r0 >= cfirst ? (r0 - cfirst) / NW + 1 : 0;
    const int n2 = r1 >= cfirst ? (r1 - cfirst) / NW + 1 : 0;
    const double l0 = r0 > j ? col[r0] : 0.0, l1 = r1 > j ? col[r1] : 0.0;
    for (int k = 0; k < n1 + n2; ++k) {
      const bool first = k < n1;
      const int r = first ? r0 : r1;
      const int c = cfirst + NW * (first ? k : k - n1);
      const double v = fma(-(first ? l0 : l1), col[c], s[c][r]);
      if (r == j + 1 && c == j + 1) {  // the next pivot (k == 0 for its thread), as soon as it is known
        if (v <= 0.0) {
          fail = j + 1;
          s[c][r] = v;
        } else {
          const double y = rsqrt_newton<STEPS>(v);
          s[c][r] = v * y;
          piv = y;
        }
      } else {
        s[c][r] = v;
      }
    }
    __syncthreads();
  }
  __syncthreads();
  for (int idx = tid; idx < NB * NB; idx += 32 * NW) {
    const int c = idx / NB, r = idx % NB;
    if (r < bs && c < bs && r >= c) blk[(long long)c * lda + r] = (T)s[c][r];
  }
  if (tid == 0 && fail >= 0) st->fail_col = k0 + fail;
}

// A21 (rs x bs, rows k0+bs.., columns k0..) <- A21 * L11^{-T}.  One thread per row.
template <typename T>
__device__ __forceinline__ void ld4(const T* p, T* v) {
  if constexpr (sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else {
    const double2 q0 = *reinterpret_cast<const double2*>(p);
    const double2 q1 = *reinterpret_cast<const double2*>(p + 2);
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
  }
}

// A21 <- A21 L11^{-T}, four threads per row of A21: sub-lane s of a quad holds the row's columns
// p = 4m + s (m < 16) in registers.  The substitution runs right-looking: for column j the owner
// (s = j % 4) scales x_j by 1 / L11(j, j), one shuffle hands it to the quad, and each thread
// updates its later columns x_p -= x_j L11(p, j), which are independent of each other.  L11 is kept
// per sub-lane (Lq[s][j][m] = L11(4m + s, j)), so a thread's reads are 16-byte vectors; the
// sub-lane blocks are 16 bytes apart in bank order.  Compared with one thread per row, the code is
// a third as long and four times as many warps share it.  (The split precisions of the mixed
// factorisation use trsm_panel_tc_kernel below instead.)
constexpr int TRSM_ROWS = 32;  // rows per CTA of 128 threads
template <typename T>
__global__ void __launch_bounds__(128) trsm_panel_kernel(T* __restrict__ a, long long lda, long long k0, int bs,
                                                         long long rs, const DevStatus* __restrict__ st) {
  if (st->fail_col >= 0) return;
  constexpr int QS = NB * 16 + 16 / (int)sizeof(T);  // sub-lane block stride
  __shared__ __align__(16) T Lq[4 * QS];
  __shared__ T rdiag[NB];  // 1 / L11(j, j); 1 outside the bs x bs block
  const T* l11 = a + (long long)k0 * lda + k0;
  for (int idx = threadIdx.x; idx < NB * NB; idx += 128) {
    const int p = idx % NB, j = idx / NB;  // consecutive threads read consecutive rows of column j
    T v = T(0);
    if (p > j && p < bs && j < bs) v = l11[(long long)j * lda + p];
    Lq[(p & 3) * QS + j * 16 + (p >> 2)] = v;
  }
  if (threadIdx.x < NB) rdiag[threadIdx.x] = threadIdx.x < bs ? T(1) / l11[(long long)threadIdx.x * (lda + 1)] : T(1);
  __syncthreads();
  const int lane = threadIdx.x & 31, sl = threadIdx.x & 3, rl = threadIdx.x >> 2;
  const long long r = (long long)blockIdx.x * TRSM_ROWS + rl;
  const bool live = r < rs;  // every lane stays for the quad shuffles
  T* row = a + (long long)k0 * lda + (k0 + bs) + (live ? r : 0);  // element (r, p) at row[p * lda]
  T x[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) x[m] = (live && 4 * m + sl < bs) ? row[(long long)(4 * m + sl) * lda] : T(0);
  const T* lq = Lq + sl * QS;
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    const int owner = j & 3, mj = j >> 2;
    if (sl == owner) x[mj] *= rdiag[j];
    const T xj = __shfl_sync(0xffffffffu, x[mj], (lane & ~3) | owner);
    if (sl > owner) x[mj] = fma(-xj, lq[j * 16 + mj], x[mj]);
#pragma unroll
    for (int c = (mj + 1) >> 2; c < 4; ++c) {  // later chunks of four m
      T l[4];
      ld4<T>(lq + j * 16 + 4 * c, l);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (4 * c + u > mj) x[4 * c + u] = fma(-xj, l[u], x[4 * c + u]);
    }
  }
  if (live) {
#pragma unroll
    for (int m = 0; m < 16; ++m)
      if (4 * m + sl < bs) row[(long long)(4 * m + sl) * lda] = x[m];
  }
}

// A21 <- A21 L11^{-T} as a product with the inverse that the diagonal kernel wrote (linv[c * 64 + p]
// = L11^{-1}(c, p)), on the tensor cores: mma.sync m16n8k16 with the three-part BF16 split of
// mma_split.cuh (FP32-accurate; the six products of each output go into a zeroed accumulator, 64
// deep).  The substitution kernel above is a chain of 64 dependent steps per row with a shuffle
// each; this is one 64-deep product per row, the rows independent.  Linv's zero upper triangle is
// skipped (8-column tiles left of the k16 step).
// CTA: 128 threads, 64 rows (TT_ROWS).  The A21 tile is staged column by column (As[p * 68 + r],
// coalesced 16-byte loads) and the inverse's parts as rows (Lp[part][c * 72 + p]); both pitches make
// the fragment reads conflict-free.  Warp w owns rows 16 w .. 16 w + 15 and all 64 columns (eight
// n8 tiles).  X goes back through As: column-major to A21, and as np split parts (K-major, 64 per
// row) for the in-panel update.
constexpr int TT_ROWS = 64, TT_PITCH = 68, TL_PITCH = 72;
template <int SPLIT>
__global__ void __launch_bounds__(128) trsm_panel_tc_kernel(float* __restrict__ a, long long lda, long long k0, int bs,
                                                            long long rs, const DevStatus* __restrict__ st,
                                                            const float* __restrict__ linv, int np,
                                                            void* __restrict__ p0, void* __restrict__ p1,
                                                            void* __restrict__ p2) {
  if (st->fail_col >= 0) return;
  __shared__ __align__(16) float As[NB * TT_PITCH];
  __shared__ __align__(16) __nv_bfloat16 Lp[3][NB * TL_PITCH];
  const int tid = threadIdx.x;
  const long long row0 = (long long)blockIdx.x * TT_ROWS;
  float* const src = a + k0 * lda + (k0 + bs) + row0;  // element (r, p) at src[p * lda + r]
  const int nrow = rs - row0 < TT_ROWS ? (int)(rs - row0) : TT_ROWS;
  const bool vec = (lda & 3) == 0 && ((k0 + bs + row0) & 3) == 0 && nrow == TT_ROWS;
  // the A21 tile (zero beyond bs columns and nrow rows)
  if (vec) {
    float4 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = tid + 128 * u, p = idx >> 4, r4 = (idx & 15) * 4;
      v[u] = p < bs ? *reinterpret_cast<const float4*>(src + (long long)p * lda + r4) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = tid + 128 * u, p = idx >> 4, r4 = (idx & 15) * 4;
      *reinterpret_cast<float4*>(As + p * TT_PITCH + r4) = v[u];
    }
  } else {
    for (int idx = tid; idx < NB * TT_ROWS; idx += 128) {
      const int p = idx >> 6, r = idx & 63;
      As[p * TT_PITCH + r] = (p < bs && r < nrow) ? src[(long long)p * lda + r] : 0.f;
    }
  }
  // the inverse's three parts, row c of Linv at Lp[part][c * 72 ..]
  {
    float4 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = reinterpret_cast<const float4*>(linv)[tid + 128 * u];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = (tid + 128 * u) * 4, c = idx >> 6, p = idx & 63;
      uint32_t lo[3], hi[3];
      split3_bf16x2(v[u].x, v[u].y, lo);
      split3_bf16x2(v[u].z, v[u].w, hi);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        *reinterpret_cast<uint2*>(&Lp[k][c * TL_PITCH + p]) = make_uint2(lo[k], hi[k]);
    }
  }
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int m0 = 16 * warp;
  float c[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) c[nt][i] = 0.f;
#pragma unroll
  for (int ks = 0; ks < NB; ks += 16) {
    uint32_t ap[4][3];  // A fragment register i (rows g, g + 8, g, g + 8; k 2t / 2t + 8), part
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = m0 + g + 8 * (i & 1), k = ks + 2 * t + 8 * (i >> 1);
      split3_bf16x2(As[k * TT_PITCH + row], As[(k + 1) * TT_PITCH + row], ap[i]);
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      if (ks > 8 * nt + 7) continue;  // Linv(c, p) = 0 for p > c: the whole k16 x n8 block
      const int col = 8 * nt + g;
      uint32_t b0[3], b1[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        b0[k] = *reinterpret_cast<const uint32_t*>(&Lp[k][col * TL_PITCH + ks + 2 * t]);
        b1[k] = *reinterpret_cast<const uint32_t*>(&Lp[k][col * TL_PITCH + ks + 2 * t + 8]);
      }
      mma_split6(c[nt], ap, b0, b1);
    }
  }
  // X back into the warp's own rows of As (no other warp reads them), then out
  __syncwarp();
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) As[(8 * nt + 2 * t + (i & 1)) * TT_PITCH + m0 + g + 8 * (i >> 1)] = c[nt][i];
  __syncthreads();
  if (vec) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = tid + 128 * u, p = idx >> 4, r4 = (idx & 15) * 4;
      if (p < bs)
        *reinterpret_cast<float4*>(src + (long long)p * lda + r4) = *reinterpret_cast<const float4*>(As + p * TT_PITCH + r4);
    }
  } else {
    for (int idx = tid; idx < NB * TT_ROWS; idx += 128) {
      const int p = idx >> 6, r = idx & 63;
      if (p < bs && r < nrow) src[(long long)p * lda + r] = As[p * TT_PITCH + r];
    }
  }
  if constexpr (SPLIT != 0) {
    // 8 columns of one row per 16-byte BF16 store (two for TF32); consecutive threads, consecutive rows
    for (int idx = tid; idx < TT_ROWS * (NB / 8); idx += 128) {
      const int r = idx & 63, pc = (idx >> 6) * 8;
      if (r >= nrow) continue;
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = As[(pc + u) * TT_PITCH + r];
      const long long e = (row0 + r) * NB + pc;
      for (int k = 0; k < np; ++k) {
        void* part = k == 0 ? p0 : (k == 1 ? p1 : p2);
        if (SPLIT == 1) {
          uint32_t w[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * u], v[2 * u + 1]);
            w[u] = *reinterpret_cast<const uint32_t*>(&h);
            v[2 * u] -= __low2float(h);
            v[2 * u + 1] -= __high2float(h);
          }
          *reinterpret_cast<uint4*>((__nv_bfloat16*)part + e) = make_uint4(w[0], w[1], w[2], w[3]);
        } else {
          float h[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            h[u] = to_tf32(v[u]);
            v[u] -= h[u];
          }
          float4* dst = reinterpret_cast<float4*>((float*)part + e);
          dst[0] = make_float4(h[0], h[1], h[2], h[3]);
          dst[1] = make_float4(h[4], h[5], h[6], h[7]);
        }
      }
    }
  }
}

// A22 (rs x rs lower) -= A21 B^T, A21 = rs x bs, B = A21 (Cholesky) or the rs x bs array at bsrc
// with leading dimension ldb (LDL^T: B = A21 D).  One CTA per 64 x 64 lower tile.  Only the
// first `ncols` columns of A22 are updated (nct = ceil(ncols / 64) column tiles): the whole lower
// triangle when ncols = rs, or the remaining columns of the current panel when the mixed-precision
// path factors a wide panel in 64-column steps.
template <typename T>
__global__ void __launch_bounds__(256) syrk_lower_kernel(T* __restrict__ a, long long lda, long long k0, int bs,
                                                         long long rs, long long ncols, int nct,
                                                         const DevStatus* __restrict__ st,
                                                         const T* __restrict__ bsrc, long long ldb) {
  if (st->fail_col >= 0) return;
  constexpr int KC = 32;
  __shared__ T As[KC][64 + 1];
  __shared__ T Bs[KC][64 + 1];
  int ti, tj;
  const int mt = (int)((rs + 63) / 64);
  if (nct >= mt) {
    lower_tile_coords(blockIdx.x, ti, tj);
  } else {  // column tiles 0..nct-1, each holding the row tiles tj..mt-1
    long long t = blockIdx.x;
    tj = 0;
    while (t >= mt - tj) { t -= mt - tj; ++tj; }
    ti = tj + (int)t;
  }
  const long long i0 = (long long)ti * 64, j0 = (long long)tj * 64;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const T* A = a + (long long)k0 * lda + (k0 + bs);  // A21(0, 0)
  const T* B = bsrc ? bsrc : A;
  if (!bsrc) ldb = lda;
  T acc[4][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[m][q] = T(0);
  for (int p0 = 0; p0 < bs; p0 += KC) {
    for (int idx = tid; idx < 64 * KC; idx += 256) {
      const int i = idx & 63, p = idx >> 6;
      T va = T(0), vb = T(0);
      if (p0 + p < bs) {
        if (i0 + i < rs) va = A[(long long)(p0 + p) * lda + i0 + i];
        if (j0 + i < rs) vb = B[(long long)(p0 + p) * ldb + j0 + i];
      }
      As[p][i] = va;
      Bs[p][i] = vb;
    }
    __syncthreads();
    const int pe = bs - p0 < KC ? bs - p0 : KC;
    for (int p = 0; p < pe; ++p) {
      T av[4], bv[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) av[m] = As[p][tx + 16 * m];
#pragma unroll
      for (int q = 0; q < 4; ++q) bv[q] = Bs[p][ty + 16 * q];
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][q] = fma(av[m], bv[q], acc[m][q]);
    }
    __syncthreads();
  }
  T* C = a + (long long)(k0 + bs) * lda + (k0 + bs);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const long long j = j0 + ty + 16 * q;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const long long i = i0 + tx + 16 * m;
      if (i < rs && j < ncols && i >= j) C[j * lda + i] -= acc[m][q];
    }
  }
}

// Swap strict triangles: one CTA per pair of 32 x 32 tiles (ti, tj), (tj, ti) with ti >= tj.
template <typename T>
__global__ void __launch_bounds__(256) transpose_inplace_kernel(T* __restrict__ a, long long lda, long long n) {
  __shared__ T t1[32][33];
  __shared__ T t2[32][33];
  int ti, tj;
  lower_tile_coords(blockIdx.x, ti, tj);
  const long long r1 = (long long)ti * 32, c1 = (long long)tj * 32;  // tile (ti, tj)
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int c = ty; c < 32; c += 8) {
    const long long i = r1 + tx, j = c1 + c;  // element of tile (ti,tj)
    if (i < n && j < n) t1[c][tx] = a[j * lda + i];
    const long long i2 = c1 + tx, j2 = r1 + c;  // element of tile (tj,ti)
    if (i2 < n && j2 < n) t2[c][tx] = a[j2 * lda + i2];
  }
  __syncthreads();
  // tile (ti,tj)(x, c) <- tile(tj,ti)(c, x) ; tile (tj,ti)(x, c) <- tile(ti,tj)(c, x)
  for (int c = ty; c < 32; c += 8) {
    const long long i = r1 + tx, j = c1 + c;
    if (i < n && j < n && i != j) a[j * lda + i] = t2[tx][c];
    const long long i2 = c1 + tx, j2 = r1 + c;
    if (i2 < n && j2 < n && i2 != j2) a[j2 * lda + i2] = t1[tx][c];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) transpose_kernel(long long rows, long long cols, const T* __restrict__ src,
                                                        long long lds, T* __restrict__ dst, long long ldd) {
  __shared__ T t[32][33];
  const long long r0 = (long long)blockIdx.x * 32, c0 = (long long)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int c = ty; c < 32; c += 8)
    if (r0 + tx < rows && c0 + c < cols) t[c][tx] = src[(c0 + c) * lds + r0 + tx];
  __syncthreads();
  // dst(c, r) = src(r, c): dst column r0 + c, row c0 + tx
  for (int c = ty; c < 32; c += 8)
    if (r0 + c < rows && c0 + tx < cols) dst[(r0 + c) * ldd + c0 + tx] = t[tx][c];
}

__global__ void finalize_info_kernel(const DevStatus* __restrict__ st, int64_t* __restrict__ info) {
  // a bounded device-side wait that ran out leaves the factor incomplete: reported instead of info
  info[0] = st->timeout ? (int64_t)GBLLT_ERR_TIMEOUT : st->fail_col >= 0 ? (int64_t)(st->fail_col + 1) : 0;
}

}  // namespace

template <typename T, typename TC>
void launch_potrf_diag(T* a, int64_t lda, int64_t k0, int bs, DevStatus* st, cudaStream_t s) {
  static const std::string kd = std::string("potrf_diag_") + tname<TC>();
  ProfScope ps(kd.c_str(), s, (double)bs * bs * bs / 3.0, (double)bs * (bs + 1) * sizeof(T));
  if (sizeof(TC) == 8) potrf_diag_f64_kernel<T><<<1, 512, 0, s>>>(a, lda, k0, bs, st);
  else potrf_diag_kernel<T, TC><<<1, 256, 0, s>>>(a, lda, k0, bs, st);
}

void launch_potrf_diag_f32s(float* a, int64_t lda, int64_t k0, int bs, DevStatus* st, cudaStream_t s, int64_t pk0,
                            int pk, float* linv) {
  static const std::string kd = "potrf_diag_f32";
  ProfScope ps(kd.c_str(), s, (double)bs * bs * bs / 3.0 + (double)bs * bs * pk,
               (double)bs * (bs + 1) * sizeof(float) + (double)bs * pk * sizeof(float));
  if (linv) {
    if (pk > 0) potrf_diag_f32s_kernel<true, true><<<1, DIAG_THREADS, 0, s>>>(a, lda, k0, bs, st, pk0, pk, linv);
    else potrf_diag_f32s_kernel<false, true><<<1, DIAG_THREADS, 0, s>>>(a, lda, k0, bs, st, 0, 0, linv);
  } else {
    if (pk > 0) potrf_diag_f32s_kernel<true, false><<<1, DIAG_THREADS, 0, s>>>(a, lda, k0, bs, st, pk0, pk, nullptr);
    else potrf_diag_f32s_kernel<false, false><<<1, DIAG_THREADS, 0, s>>>(a, lda, k0, bs, st, 0, 0, nullptr);
  }
}

template <typename T>
void launch_trsm_panel(T* a, int64_t lda, int64_t k0, int bs, int64_t rs, DevStatus* st, cudaStream_t s) {
  if (rs <= 0) return;
  static const std::string kt = std::string("trsm_panel_") + tname<T>();
  ProfScope ps(kt.c_str(), s, (double)rs * bs * bs, (2.0 * rs * bs + 0.5 * bs * bs) * sizeof(T));
  trsm_panel_kernel<T><<<(unsigned)ceil_div(rs, TRSM_ROWS), 128, 0, s>>>(a, lda, k0, bs, rs, st);
}

void launch_trsm_panel_tc(float* a, int64_t lda, int64_t k0, int bs, int64_t rs, DevStatus* st, const float* linv,
                          int tf32, int np, void* const* parts, cudaStream_t s) {
  if (rs <= 0) return;
  static const std::string kt = "trsm_panel_f32";
  ProfScope ps(kt.c_str(), s, (double)rs * bs * bs,
               (2.0 * rs * bs + 0.5 * bs * bs) * sizeof(float) + (double)rs * NB * np * (tf32 ? 4.0 : 2.0));
  const unsigned g = (unsigned)ceil_div(rs, TT_ROWS);
  void* p0 = np > 0 ? parts[0] : nullptr;
  void* p1 = np > 1 ? parts[1] : nullptr;
  void* p2 = np > 2 ? parts[2] : nullptr;
  if (np == 0) trsm_panel_tc_kernel<0><<<g, 128, 0, s>>>(a, lda, k0, bs, rs, st, linv, 0, p0, p1, p2);
  else if (tf32) trsm_panel_tc_kernel<2><<<g, 128, 0, s>>>(a, lda, k0, bs, rs, st, linv, np, p0, p1, p2);
  else trsm_panel_tc_kernel<1><<<g, 128, 0, s>>>(a, lda, k0, bs, rs, st, linv, np, p0, p1, p2);
}

template <typename T>
void launch_syrk_lower(T* a, int64_t lda, int64_t k0, int bs, int64_t rs, int64_t ncols, DevStatus* st,
                       cudaStream_t s, const T* bsrc, int64_t ldb) {
  if (rs <= 0 || ncols <= 0) return;
  static const std::string ks = std::string("syrk_lower_") + tname<T>();
  const int64_t mt = ceil_div(rs, 64);
  const int64_t nct = ceil_div(ncols < rs ? ncols : rs, 64);
  const int64_t tiles = nct >= mt ? mt * (mt + 1) / 2 : nct * mt - nct * (nct - 1) / 2;
  // algorithmic work: the updated lower entries, each a dot of depth bs (2 bs flops), reading the
  // bs-deep operand rows once and reading + writing each updated entry once
  const double w = (double)ncols;
  const double entries = ncols >= rs ? (double)rs * (rs + 1) / 2.0 : w * (double)rs - w * (w - 1) / 2.0;
  ProfScope ps(ks.c_str(), s, 2.0 * entries * bs, ((double)rs * bs + 2.0 * entries) * sizeof(T));
  syrk_lower_kernel<T><<<(unsigned)tiles, 256, 0, s>>>(a, lda, k0, bs, rs, ncols, (int)nct, st, bsrc, ldb);
}

// FP64 with the trailing updates on the tensor cores (OzakiSyrk): panels of kWide = 256 columns,
// each factored in 64-column steps (diagonal block, TRSM of the rows below, then the update of the
// panel's remaining columns by that 64-wide sub-panel), then one 256-deep update of the trailing
// matrix.  A 256-deep chunk is still exact in the tensor cores' FP32 accumulator, and a deeper
// update means four times fewer passes over the trailing matrix than 64-wide steps would make.
static int potrf_lower_tc(int64_t n, double* a, int64_t lda, DevStatus* st, cudaStream_t s, OzakiSyrk& oz) {
  for (int64_t K0 = 0; K0 < n; K0 += kWide) {
    const int pw = (int)(n - K0 < kWide ? n - K0 : kWide);
    for (int64_t k0 = K0; k0 < K0 + pw; k0 += NB) {
      const int bs = (int)(K0 + pw - k0 < NB ? K0 + pw - k0 : NB);
      const int64_t rs = n - k0 - bs;
      launch_potrf_diag<double, double>(a, lda, k0, bs, st, s);
      launch_trsm_panel<double>(a, lda, k0, bs, rs, st, s);
      const int64_t cols_left = K0 + pw - (k0 + bs);
      if (cols_left > 0 && rs > 0) {
        const int rc = oz.update(a, lda, k0, bs, rs, cols_left, st, s);
        if (rc) return rc;
      }
    }
    const int64_t rs2 = n - K0 - pw;
    if (rs2 > 0) {
      const int rc = oz.update(a, lda, K0, pw, rs2, rs2, st, s);
      if (rc) return rc;
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int potrf_lower_dev(int64_t n, T* d_a, int64_t lda, DevStatus* st, cudaStream_t s, bool may_allocate) {
  // FP64: trailing updates on the tensor cores, FP64-exact (error-free slicing; ozaki.cu), unless the
  // matrix is small or the workspace (about 5 n KB) cannot be allocated
  if constexpr (sizeof(T) == 8) {
    if (may_allocate && n >= kTensorSyrkMinN) {
      OzakiSyrk oz;
      const int rc = oz.init(n, s);
      if (rc == GBLLT_SUCCESS) return potrf_lower_tc(n, d_a, lda, st, s, oz);
      if (rc != GBLLT_ERR_ALLOC) return rc;
    }
  }
  for (int64_t k0 = 0; k0 < n; k0 += NB) {
    const int bs = (int)(n - k0 < NB ? n - k0 : NB);
    const int64_t rs = n - k0 - bs;
    launch_potrf_diag<T, T>(d_a, lda, k0, bs, st, s);
    launch_trsm_panel<T>(d_a, lda, k0, bs, rs, st, s);
    launch_syrk_lower<T>(d_a, lda, k0, bs, rs, rs, st, s);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template void launch_potrf_diag<float, double>(float*, int64_t, int64_t, int, DevStatus*, cudaStream_t);
template void launch_trsm_panel<float>(float*, int64_t, int64_t, int, int64_t, DevStatus*, cudaStream_t);
template void launch_syrk_lower<float>(float*, int64_t, int64_t, int, int64_t, int64_t, DevStatus*, cudaStream_t,
                                       const float*, int64_t);
template void launch_syrk_lower<double>(double*, int64_t, int64_t, int, int64_t, int64_t, DevStatus*, cudaStream_t,
                                        const double*, int64_t);

template <typename T>
int transpose_inplace_dev(int64_t n, T* d_a, int64_t lda, cudaStream_t s) {
  if (n <= 1) return GBLLT_SUCCESS;
  const int64_t nt = ceil_div(n, 32);
  transpose_inplace_kernel<T><<<(unsigned)(nt * (nt + 1) / 2), 256, 0, s>>>(d_a, lda, n);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int transpose_dev(int64_t rows, int64_t cols, const T* src, int64_t lds, T* dst, int64_t ldd, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return GBLLT_SUCCESS;
  dim3 grid((unsigned)ceil_div(rows, 32), (unsigned)ceil_div(cols, 32));
  transpose_kernel<T><<<grid, 256, 0, s>>>(rows, cols, src, lds, dst, ldd);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

int finalize_info_dev(const DevStatus* st, int64_t* d_info, cudaStream_t s) {
  finalize_info_kernel<<<1, 1, 0, s>>>(st, d_info);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template int potrf_lower_dev<double>(int64_t, double*, int64_t, DevStatus*, cudaStream_t, bool);
template int potrf_lower_dev<float>(int64_t, float*, int64_t, DevStatus*, cudaStream_t, bool);
template int transpose_inplace_dev<double>(int64_t, double*, int64_t, cudaStream_t);
template int transpose_inplace_dev<float>(int64_t, float*, int64_t, cudaStream_t);
template int transpose_dev<double>(int64_t, int64_t, const double*, int64_t, double*, int64_t, cudaStream_t);
template int transpose_dev<float>(int64_t, int64_t, const float*, int64_t, float*, int64_t, cudaStream_t);

}  // namespace gbllt
