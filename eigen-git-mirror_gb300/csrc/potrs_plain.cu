// Two-sweep triangular solve from a Cholesky factor (LLT::_solve_impl_transposed,
// Eigen/src/Cholesky/LLT.h:490-498): forward sweep L Y = B, then backward sweep L^T X = Y.
//
// Both sweeps are blocked by 64 rows.  For block j:
//   trsv_diag_kernel    solves the 64 x 64 triangle against the 64 x nrhs block of B, one thread
//                       per right-hand side with its 64 values in registers (the in-panel
//                       substitution of TriangularSolverVector.h:88-142 / TriangularSolverMatrix.h:116-146);
//   solve_update_kernel applies the block to the remaining rows of B, a GEMM of depth 64
//                       (the GEMV/GEPP part, TriangularSolverVector.h:134-138,
//                       TriangularSolverMatrix.h:162-182).  The 64 x 64 tile of L is staged in
//                       shared memory with loads that are coalesced for either storage of L.
//
// The factor may be stored lower (element L(i,j) at a[i + j*lda]) or upper (U = L^T,
// L(i,j) at a[j + i*lda]); the template flag UP selects the addressing, so no copy is made.
#include "internal.h"

namespace gbllt {

namespace {

constexpr int SB = 64;   // block height
constexpr int RC = 16;   // right-hand sides per CTA in the update kernel

template <typename T, bool UP>
__device__ __forceinline__ T lget(const T* __restrict__ a, long long lda, long long i, long long j) {
  return UP ? a[i * lda + j] : a[j * lda + i];
}

// BWD == false: Y_j = L_jj^{-1} B_j ; BWD == true: X_j = L_jj^{-T} Y_j.  One thread per RHS.
template <typename T, bool UP, bool BWD>
__global__ void __launch_bounds__(128) trsv_diag_kernel(const T* __restrict__ a, long long lda, long long j0, int bs,
                                                        T* __restrict__ b, long long ldb, long long nrhs) {
  __shared__ T L[SB][SB + 1];  // L[i][p] = L(j0+i, j0+p), identity padding
  for (int idx = threadIdx.x; idx < SB * SB; idx += 128) {
    int i, p;
    if (UP) { p = idx % SB; i = idx / SB; }   // U stored: contiguous along p for fixed i
    else    { i = idx % SB; p = idx / SB; }
    T v = (i == p) ? T(1) : T(0);
    if (i < bs && p < bs && i >= p) v = lget<T, UP>(a, lda, j0 + i, j0 + p);
    L[i][p] = v;
  }
  __syncthreads();
  const long long c = (long long)blockIdx.x * 128 + threadIdx.x;
  if (c >= nrhs) return;
  T* col = b + c * ldb + j0;
  T x[SB];
#pragma unroll
  for (int i = 0; i < SB; ++i) x[i] = i < bs ? col[i] : T(0);
  if (!BWD) {
#pragma unroll
    for (int i = 0; i < SB; ++i) {
      T v = x[i];
#pragma unroll
      for (int p = 0; p < i; ++p) v = fma(-L[i][p], x[p], v);
      x[i] = v / L[i][i];
    }
  } else {
#pragma unroll
    for (int i = SB - 1; i >= 0; --i) {
      T v = x[i];
#pragma unroll
      for (int p = i + 1; p < SB; ++p) v = fma(-L[p][i], x[p], v);
      x[i] = v / L[i][i];
    }
  }
#pragma unroll
  for (int i = 0; i < SB; ++i)
    if (i < bs) col[i] = x[i];
}

// Forward (BWD == false): B(r0+r, c) -= sum_p L(r0+r, j0+p) * B(j0+p, c), rows r0+r in [row_lo, row_hi).
// Backward (BWD == true): B(r0+r, c) -= sum_p L(j0+p, r0+r) * B(j0+p, c), rows in [row_lo, row_hi).
template <typename T, bool UP, bool BWD>
__global__ void __launch_bounds__(256) solve_update_kernel(const T* __restrict__ a, long long lda, long long j0, int bs,
                                                           long long row_lo, long long row_hi, T* __restrict__ b,
                                                           long long ldb, long long nrhs) {
  __shared__ T Ls[SB][SB + 1];  // Ls[p][r]
  __shared__ T Ys[SB][RC + 1];  // Ys[p][c]
  const long long r0 = row_lo + (long long)blockIdx.x * SB;
  const long long c0 = (long long)blockIdx.y * RC;
  const int tid = threadIdx.x;
  // element (r, p) of the tile: matrix entry L(r0+r, j0+p) (forward) or L(j0+p, r0+r) (backward).
  // Storage of that entry is contiguous along r when (forward, lower) or (backward, upper), else along p.
  constexpr bool r_fast = (!BWD && !UP) || (BWD && UP);
  for (int idx = tid; idx < SB * SB; idx += 256) {
    int r, p;
    if (r_fast) { r = idx % SB; p = idx / SB; }
    else        { p = idx % SB; r = idx / SB; }
    T v = T(0);
    if (p < bs && r0 + r < row_hi)
      v = BWD ? lget<T, UP>(a, lda, j0 + p, r0 + r) : lget<T, UP>(a, lda, r0 + r, j0 + p);
    Ls[p][r] = v;
  }
  for (int idx = tid; idx < SB * RC; idx += 256) {
    const int p = idx % SB, c = idx / SB;
    Ys[p][c] = (p < bs && c0 + c < nrhs) ? b[(c0 + c) * ldb + j0 + p] : T(0);
  }
  __syncthreads();
  const int r = tid & 63, cq = tid >> 6;  // 4 groups of 4 right-hand sides
  T acc[4] = {T(0), T(0), T(0), T(0)};
  for (int p = 0; p < bs; ++p) {
    const T l = Ls[p][r];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = fma(l, Ys[p][cq * 4 + q], acc[q]);
  }
  const long long row = r0 + r;
  if (row < row_hi) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long c = c0 + cq * 4 + q;
      if (c < nrhs) b[c * ldb + row] -= acc[q];
    }
  }
}

template <typename T, bool UP>
int potrs_impl(int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, cudaStream_t s) {
  static const std::string kd = std::string("trsv_diag_") + tname<T>();
  static const std::string ku = std::string("solve_update_") + tname<T>();
  const double es = sizeof(T);
  const unsigned dgrid = (unsigned)ceil_div(nrhs, 128);
  const unsigned ygrid = (unsigned)ceil_div(nrhs, RC);
  auto diag = [&](int64_t j0, int bs, bool bwd) {
    ProfScope ps(kd.c_str(), s, (double)bs * bs * nrhs, (2.0 * bs * nrhs + 0.5 * bs * bs) * es);
    if (bwd) trsv_diag_kernel<T, UP, true><<<dgrid, 128, 0, s>>>(a, lda, j0, bs, b, ldb, nrhs);
    else     trsv_diag_kernel<T, UP, false><<<dgrid, 128, 0, s>>>(a, lda, j0, bs, b, ldb, nrhs);
  };
  auto update = [&](int64_t j0, int bs, int64_t lo, int64_t hi, bool bwd) {
    // algorithmic work: a (hi-lo) x bs block of L against bs x nrhs, read L once, read+write B rows
    ProfScope ps(ku.c_str(), s, 2.0 * (hi - lo) * bs * nrhs, ((double)(hi - lo) * bs + 2.0 * (hi - lo) * nrhs) * es);
    dim3 grid((unsigned)ceil_div(hi - lo, SB), ygrid);
    if (bwd) solve_update_kernel<T, UP, true><<<grid, 256, 0, s>>>(a, lda, j0, bs, lo, hi, b, ldb, nrhs);
    else     solve_update_kernel<T, UP, false><<<grid, 256, 0, s>>>(a, lda, j0, bs, lo, hi, b, ldb, nrhs);
  };
  for (int64_t j0 = 0; j0 < n; j0 += SB) {  // L Y = B
    const int bs = (int)(n - j0 < SB ? n - j0 : SB);
    diag(j0, bs, false);
    if (n > j0 + bs) update(j0, bs, j0 + bs, n, false);
  }
  const int64_t last = ((n - 1) / SB) * SB;
  for (int64_t j0 = last; j0 >= 0; j0 -= SB) {  // L^T X = Y
    const int bs = (int)(n - j0 < SB ? n - j0 : SB);
    diag(j0, bs, true);
    if (j0 > 0) update(j0, bs, 0, j0, true);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace

template <typename T>
int potrs_dev(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
  return upper ? potrs_impl<T, true>(n, nrhs, d_a, lda, d_b, ldb, s)
               : potrs_impl<T, false>(n, nrhs, d_a, lda, d_b, ldb, s);
}

template int potrs_dev<double>(bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, cudaStream_t);
template int potrs_dev<float>(bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, cudaStream_t);

}  // namespace gbllt
