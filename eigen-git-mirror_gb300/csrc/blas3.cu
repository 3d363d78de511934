// BLAS level-3 routines of the Cholesky path on the GPU: SYRK and TRSM with every real
// uplo / trans / side / diag combination, the operations behind Eigen's Fortran BLAS
// dsyrk_/ssyrk_ (blas/level3_impl.h:355-417) and dtrsm_/strsm_ (blas/level3_impl.h:78-160).
//
//   SYRK  C = alpha op(A) op(A)^T + beta C on the `uplo` triangle of the n x n C; op(A) = A (n x k,
//         trans 'N') or A^T (A k x n, trans 'T'/'C').  syrk_kernel: one CTA per 64 x 64 tile of the
//         triangle, a 4 x 4 register block per thread over 32-deep shared-memory stages (the tiling of
//         the Cholesky's trailing update).  As in the reference, beta is applied first (beta = 0 clears
//         the triangle without reading it, beta = 1 leaves it) and alpha multiplies the product.
//   TRSM  B = alpha op(A)^{-1} B (side 'L', A m x m) or alpha B op(A)^{-1} (side 'R', A n x n), A
//         triangular with a unit or stored diagonal.  The solve is one single-pass look-back sweep
//         (potrs_lookback.cu) on the right-hand sides; the right-side case transposes B, solves with
//         op(A)^T and transposes back.  As in the reference, the solve comes first and alpha scales
//         the result.
#include "internal.h"

namespace gbllt {

namespace {

constexpr int KC = 32;

// C tile (64 x 64) of the `UP ? upper : lower` triangle; op(A)(r, p) = TRANS ? A(p, r) : A(r, p).
template <typename T, bool UP, bool TRANS>
__global__ void __launch_bounds__(256) syrk_kernel(long long n, long long k, T alpha, const T* __restrict__ a,
                                                   long long lda, T beta, T* __restrict__ c, long long ldc) {
  __shared__ T As[KC][64 + 1];
  __shared__ T Bs[KC][64 + 1];
  int ti, tj;
  lower_tile_coords(blockIdx.x, ti, tj);  // ti >= tj
  const long long i0 = (long long)(UP ? tj : ti) * 64, j0 = (long long)(UP ? ti : tj) * 64;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[m][q] = T(0);
  for (long long p0 = 0; p0 < k; p0 += KC) {
    for (int idx = tid; idx < 64 * KC; idx += 256) {
      int r, p;
      if (TRANS) { p = idx % KC; r = idx / KC; }  // A(p, r): consecutive p are contiguous
      else       { r = idx & 63; p = idx >> 6; }  // A(r, p): consecutive r are contiguous
      const long long pp = p0 + p;
      T va = T(0), vb = T(0);
      if (pp < k) {
        if (i0 + r < n) va = TRANS ? a[(i0 + r) * lda + pp] : a[pp * lda + i0 + r];
        if (j0 + r < n) vb = TRANS ? a[(j0 + r) * lda + pp] : a[pp * lda + j0 + r];
      }
      As[p][r] = va;
      Bs[p][r] = vb;
    }
    __syncthreads();
    const int pe = k - p0 < KC ? (int)(k - p0) : KC;
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
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const long long j = j0 + ty + 16 * q;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const long long i = i0 + tx + 16 * m;
      if (i < n && j < n && (UP ? i <= j : i >= j)) {
        T* cij = c + j * ldc + i;
        const T base = beta == T(0) ? T(0) : (beta == T(1) ? *cij : beta * *cij);
        *cij = base + alpha * acc[m][q];
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) scale_kernel(long long m, long long n, T alpha, T* __restrict__ b,
                                                    long long ldb) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= m) return;
  for (long long j = blockIdx.y; j < n; j += gridDim.y) b[j * ldb + i] *= alpha;
}

struct Scratch {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
  int get(size_t bytes, cudaStream_t st) {
    s = st;
    if (dev_malloc_async(&p, bytes < 256 ? 256 : bytes, st) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error_message("cudaMallocAsync failed");
      return GBLLT_ERR_ALLOC;
    }
    return GBLLT_SUCCESS;
  }
};

inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }
inline bool is_trans(char t) { return t == 'T' || t == 't' || t == 'C' || t == 'c'; }
inline bool valid_trans(char t) { return t == 'N' || t == 'n' || is_trans(t); }
inline bool is_up(char u) { return u == 'U' || u == 'u'; }
inline bool valid_side(char c) { return c == 'L' || c == 'l' || c == 'R' || c == 'r'; }
inline bool valid_diag(char c) { return c == 'N' || c == 'n' || c == 'U' || c == 'u'; }
inline int64_t max1(int64_t v) { return v > 1 ? v : 1; }

template <typename T>
int syrk_dev(bool upper, bool trans, int64_t n, int64_t k, T alpha, const T* a, int64_t lda, T beta, T* c,
             int64_t ldc, cudaStream_t s) {
  if (n == 0) return GBLLT_SUCCESS;
  static const std::string kn = std::string("syrk_") + tname<T>();
  const int64_t t = ceil_div(n, 64);
  const unsigned tiles = (unsigned)(t * (t + 1) / 2);
  const double entries = (double)n * (n + 1) / 2.0;
  ProfScope ps(kn.c_str(), s, 2.0 * entries * k, ((double)n * k + 2.0 * entries) * sizeof(T));
  if (upper) {
    if (trans) syrk_kernel<T, true, true><<<tiles, 256, 0, s>>>(n, k, alpha, a, lda, beta, c, ldc);
    else syrk_kernel<T, true, false><<<tiles, 256, 0, s>>>(n, k, alpha, a, lda, beta, c, ldc);
  } else {
    if (trans) syrk_kernel<T, false, true><<<tiles, 256, 0, s>>>(n, k, alpha, a, lda, beta, c, ldc);
    else syrk_kernel<T, false, false><<<tiles, 256, 0, s>>>(n, k, alpha, a, lda, beta, c, ldc);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

// op(A) X = B for an m x m triangular A and n right-hand sides, in place in B.  The sweep solves
// L X = B or L^T X = B for L lower; an upper A is L^T with L stored transposed, so U X = B is the
// backward sweep and U^T X = B the forward one.
template <typename T>
int trsm_left(bool upper, bool trans, bool unit, int64_t m, int64_t n, const T* a, int64_t lda, T* b, int64_t ldb,
              cudaStream_t s) {
  Scratch ws;
  int rc = ws.get(potrs_ws_bytes(m, sizeof(T)), s);
  if (rc) return rc;
  return trsm_sweep_ws<T>(upper, upper != trans, unit, m, n, a, lda, b, ldb, ws.p, s);
}

template <typename T>
int trsm_dev(bool left, bool upper, bool trans, bool unit, int64_t m, int64_t n, T alpha, const T* a, int64_t lda,
             T* b, int64_t ldb, cudaStream_t s) {
  if (m == 0 || n == 0) return GBLLT_SUCCESS;
  int rc;
  if (left) {
    if ((rc = trsm_left<T>(upper, trans, unit, m, n, a, lda, b, ldb, s))) return rc;
  } else {  // X op(A) = B  <=>  op(A)^T X^T = B^T, A n x n
    Scratch tmp;
    if ((rc = tmp.get((size_t)n * m * sizeof(T), s))) return rc;
    T* bt = (T*)tmp.p;  // n x m, leading dimension n
    if ((rc = transpose_dev<T>(m, n, b, ldb, bt, n, s))) return rc;
    if ((rc = trsm_left<T>(upper, !trans, unit, n, m, a, lda, bt, n, s))) return rc;
    if ((rc = transpose_dev<T>(n, m, bt, n, b, ldb, s))) return rc;
  }
  if (alpha != T(1)) {
    const dim3 grid((unsigned)ceil_div(m, 256), (unsigned)(n < 1024 ? n : 1024));
    scale_kernel<T><<<grid, 256, 0, s>>>(m, n, alpha, b, ldb);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

// ---- argument checks (blas/level3_impl.h:381-388 syrk, :136-146 trsm), base = 1 with a layout ----

int syrk_args(char uplo, char trans, int64_t n, int64_t k, const void* a, int64_t lda, const void* c, int64_t ldc,
              int base) {
  if (check_uplo(uplo)) return -(1 + base);
  if (!valid_trans(trans)) return -(2 + base);
  if (n < 0) return -(3 + base);
  if (k < 0) return -(4 + base);
  if (n > 0 && k > 0 && !a) return -(6 + base);
  if (lda < max1(is_trans(trans) ? k : n)) return -(7 + base);
  if (n > 0 && !c) return -(9 + base);
  if (ldc < max1(n)) return -(10 + base);
  return 0;
}

int trsm_args(char side, char uplo, char transa, char diag, int64_t m, int64_t n, const void* a, int64_t lda,
              const void* b, int64_t ldb, int base) {
  if (!valid_side(side)) return -(1 + base);
  if (check_uplo(uplo)) return -(2 + base);
  if (!valid_trans(transa)) return -(3 + base);
  if (!valid_diag(diag)) return -(4 + base);
  if (m < 0) return -(5 + base);
  if (n < 0) return -(6 + base);
  const bool left = side == 'L' || side == 'l';
  if (m > 0 && n > 0 && !a) return -(8 + base);
  if (lda < max1(left ? m : n)) return -(9 + base);
  if (m > 0 && n > 0 && !b) return -(10 + base);
  if (ldb < max1(m)) return -(11 + base);
  return 0;
}

template <typename T>
int host_syrk(int layout, char uplo, char trans, int64_t n, int64_t k, T alpha, const T* a, int64_t lda, T beta,
              T* c, int64_t ldc) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  const bool rm = layout == GBLLT_ROW_MAJOR;
  // a row-major C is C^T column-major (the other triangle of the same symmetric result), and a
  // row-major A is A^T column-major (the other op): its leading dimension is checked as such
  const char tchk = (rm && valid_trans(trans)) ? (is_trans(trans) ? 'N' : 'T') : trans;
  int rc = syrk_args(uplo, tchk, n, k, a, lda, c, ldc, 1);
  if (rc) return rc;
  if (n == 0) return GBLLT_SUCCESS;
  if ((rc = ensure_device())) return rc;
  const bool upper = is_up(uplo) != rm, tr = is_trans(trans) != rm;
  const int64_t ar = tr ? k : n, ac = tr ? n : k;  // column-major A as seen by the kernel: ar x ac
  cudaStream_t s = lib_stream();
  const size_t es = sizeof(T);
  const size_t ab = up256((size_t)ar * ac * es);
  Scratch buf;
  if ((rc = buf.get(ab + (size_t)n * n * es, s))) return rc;
  T* d_a = (T*)buf.p;
  T* d_c = (T*)((char*)buf.p + ab);
  if (ar > 0 && ac > 0)
    GB_CUDA_TRY(copy2d_async(d_a, ar * es, a, lda * es, ar * es, ac, cudaMemcpyHostToDevice, s));
  // all of C goes up and comes back, so that the triangle the kernel does not touch is returned as
  // it was (with beta = 0 the kernel does not read the updated triangle)
  GB_CUDA_TRY(copy2d_async(d_c, n * es, c, ldc * es, n * es, n, cudaMemcpyHostToDevice, s));
  if ((rc = syrk_dev<T>(upper, tr, n, k, alpha, d_a, max1(ar), beta, d_c, n, s))) return rc;
  GB_CUDA_TRY(copy2d_async(c, ldc * es, d_c, n * es, n * es, n, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBLLT_SUCCESS;
}

template <typename T>
int dev_syrk(char uplo, char trans, int64_t n, int64_t k, T alpha, const T* a, int64_t lda, T beta, T* c,
             int64_t ldc, void* stream) {
  int rc = syrk_args(uplo, trans, n, k, a, lda, c, ldc, 0);
  if (rc) return rc;
  if (n == 0) return GBLLT_SUCCESS;
  if ((rc = ensure_device())) return rc;
  return syrk_dev<T>(is_up(uplo), is_trans(trans), n, k, alpha, a, lda, beta, c, ldc, (cudaStream_t)stream);
}

template <typename T>
int host_trsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n, T alpha, const T* a,
              int64_t lda, T* b, int64_t ldb) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  const bool rm = layout == GBLLT_ROW_MAJOR;
  // row-major B (m x n, ldb >= n) is B^T column-major: the other side, the other triangle of the
  // same A, the same op, m and n exchanged
  int rc = rm ? trsm_args(side, uplo, transa, diag, m, n, a, lda, b, ldb >= max1(n) ? max1(m) : 0, 1)
              : trsm_args(side, uplo, transa, diag, m, n, a, lda, b, ldb, 1);
  if (rc) return rc;
  if (m == 0 || n == 0) return GBLLT_SUCCESS;
  if ((rc = ensure_device())) return rc;
  bool left = side == 'L' || side == 'l';
  const int64_t na = left ? m : n;  // order of A
  bool upper = is_up(uplo);
  int64_t mm = m, nn = n;
  if (rm) {
    left = !left;
    upper = !upper;
    mm = n;
    nn = m;
  }
  cudaStream_t s = lib_stream();
  const size_t es = sizeof(T);
  const size_t ab = up256((size_t)na * na * es);
  Scratch buf;
  if ((rc = buf.get(ab + (size_t)mm * nn * es, s))) return rc;
  T* d_a = (T*)buf.p;
  T* d_b = (T*)((char*)buf.p + ab);
  GB_CUDA_TRY(copy2d_async(d_a, na * es, a, lda * es, na * es, na, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(copy2d_async(d_b, mm * es, b, ldb * es, mm * es, nn, cudaMemcpyHostToDevice, s));
  if ((rc = trsm_dev<T>(left, upper, is_trans(transa), diag == 'U' || diag == 'u', mm, nn, alpha, d_a, na, d_b, mm,
                        s)))
    return rc;
  GB_CUDA_TRY(copy2d_async(b, ldb * es, d_b, mm * es, mm * es, nn, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBLLT_SUCCESS;
}

template <typename T>
int dev_trsm(char side, char uplo, char transa, char diag, int64_t m, int64_t n, T alpha, const T* a, int64_t lda,
             T* b, int64_t ldb, void* stream) {
  int rc = trsm_args(side, uplo, transa, diag, m, n, a, lda, b, ldb, 0);
  if (rc) return rc;
  if (m == 0 || n == 0) return GBLLT_SUCCESS;
  if ((rc = ensure_device())) return rc;
  return trsm_dev<T>(side == 'L' || side == 'l', is_up(uplo), is_trans(transa), diag == 'U' || diag == 'u', m, n,
                     alpha, a, lda, b, ldb, (cudaStream_t)stream);
}

}  // namespace
}  // namespace gbllt

using namespace gbllt;

extern "C" {

int gbllt_dsyrk(int layout, char uplo, char trans, int64_t n, int64_t k, double alpha, const double* a, int64_t lda,
                double beta, double* c, int64_t ldc) {
  return host_syrk<double>(layout, uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
}
int gbllt_ssyrk(int layout, char uplo, char trans, int64_t n, int64_t k, float alpha, const float* a, int64_t lda,
                float beta, float* c, int64_t ldc) {
  return host_syrk<float>(layout, uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
}
int gbllt_dsyrk_dev(char uplo, char trans, int64_t n, int64_t k, double alpha, const double* d_a, int64_t lda,
                    double beta, double* d_c, int64_t ldc, void* stream) {
  return dev_syrk<double>(uplo, trans, n, k, alpha, d_a, lda, beta, d_c, ldc, stream);
}
int gbllt_ssyrk_dev(char uplo, char trans, int64_t n, int64_t k, float alpha, const float* d_a, int64_t lda,
                    float beta, float* d_c, int64_t ldc, void* stream) {
  return dev_syrk<float>(uplo, trans, n, k, alpha, d_a, lda, beta, d_c, ldc, stream);
}
int gbllt_dtrsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
                const double* a, int64_t lda, double* b, int64_t ldb) {
  return host_trsm<double>(layout, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}
int gbllt_strsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n, float alpha,
                const float* a, int64_t lda, float* b, int64_t ldb) {
  return host_trsm<float>(layout, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}
int gbllt_dtrsm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
                    const double* d_a, int64_t lda, double* d_b, int64_t ldb, void* stream) {
  return dev_trsm<double>(side, uplo, transa, diag, m, n, alpha, d_a, lda, d_b, ldb, stream);
}
int gbllt_strsm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n, float alpha,
                    const float* d_a, int64_t lda, float* d_b, int64_t ldb, void* stream) {
  return dev_trsm<float>(side, uplo, transa, diag, m, n, alpha, d_a, lda, d_b, ldb, stream);
}

}  // extern "C"
