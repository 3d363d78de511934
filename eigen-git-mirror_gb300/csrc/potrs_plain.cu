// Solve L L^T X = B (or U^T U X = B) from a Cholesky factor on the caller's stream: the
// stream-ordered allocating wrapper over the single-pass sweeps of potrs_lookback.cu, which need a
// small workspace (the inverted 64 x 64 diagonal triangles, ready flags and queue tickets).
#include "internal.h"

namespace gbllt {

namespace {

// FP64 with many right-hand sides: 256-row panels.  Each panel's triangle is solved by the look-back
// sweep (on its 256 x 256 diagonal block, four 64-row links) and the rest of the right-hand sides
// is updated by one FP64-exact product on the tensor cores (OzakiGemm), so the 2 n^2 k flops of the
// two sweeps leave the FP64 pipe:
//   forward,  L Y = B:    Y_J = L_JJ^-1 B_J,    then B_I -= L_IJ Y_J for the rows I below J;
//   backward, L^T X = Y:  X_J = L_JJ^-T Y_J,    then Y_K -= L_JK^T X_J for the rows K above J.
// (TriangularSolverMatrix.h:38-184 blocks the same way, with the panel products on gebp.)
constexpr int64_t kTensorSolveMinN = 2048;
constexpr int64_t kTensorSolveMinRhs = 16;
constexpr int kSolvePanel = 256;

int potrs_tc(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, double* b, int64_t ldb,
             cudaStream_t s, int* host_err) {
  const size_t sw = (potrs_ws_bytes(kSolvePanel, 8) + 255) & ~(size_t)255;
  const size_t gb = (OzakiGemm::bytes(n, nrhs, kSolvePanel) + 255) & ~(size_t)255;
  const size_t ib = (size_t)ceil_div(n, 64) * 64 * 64 * 8;  // the diagonal blocks' inverses
  char* ws = nullptr;
  if (dev_malloc_async((void**)&ws, sw + gb + 256 + ib, s) != cudaSuccess) {
    cudaGetLastError();
    return GBLLT_ERR_ALLOC;
  }
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{ws, s};
  OzakiGemm g;
  int rc = g.attach(ws + sw, n, nrhs, kSolvePanel);
  if (rc) return rc;
  int* err = (int*)(ws + sw + gb);  // every bounded wait of the solve reports here
  GB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  double* inv = (double*)(ws + sw + gb + 256);  // all 64 x 64 diagonal inverses, in one launch
  if ((rc = trinv_all<double>(upper, n, a, lda, inv, s))) return rc;
  // element (r, c) of L: a[c * lda + r] (lower storage) or a[r * lda + c] (upper storage of L^T)
  const int64_t lr = upper ? lda : 1, lc = upper ? 1 : lda;
  for (int64_t j0 = 0; j0 < n; j0 += kSolvePanel) {
    const int64_t jb = n - j0 < kSolvePanel ? n - j0 : kSolvePanel;
    if ((rc = trsm_sweep_ws<double>(upper, false, false, jb, nrhs, a + j0 * lda + j0, lda, b + j0, ldb, ws, s, err,
                                    inv + j0 * 64)))
      return rc;
    const int64_t below = n - j0 - jb;
    // B_I -= L_IJ Y_J: P = L_IJ (element (i, k) = L(j0 + jb + i, j0 + k)), Q = Y_J^T
    if (below > 0 && (rc = g.run(b + j0 + jb, ldb, below, nrhs, jb, a + (j0 + jb) * lr + j0 * lc, lr, lc, b + j0, ldb,
                                 1, 0, err, s)))
      return rc;
  }
  for (int64_t j0 = (n - 1) / kSolvePanel * kSolvePanel; j0 >= 0; j0 -= kSolvePanel) {
    const int64_t jb = n - j0 < kSolvePanel ? n - j0 : kSolvePanel;
    if ((rc = trsm_sweep_ws<double>(upper, true, false, jb, nrhs, a + j0 * lda + j0, lda, b + j0, ldb, ws, s, err,
                                    inv + j0 * 64)))
      return rc;
    // Y_K -= L_JK^T X_J: P = L_JK^T (element (k, i) = L(j0 + i, k)), Q = X_J^T
    if (j0 > 0 && (rc = g.run(b, ldb, j0, nrhs, jb, a + j0 * lr, lc, lr, b + j0, ldb, 1, 0, err, s))) return rc;
  }
  if (host_err) GB_CUDA_TRY(cudaMemcpyAsync(host_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace

template <typename T>
int potrs_dev(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb, cudaStream_t s,
              int* host_err) {
  if (host_err) *host_err = 0;
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
  if constexpr (sizeof(T) == 8) {
    if (n >= kTensorSolveMinN && nrhs >= kTensorSolveMinRhs) {
      const int rc = potrs_tc(upper, n, nrhs, d_a, lda, d_b, ldb, s, host_err);
      if (rc != GBLLT_ERR_ALLOC) return rc;
      // not enough memory for the slices: the sweeps below need far less
    }
  }
  void* ws = nullptr;
  if (dev_malloc_async((void**)&ws, potrs_ws_bytes(n, sizeof(T)), s) != cudaSuccess) {
    cudaGetLastError();
    return GBLLT_ERR_ALLOC;
  }
  int rc = potrs_ws<T>(upper, n, nrhs, d_a, lda, d_b, ldb, ws, s);
  if (!rc && host_err &&
      cudaMemcpyAsync(host_err, potrs_ws_error_word(n, sizeof(T), ws), sizeof(int), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess) {
    cudaGetLastError();
    rc = GBLLT_ERR_CUDA;
  }
  cudaFreeAsync(ws, s);
  return rc;
}

template int potrs_dev<double>(bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, cudaStream_t, int*);
template int potrs_dev<float>(bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, cudaStream_t, int*);

}  // namespace gbllt
