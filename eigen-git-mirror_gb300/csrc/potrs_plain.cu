// Solve L L^T X = B (or U^T U X = B) from a Cholesky factor on the caller's stream: the
// stream-ordered allocating wrapper over the single-pass sweeps of potrs_lookback.cu, which need a
// small workspace (the inverted 64 x 64 diagonal triangles, ready flags and queue tickets).
#include "internal.h"

namespace gbllt {

template <typename T>
int potrs_dev(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb, cudaStream_t s,
              int* host_err) {
  if (host_err) *host_err = 0;
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
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
