// extern "C" entry points of libgbllt (declared in include/gbllt.h) for the plain-precision
// factor / solve, plus the library plumbing they share: per-thread streams, the error string
// and the device check.
#include <cstring>
#include <mutex>
#include <string>

#include <cstdlib>

#include "internal.h"

namespace gbllt {

namespace {
thread_local std::string g_last_error;
std::mutex g_dev_mutex;
int g_dev_ok[64];              // 0 = unchecked, 1 = ok, -1 = unusable
cudaMemPool_t g_pool[64] = {};  // the library's own stream-ordered pool per device (null: default pool)
}  // namespace

void set_last_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
  // a non-sticky error stays reported to the next caller of cudaGetLastError (another library in
  // the process) unless it is consumed here; it has been turned into our return code
  cudaGetLastError();
}

void set_error_message(const char* msg) { g_last_error = msg; }

static bool alloc_failure_injected() {
  const char* e = getenv("GBLLT_INJECT_ALLOC_FAILURE");
  return e && e[0] == '1';
}

cudaError_t dev_malloc_async(void** p, size_t bytes, cudaStream_t s) {
  if (alloc_failure_injected()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && g_pool[dev])
    return cudaMallocFromPoolAsync(p, bytes, g_pool[dev], s);
  return cudaMallocAsync(p, bytes, s);
}

cudaError_t dev_malloc(void** p, size_t bytes) {
  if (alloc_failure_injected()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

int ensure_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    g_last_error = "no CUDA device";
    return GBLLT_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= 64) return GBLLT_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if (g_dev_ok[dev] == 0) {
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    g_dev_ok[dev] = (major == 10 && minor == 3) ? 1 : -1;
    if (g_dev_ok[dev] > 0) {
      // The library's workspaces come from a stream-ordered pool of its own on each device, which
      // keeps freed memory cached in the process: a pool that returns it at every synchronisation
      // makes the next call map it again (gigabytes for a large solve).  The device's default pool,
      // which other code in the process may use, keeps its own settings.
      // gbllt_release_cached_memory() gives the cached memory back.  If the pool cannot be created,
      // allocations fall back to the default pool with its settings unchanged.
      cudaMemPoolProps props;
      memset(&props, 0, sizeof props);
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t pool = nullptr;
      if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        g_pool[dev] = pool;
      }
      cudaGetLastError();
    }
    if (g_dev_ok[dev] < 0) {
      char buf[128];
      snprintf(buf, sizeof buf, "device %d is sm_%d%d; this library is built for sm_103a only", dev, major, minor);
      g_last_error = buf;
    }
  }
  return g_dev_ok[dev] > 0 ? GBLLT_SUCCESS : GBLLT_ERR_NO_DEVICE;
}

cudaStream_t lib_stream() {
  thread_local cudaStream_t streams[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!streams[dev]) cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking);
  return streams[dev];
}

int check_uplo(char uplo) { return (uplo == 'L' || uplo == 'l' || uplo == 'U' || uplo == 'u') ? 0 : -1; }

namespace {

inline bool is_upper(char uplo) { return uplo == 'U' || uplo == 'u'; }

// Device memory taken from the stream-ordered pool and returned on scope exit.
struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
};

int alloc(DevBuf& b, size_t bytes, cudaStream_t s) {
  b.s = s;
  if (dev_malloc_async(&b.p, bytes < 256 ? 256 : bytes, s) != cudaSuccess) {
    cudaGetLastError();
    g_last_error = "cudaMallocAsync failed";
    b.p = nullptr;
    return GBLLT_ERR_ALLOC;
  }
  return GBLLT_SUCCESS;
}

int init_status(DevStatus* st, cudaStream_t s) {
  GB_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
  GB_CUDA_TRY(cudaMemsetAsync(&st->fail_col, 0xFF, sizeof(long long), s));
  return GBLLT_SUCCESS;
}

// Factor the `upper ? upper : lower` triangle of the column-major matrix at d_a in place.
template <typename T>
int factor_dev(bool upper, int64_t n, T* d_a, int64_t lda, DevStatus* st, int64_t* d_info, cudaStream_t s) {
  int rc;
  if ((rc = init_status(st, s))) return rc;
  if (upper && (rc = transpose_inplace_dev<T>(n, d_a, lda, s))) return rc;
  if ((rc = potrf_lower_dev<T>(n, d_a, lda, st, s))) return rc;
  if (upper && (rc = transpose_inplace_dev<T>(n, d_a, lda, s))) return rc;
  return finalize_info_dev(st, d_info, s);
}

template <typename T>
int dev_potrf(char uplo, int64_t n, T* d_a, int64_t lda, int64_t* d_info, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (n > 0 && !d_a) return -3;
  if (lda < (n > 1 ? n : 1)) return -4;
  if (!d_info) return -5;
  int rc = ensure_device();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    GB_CUDA_TRY(cudaMemsetAsync(d_info, 0, sizeof(int64_t), s));
    return GBLLT_SUCCESS;
  }
  DevBuf st;
  if ((rc = alloc(st, sizeof(DevStatus), s))) return rc;
  return factor_dev<T>(is_upper(uplo), n, d_a, lda, (DevStatus*)st.p, d_info, s);
}

template <typename T>
int dev_potrs(char uplo, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (n > 0 && !d_a) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (n > 0 && nrhs > 0 && !d_b) return -6;
  if (ldb < (n > 1 ? n : 1)) return -7;
  int rc = ensure_device();
  if (rc) return rc;
  return potrs_dev<T>(is_upper(uplo), n, nrhs, d_a, lda, d_b, ldb, (cudaStream_t)stream);
}

// Host-pointer entry points: stage to device, compute, copy back, synchronise.
template <typename T>
int host_posv(bool do_factor, bool do_solve, int layout, char uplo, int64_t n, int64_t nrhs, T* a, int64_t lda,
              T* b, int64_t ldb, int64_t* info) {
  const bool rowmajor = layout == GBLLT_ROW_MAJOR;
  const bool upper = is_upper(uplo) != rowmajor;  // a row-major lower factor is a column-major upper one
  cudaStream_t s = lib_stream();
  const size_t es = sizeof(T);
  const size_t abytes = (size_t)n * n * es;
  const size_t bbytes = do_solve ? (size_t)n * nrhs * es : 0;
  DevBuf work;
  // layout: [A | B | B^T | status | info], each part starting on a 256-byte boundary
  int rc = alloc(work, abytes + 2 * bbytes + 4 * 256 + 512, s);
  if (rc) return rc;
  char* base = (char*)work.p;
  T* d_a = (T*)base;
  T* d_b = (T*)(base + ((abytes + 255) / 256) * 256);
  T* d_bt = (T*)((char*)d_b + ((bbytes + 255) / 256) * 256);
  DevStatus* st = (DevStatus*)((char*)d_bt + ((bbytes + 255) / 256) * 256);
  int64_t* dinfo = (int64_t*)((char*)st + 256);  // the allocation reserves 2 x 256 B past d_bt

  // only the stored triangle is read (and written) on the device
  GB_CUDA_TRY(copy_triangle_async(upper, n, d_a, n, a, lda, es, cudaMemcpyHostToDevice, s));
  if (do_solve && nrhs > 0) {
    if (!rowmajor) {
      GB_CUDA_TRY(copy2d_async(d_b, n * es, b, ldb * es, n * es, nrhs, cudaMemcpyHostToDevice, s));
    } else {  // row-major B (n x nrhs, ldb >= nrhs) seen column-major is B^T (nrhs x n)
      GB_CUDA_TRY(copy2d_async(d_bt, nrhs * es, b, ldb * es, nrhs * es, n, cudaMemcpyHostToDevice, s));
      if ((rc = transpose_dev<T>(nrhs, n, d_bt, nrhs, d_b, n, s))) return rc;
    }
  }
  int64_t h_info = 0;
  if (do_factor) {
    if ((rc = factor_dev<T>(upper, n, d_a, n, st, dinfo, s))) return rc;
    GB_CUDA_TRY(copy_triangle_async(upper, n, a, lda, d_a, n, es, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaMemcpyAsync(&h_info, dinfo, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_info == GBLLT_ERR_TIMEOUT) return GBLLT_ERR_TIMEOUT;
    if (info) *info = h_info;
  }
  if (do_solve && nrhs > 0 && h_info == 0) {
    int herr = 0;
    if ((rc = potrs_dev<T>(upper, n, nrhs, d_a, n, d_b, n, s, &herr))) return rc;
    if (!rowmajor) {
      GB_CUDA_TRY(copy2d_async(b, ldb * es, d_b, n * es, n * es, nrhs, cudaMemcpyDeviceToHost, s));
    } else {
      if ((rc = transpose_dev<T>(n, nrhs, d_b, n, d_bt, nrhs, s))) return rc;
      GB_CUDA_TRY(copy2d_async(b, ldb * es, d_bt, nrhs * es, nrhs * es, n, cudaMemcpyDeviceToHost, s));
    }
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) {
      g_last_error = "a bounded wait of the triangular sweeps ran out";
      return GBLLT_ERR_TIMEOUT;
    }
  }
  return GBLLT_SUCCESS;
}

template <typename T>
int host_potrf(int layout, char uplo, int64_t n, T* a, int64_t lda, int64_t* info) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (n > 0 && !a) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (!info) return -6;
  *info = 0;
  if (n == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return host_posv<T>(true, false, layout, uplo, n, 0, a, lda, nullptr, 1, info);
}

template <typename T>
int host_potrs(int layout, char uplo, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (n > 0 && !a) return -5;
  if (lda < (n > 1 ? n : 1)) return -6;
  if (n > 0 && nrhs > 0 && !b) return -7;
  const int64_t minldb = layout == GBLLT_COL_MAJOR ? (n > 1 ? n : 1) : (nrhs > 1 ? nrhs : 1);
  if (ldb < minldb) return -8;
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return host_posv<T>(false, true, layout, uplo, n, nrhs, const_cast<T*>(a), lda, b, ldb, nullptr);
}

template <typename T>
int host_posv_entry(int layout, char uplo, int64_t n, int64_t nrhs, T* a, int64_t lda, T* b, int64_t ldb,
                    int64_t* info) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (n > 0 && !a) return -5;
  if (lda < (n > 1 ? n : 1)) return -6;
  if (n > 0 && nrhs > 0 && !b) return -7;
  const int64_t minldb = layout == GBLLT_COL_MAJOR ? (n > 1 ? n : 1) : (nrhs > 1 ? nrhs : 1);
  if (ldb < minldb) return -8;
  if (!info) return -9;
  *info = 0;
  if (n == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return host_posv<T>(true, true, layout, uplo, n, nrhs, a, lda, b, ldb, info);
}

int check_mixed_args(char uplo, int64_t n, int64_t nrhs, const void* a, int64_t lda, const void* b, int64_t ldb,
                     const void* x, int64_t ldx, int base) {
  // base = 0 for the _dev entry (uplo is argument 1), 1 for the host entry (layout first)
  if (check_uplo(uplo)) return -(1 + base);
  if (n < 0) return -(2 + base);
  if (nrhs < 0) return -(3 + base);
  if (n > 0 && !a) return -(4 + base);
  if (lda < (n > 1 ? n : 1)) return -(5 + base);
  if (n > 0 && nrhs > 0 && !b) return -(6 + base);
  if (ldb < (n > 1 ? n : 1)) return -(7 + base);
  if (n > 0 && nrhs > 0 && !x) return -(8 + base);
  if (ldx < (n > 1 ? n : 1)) return -(9 + base);
  return 0;
}

}  // namespace
}  // namespace gbllt

using namespace gbllt;

extern "C" int gbllt_dposv_mixed_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                     const double* d_b, int64_t ldb, double* d_x, int64_t ldx,
                                     const gbllt_mixed_opts* opts, gbllt_mixed_report* report, void* stream) {
  int rc = check_mixed_args(uplo, n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, 0);
  if (rc) return rc;
  if (report) memset(report, 0, sizeof *report);
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  if ((rc = ensure_device())) return rc;
  return posv_mixed_dev(is_upper(uplo), n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, opts, report, (cudaStream_t)stream);
}

extern "C" int gbllt_dposv_mixed(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda,
                                 const double* b, int64_t ldb, double* x, int64_t ldx, const gbllt_mixed_opts* opts,
                                 gbllt_mixed_report* report) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  const bool rowmajor = layout == GBLLT_ROW_MAJOR;
  // row-major B / X are n x nrhs with leading dimension >= nrhs
  const int64_t ldb_chk = rowmajor ? (ldb >= (nrhs > 1 ? nrhs : 1) ? (n > 1 ? n : 1) : 0) : ldb;
  const int64_t ldx_chk = rowmajor ? (ldx >= (nrhs > 1 ? nrhs : 1) ? (n > 1 ? n : 1) : 0) : ldx;
  int rc = check_mixed_args(uplo, n, nrhs, a, lda, b, ldb_chk, x, ldx_chk, 1);
  if (rc) return rc;
  if (report) memset(report, 0, sizeof *report);
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  if ((rc = ensure_device())) return rc;
  const bool upper = is_upper(uplo) != rowmajor;
  cudaStream_t s = lib_stream();
  const size_t es = 8;
  DevBuf work;
  const size_t abytes = ((size_t)n * n * es + 255) / 256 * 256, bbytes = ((size_t)n * nrhs * es + 255) / 256 * 256;
  if ((rc = alloc(work, abytes + 3 * bbytes, s))) return rc;
  double* d_a = (double*)work.p;
  double* d_b = (double*)((char*)work.p + abytes);
  double* d_x = (double*)((char*)d_b + bbytes);
  double* d_t = (double*)((char*)d_x + bbytes);
  // the solve reads only the stored triangle of A
  GB_CUDA_TRY(copy_triangle_async(upper, n, d_a, n, a, lda, es, cudaMemcpyHostToDevice, s));
  if (!rowmajor) {
    GB_CUDA_TRY(copy2d_async(d_b, n * es, b, ldb * es, n * es, nrhs, cudaMemcpyHostToDevice, s));
  } else {
    GB_CUDA_TRY(copy2d_async(d_t, nrhs * es, b, ldb * es, nrhs * es, n, cudaMemcpyHostToDevice, s));
    if ((rc = transpose_dev<double>(nrhs, n, d_t, nrhs, d_b, n, s))) return rc;
  }
  gbllt_mixed_report local;
  rc = posv_mixed_dev(upper, n, nrhs, d_a, n, d_b, n, d_x, n, opts, report ? report : &local, s);
  if (rc && rc != GBLLT_ERR_NOT_CONVERGED) return rc;
  if (!rowmajor) {
    GB_CUDA_TRY(copy2d_async(x, ldx * es, d_x, n * es, n * es, nrhs, cudaMemcpyDeviceToHost, s));
  } else {
    int rc2 = transpose_dev<double>(n, nrhs, d_x, n, d_t, nrhs, s);
    if (rc2) return rc2;
    GB_CUDA_TRY(copy2d_async(x, ldx * es, d_t, nrhs * es, nrhs * es, n, cudaMemcpyDeviceToHost, s));
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return rc;
}

extern "C" {

int gbllt_version(void) { return 100; }

const char* gbllt_last_error(void) { return g_last_error.c_str(); }

int gbllt_release_cached_memory(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return GBLLT_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= 64 || !g_pool[dev]) return GBLLT_SUCCESS;  // nothing cached by the library
  GB_CUDA_TRY(cudaDeviceSynchronize());
  GB_CUDA_TRY(cudaMemPoolTrimTo(g_pool[dev], 0));
  return GBLLT_SUCCESS;
}

int gbllt_selftest_wait_timeout(int64_t wait_us, int* observed) {
  if (wait_us < 1000 || wait_us > 2000000) return -1;
  if (!observed) return -2;
  *observed = GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return sweep_wait_selftest((unsigned long long)wait_us * 1000ull, lib_stream(), observed);
}

int gbllt_dpotrf(int layout, char uplo, int64_t n, double* a, int64_t lda, int64_t* info) {
  return host_potrf<double>(layout, uplo, n, a, lda, info);
}
int gbllt_spotrf(int layout, char uplo, int64_t n, float* a, int64_t lda, int64_t* info) {
  return host_potrf<float>(layout, uplo, n, a, lda, info);
}
int gbllt_dpotrs(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda, double* b,
                 int64_t ldb) {
  return host_potrs<double>(layout, uplo, n, nrhs, a, lda, b, ldb);
}
int gbllt_spotrs(int layout, char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda, float* b,
                 int64_t ldb) {
  return host_potrs<float>(layout, uplo, n, nrhs, a, lda, b, ldb);
}
int gbllt_dposv(int layout, char uplo, int64_t n, int64_t nrhs, double* a, int64_t lda, double* b, int64_t ldb,
                int64_t* info) {
  return host_posv_entry<double>(layout, uplo, n, nrhs, a, lda, b, ldb, info);
}
int gbllt_sposv(int layout, char uplo, int64_t n, int64_t nrhs, float* a, int64_t lda, float* b, int64_t ldb,
                int64_t* info) {
  return host_posv_entry<float>(layout, uplo, n, nrhs, a, lda, b, ldb, info);
}
int gbllt_dpotrf_dev(char uplo, int64_t n, double* d_a, int64_t lda, int64_t* d_info, void* stream) {
  return dev_potrf<double>(uplo, n, d_a, lda, d_info, stream);
}
int gbllt_spotrf_dev(char uplo, int64_t n, float* d_a, int64_t lda, int64_t* d_info, void* stream) {
  return dev_potrf<float>(uplo, n, d_a, lda, d_info, stream);
}
int gbllt_dpotrs_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda, double* d_b, int64_t ldb,
                     void* stream) {
  return dev_potrs<double>(uplo, n, nrhs, d_a, lda, d_b, ldb, stream);
}
int gbllt_spotrs_dev(char uplo, int64_t n, int64_t nrhs, const float* d_a, int64_t lda, float* d_b, int64_t ldb,
                     void* stream) {
  return dev_potrs<float>(uplo, n, nrhs, d_a, lda, d_b, ldb, stream);
}

}  // extern "C"
