// Reciprocal condition number of an SPD matrix from its Cholesky factor, on the device.
//
// LLT::rcond() (Eigen/src/Cholesky/LLT.h:166-171) combines two pieces:
//   - m_l1_norm, the 1-norm of the symmetric input, which LLT::compute takes from one stored
//     triangle with a host loop over columns (LLT.h:443-453);
//   - rcond_estimate_helper / rcond_invmatrix_L1_norm_estimate (Eigen/src/Core/ConditionEstimator.h:
//     56-171): Hager's 1-norm estimate of A^{-1} with Higham's refinements (Higham, "FORTRAN codes
//     for estimating the one-norm of a real or complex matrix", 1988, Algorithms 4.1 and 5.1),
//     driven by at most 11 solves with the factor.
// Here the factor stays in device memory for every solve (potrs_ws, the single-pass sweeps), and
// the vector work between solves (signs, first index of max |v|, 1-norms, unit and alternating
// vectors) runs in small kernels; the host only reads the scalars that steer the iteration.  The
// iteration, its stopping tests and its quirks (the estimate that failed to increase is still the
// one compared with the alternating-sign bound) follow ConditionEstimator.h:79-150 step by step.
#include <cmath>
#include <limits>

#include "internal.h"

namespace gbllt {

namespace {

constexpr int CB = 32;  // columns (and rows) per block of the norm kernel

// cs[j] = sum_i |A(i, j)| of the symmetric A stored in the `UP ? upper : lower` triangle of the
// column-major array a.  Block b owns columns/rows [b*CB, b*CB + CB):
//   column part: the stored entries of column j (contiguous), one warp per column;
//   row part:    the stored entries of row j that belong to column j by symmetry, read as
//                32-row strips (lane = row) that are contiguous in memory.
// Each sum is formed in a fixed order, so the result is deterministic.
template <typename T, bool UP>
__global__ void __launch_bounds__(256) sym_abs_colsum_kernel(long long n, const T* __restrict__ a, long long lda,
                                                             double* __restrict__ cs) {
  __shared__ double part[8][CB];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long c0 = (long long)blockIdx.x * CB;
  // row part: lane = row c0 + lane; warps split the columns of the other triangle
  const long long r = c0 + lane;
  double rs = 0.0;
  if (r < n) {
    if (!UP) {  // row r of the lower triangle left of the diagonal: A(r, j), j < r
      for (long long j = warp; j < r; j += 8) rs += fabs((double)a[j * lda + r]);
    } else {    // row r of the upper triangle right of the diagonal: A(r, j), j > r
      for (long long j = c0 + warp; j < n; j += 8)
        if (j > r) rs += fabs((double)a[j * lda + r]);
    }
  }
  part[warp][lane] = rs;
  __syncthreads();
  // column part: warp w sums the stored entries of columns c0 + w, c0 + w + 8, ...
  for (int cc = warp; cc < CB; cc += 8) {
    const long long j = c0 + cc;
    if (j >= n) break;
    double s = 0.0;
    const long long i0 = UP ? 0 : j, i1 = UP ? j + 1 : n;
    for (long long i = i0 + lane; i < i1; i += 32) s += fabs((double)a[j * lda + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      double t = s;
      for (int w = 0; w < 8; ++w) t += part[w][cc];
      cs[j] = t;
    }
  }
}

// out[0] = max_j cs[j]  (one block)
__global__ void __launch_bounds__(1024) max_kernel(long long n, const double* __restrict__ cs, double* __restrict__ out) {
  __shared__ double m[1024];
  double v = 0.0;
  for (long long j = threadIdx.x; j < n; j += 1024) v = fmax(v, cs[j]);
  m[threadIdx.x] = v;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) m[threadIdx.x] = fmax(m[threadIdx.x], m[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = m[0];
}

template <typename T>
__global__ void to_type_kernel(const double* __restrict__ in, T* __restrict__ out) {
  out[0] = (T)in[0];
}

// ---- vector kernels of the estimator (one block of 1024 threads for the reductions) --------------

// 1-norm of v (fixed-order tree) -> res[0]
template <typename T>
__global__ void __launch_bounds__(1024) l1_kernel(long long n, const T* __restrict__ v, double* __restrict__ res) {
  __shared__ double m[1024];
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += 1024) s += fabs((double)v[i]);
  m[threadIdx.x] = s;
  __syncthreads();
  for (int k = 512; k > 0; k >>= 1) {
    if (threadIdx.x < k) m[threadIdx.x] += m[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) res[0] = m[0];
}

// first index of max |v| (the first maximum wins, as in DenseBase::maxCoeff(&index)) -> idx[0]
template <typename T>
__global__ void __launch_bounds__(1024) argmax_abs_kernel(long long n, const T* __restrict__ v, long long* __restrict__ idx) {
  __shared__ double mv[1024];
  __shared__ long long mi[1024];
  double best = -1.0;
  long long bi = -1;
  for (long long i = threadIdx.x; i < n; i += 1024) {
    const double x = fabs((double)v[i]);
    if (x > best) { best = x; bi = i; }
  }
  mv[threadIdx.x] = best;
  mi[threadIdx.x] = bi;
  __syncthreads();
  for (int k = 512; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      const double o = mv[threadIdx.x + k];
      const long long oi = mi[threadIdx.x + k];
      if (oi >= 0 && (o > mv[threadIdx.x] || (o == mv[threadIdx.x] && (mi[threadIdx.x] < 0 || oi < mi[threadIdx.x])))) {
        mv[threadIdx.x] = o;
        mi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) idx[0] = mi[0] < 0 ? 0 : mi[0];
}

// sign[i] = v[i] < 0 ? -1 : 1 (ConditionEstimator.h:29-35); *differs |= (sign != old) anywhere
template <typename T>
__global__ void sign_kernel(long long n, const T* __restrict__ v, T* __restrict__ sign, const T* __restrict__ old,
                            int* __restrict__ differs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T sv = v[i] < T(0) ? T(-1) : T(1);
  sign[i] = sv;
  if (old && sv != old[i]) *differs = 1;
}

// kind 0: v = 1/n everywhere; 1: v = e_j; 2: v_i = (-1)^i (1 + i/(n-1))   (arithmetic in T)
template <typename T>
__global__ void fill_kernel(long long n, T* __restrict__ v, int kind, const long long* __restrict__ j) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T x;
  if (kind == 0) x = T(1) / T(n);
  else if (kind == 1) x = (i == *j) ? T(1) : T(0);
  else x = ((i & 1) ? T(-1) : T(1)) * (T(1) + T(i) / T(n - 1));
  v[i] = x;
}

template <typename T>
int sym_l1_norm_into(bool upper, int64_t n, const T* a, int64_t lda, double* d_cs, double* d_out, cudaStream_t s) {
  static const std::string kn = std::string("sym_l1_norm_") + tname<T>();
  ProfScope ps(kn.c_str(), s, (double)n * n, (double)n * n * sizeof(T));
  const unsigned nb = (unsigned)ceil_div(n, CB);
  if (upper) sym_abs_colsum_kernel<T, true><<<nb, 256, 0, s>>>(n, a, lda, d_cs);
  else sym_abs_colsum_kernel<T, false><<<nb, 256, 0, s>>>(n, a, lda, d_cs);
  max_kernel<<<1, 1024, 0, s>>>(n, d_cs, d_out);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

int alloc_async(void** p, size_t bytes, cudaStream_t s) {
  if (dev_malloc_async((void**)p, bytes, s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("cudaMallocAsync failed");
    return GBLLT_ERR_ALLOC;
  }
  return GBLLT_SUCCESS;
}

template <typename T>
int sym_l1_norm_dev(bool upper, int64_t n, const T* a, int64_t lda, T* d_norm, cudaStream_t s) {
  void* w = nullptr;
  int rc = alloc_async(&w, (size_t)(n + 1) * sizeof(double), s);
  if (rc) return rc;
  double* cs = (double*)w;
  rc = sym_l1_norm_into<T>(upper, n, a, lda, cs, cs + n, s);
  if (!rc) {
    to_type_kernel<T><<<1, 1, 0, s>>>(cs + n, d_norm);
    if (cudaGetLastError() != cudaSuccess) rc = GBLLT_ERR_CUDA;
  }
  cudaFreeAsync(w, s);
  return rc;
}

// The estimate of ||A^{-1}||_1 from the factor at d_l (ConditionEstimator.h:56-151); synchronous.
// Like GB_CUDA_TRY, but leaves the enclosing loop with rc set, so that scratch is still freed.
#define CE_TRY(expr)                                                 \
  {                                                                  \
    cudaError_t e__ = (expr);                                        \
    if (e__ != cudaSuccess) {                                        \
      set_last_error(e__, #expr, __FILE__, __LINE__);                \
      rc = GBLLT_ERR_CUDA;                                           \
      break;                                                         \
    }                                                                \
  }

template <typename T>
int inv_l1_estimate(bool upper, int64_t n, const T* d_l, int64_t ldl, double* est, cudaStream_t s) {
  const size_t vb = (((size_t)n * sizeof(T) + 255) / 256) * 256;
  const size_t wsb = potrs_ws_bytes(n, sizeof(T));
  void* w = nullptr;
  int rc = alloc_async(&w, 3 * vb + 256 + wsb, s);
  if (rc) return rc;
  char* base = (char*)w;
  T* v = (T*)base;
  T* sign = (T*)(base + vb);
  T* old_sign = (T*)(base + 2 * vb);
  double* d_l1 = (double*)(base + 3 * vb);
  long long* d_idx = (long long*)(d_l1 + 1);
  int* d_diff = (int*)(d_idx + 1);
  void* ws = base + 3 * vb + 256;
  const unsigned g = (unsigned)ceil_div(n, 256);
  struct Host {
    double l1;
    long long idx;
    int diff;
  } h{};

  // each solve's error word is read back (the estimate synchronises after every solve anyway)
  auto solve = [&](T* x) -> int {
    int r2 = potrs_ws<T>(upper, n, 1, d_l, ldl, x, n, ws, s);
    if (r2) return r2;
    int herr = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&herr, potrs_ws_error_word(n, sizeof(T), ws), sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return herr ? GBLLT_ERR_TIMEOUT : GBLLT_SUCCESS;
  };
  auto read_l1 = [&](double* out) -> int {
    l1_kernel<T><<<1, 1024, 0, s>>>(n, v, d_l1);
    GB_CUDA_TRY(cudaMemcpyAsync(&h.l1, d_l1, sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    *out = h.l1;
    return GBLLT_SUCCESS;
  };

  do {
    // v = A^{-1} (ones / n); lower_bound = ||v||_1
    fill_kernel<T><<<g, 256, 0, s>>>(n, v, 0, nullptr);
    if ((rc = solve(v))) break;
    double lower = 0.0;
    if ((rc = read_l1(&lower))) break;
    if (n == 1) {
      *est = lower;
      break;
    }
    double old_lower = lower;
    long long old_idx = -1;
    for (int k = 0; k < 4; ++k) {
      // sign vector of v; stop when it repeats
      CE_TRY(cudaMemsetAsync(d_diff, 0, sizeof(int), s));
      sign_kernel<T><<<g, 256, 0, s>>>(n, v, sign, k > 0 ? old_sign : nullptr, d_diff);
      if (k > 0) {
        CE_TRY(cudaMemcpyAsync(&h.diff, d_diff, sizeof(int), cudaMemcpyDeviceToHost, s));
        CE_TRY(cudaStreamSynchronize(s));
        if (!h.diff) break;
      }
      // v = A^{-T} sign (A symmetric: the same solve); j = first argmax |v|; stop when it repeats
      CE_TRY(cudaMemcpyAsync(v, sign, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, s));
      if ((rc = solve(v))) break;
      argmax_abs_kernel<T><<<1, 1024, 0, s>>>(n, v, d_idx);
      CE_TRY(cudaMemcpyAsync(&h.idx, d_idx, sizeof(long long), cudaMemcpyDeviceToHost, s));
      CE_TRY(cudaStreamSynchronize(s));
      if (h.idx == old_idx) break;
      // v = A^{-1} e_j; the new lower bound must grow
      fill_kernel<T><<<g, 256, 0, s>>>(n, v, 1, d_idx);
      if ((rc = solve(v))) break;
      if ((rc = read_l1(&lower))) break;
      if (lower <= old_lower) break;
      CE_TRY(cudaMemcpyAsync(old_sign, sign, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, s));
      old_idx = h.idx;
      old_lower = lower;
    }
    if (rc) break;
    // Higham's alternating-sign vector: an independent lower bound 2 ||A^{-1} b||_1 / (3n)
    fill_kernel<T><<<g, 256, 0, s>>>(n, v, 2, nullptr);
    if ((rc = solve(v))) break;
    double alt = 0.0;
    if ((rc = read_l1(&alt))) break;
    alt = 2.0 * alt / (3.0 * (double)n);
    *est = lower > alt ? lower : alt;
  } while (false);
  cudaFreeAsync(w, s);
  if (!rc) GB_CUDA_TRY(cudaGetLastError());
  return rc;
}

// rcond_estimate_helper (ConditionEstimator.h:161-171)
template <typename T>
int pocon_dev(bool upper, int64_t n, const T* d_l, int64_t ldl, double anorm, double* rcond, cudaStream_t s) {
  if (n == 0) {
    *rcond = std::numeric_limits<double>::infinity();
    return GBLLT_SUCCESS;
  }
  if (anorm == 0.0) {
    *rcond = 0.0;
    return GBLLT_SUCCESS;
  }
  if (n == 1) {
    *rcond = 1.0;
    return GBLLT_SUCCESS;
  }
  double est = 0.0;
  int rc = inv_l1_estimate<T>(upper, n, d_l, ldl, &est, s);
  if (rc) return rc;
  *rcond = est == 0.0 ? 0.0 : (1.0 / est) / anorm;
  return GBLLT_SUCCESS;
}

bool upper_of(char uplo) { return uplo == 'U' || uplo == 'u'; }

template <typename T>
int dev_lansy(char uplo, int64_t n, const T* d_a, int64_t lda, T* d_norm, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (n > 0 && !d_a) return -3;
  if (lda < (n > 1 ? n : 1)) return -4;
  if (!d_norm) return -5;
  int rc = ensure_device();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    GB_CUDA_TRY(cudaMemsetAsync(d_norm, 0, sizeof(T), s));
    return GBLLT_SUCCESS;
  }
  return sym_l1_norm_dev<T>(upper_of(uplo), n, d_a, lda, d_norm, s);
}

template <typename T>
int dev_pocon(char uplo, int64_t n, const T* d_l, int64_t ldl, T anorm, T* rcond, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (n > 0 && !d_l) return -3;
  if (ldl < (n > 1 ? n : 1)) return -4;
  if (!(anorm >= T(0))) return -5;
  if (!rcond) return -6;
  int rc = ensure_device();
  if (rc) return rc;
  double r = 0.0;
  rc = pocon_dev<T>(upper_of(uplo), n, d_l, ldl, (double)anorm, &r, (cudaStream_t)stream);
  if (!rc) *rcond = (T)r;
  return rc;
}

template <typename T>
int host_pocon(int layout, char uplo, int64_t n, const T* l, int64_t ldl, T anorm, T* rcond) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (n > 0 && !l) return -4;
  if (ldl < (n > 1 ? n : 1)) return -5;
  if (!(anorm >= T(0))) return -6;
  if (!rcond) return -7;
  if (n <= 1 || anorm == T(0)) {  // answered without the factor (ConditionEstimator.h:165-167)
    double r = 0.0;
    pocon_dev<T>(false, n, nullptr, 1, (double)anorm, &r, nullptr);
    *rcond = (T)r;
    return GBLLT_SUCCESS;
  }
  int rc = ensure_device();
  if (rc) return rc;
  // a row-major lower factor is a column-major upper one (L L^T = U^T U with U = L^T)
  const bool upper = upper_of(uplo) != (layout == GBLLT_ROW_MAJOR);
  cudaStream_t s = lib_stream();
  T* d = nullptr;
  if ((rc = alloc_async((void**)&d, (size_t)n * n * sizeof(T), s))) return rc;
  double r = 0.0;
  if (copy2d_async(d, n * sizeof(T), l, ldl * sizeof(T), n * sizeof(T), n, cudaMemcpyHostToDevice, s) !=
      cudaSuccess) {
    cudaGetLastError();
    set_error_message("gbllt_?pocon: host-to-device copy of the factor failed");
    rc = GBLLT_ERR_CUDA;
  } else {
    rc = pocon_dev<T>(upper, n, d, n, (double)anorm, &r, s);
  }
  cudaFreeAsync(d, s);
  if (!rc) *rcond = (T)r;
  return rc;
}

}  // namespace

}  // namespace gbllt

using namespace gbllt;

extern "C" {

int gbllt_dlansy_l1_dev(char uplo, int64_t n, const double* d_a, int64_t lda, double* d_norm, void* stream) {
  return dev_lansy<double>(uplo, n, d_a, lda, d_norm, stream);
}
int gbllt_slansy_l1_dev(char uplo, int64_t n, const float* d_a, int64_t lda, float* d_norm, void* stream) {
  return dev_lansy<float>(uplo, n, d_a, lda, d_norm, stream);
}
int gbllt_dpocon_dev(char uplo, int64_t n, const double* d_l, int64_t ldl, double anorm, double* rcond, void* stream) {
  return dev_pocon<double>(uplo, n, d_l, ldl, anorm, rcond, stream);
}
int gbllt_spocon_dev(char uplo, int64_t n, const float* d_l, int64_t ldl, float anorm, float* rcond, void* stream) {
  return dev_pocon<float>(uplo, n, d_l, ldl, anorm, rcond, stream);
}
int gbllt_dpocon(int layout, char uplo, int64_t n, const double* l, int64_t ldl, double anorm, double* rcond) {
  return host_pocon<double>(layout, uplo, n, l, ldl, anorm, rcond);
}
int gbllt_spocon(int layout, char uplo, int64_t n, const float* l, int64_t ldl, float anorm, float* rcond) {
  return host_pocon<float>(layout, uplo, n, l, ldl, anorm, rcond);
}

}  // extern "C"
