// Rank-1 update / downdate of a Cholesky factor on the device: L L^T + sigma v v^T = L' L'^T,
// LLT::rankUpdate (Eigen/src/Cholesky/LLT.h:469-478) -> llt_rank_update_lower (LLT.h:238-307).
//
// The reference walks the columns j = 0 .. n-1 in order; column j's coefficients depend on row j
// after all earlier columns have touched it, and every later row then applies them:
//   sigma > 0: a Givens rotation made from (L(j,j), -w(j)) (JacobiRotation::makeGivens,
//              Eigen/src/Jacobi/Jacobi.h:231-267) applied to the pairs (L(k,j), w(k)), k > j;
//   sigma <= 0: the beta recurrence (gamma, x = dj + sigma wj^2 / beta, a failure when x <= 0),
//              applied as w(k) -= (wj/Ljj) L(k,j), L(k,j) = a L(k,j) + b w(k).
// Here 64-row blocks are taken in ticket order by CTAs of 64 threads, thread = row, w(k) in a
// register.  CTA I first applies the columns of every earlier block J as soon as J's flag is up
// (the 64 x 64 tile of L loaded ahead, then 64 steps in registers), then makes its own 64 columns'
// coefficients one at a time (the thread that owns row j makes column j's), applies them to the
// rows below in its block, publishes the coefficients and raises its flag.  A CTA only waits on
// blocks whose CTAs started before it, so there is no deadlock; waits are bounded (2 s), after which
// an error word is set.  The coefficient formulas are the reference's, operation for operation, so
// the result matches Eigen to rounding.  A failing downdate sets the failing column; the factor's
// contents are then unspecified (LLT::rankUpdate reports NumericalIssue).
#include <climits>

#include "internal.h"

namespace gbllt {

namespace {

constexpr int RB = 64;   // rows per CTA and columns per block
constexpr int CW = 8;    // coefficient record width: sigma > 0: c, s; sigma <= 0: f, a, b, g, beta
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// L(i, j) of the lower view: lower column-major, or upper column-major read as its transpose
template <typename T, bool UP>
__device__ __forceinline__ T& lref(T* l, long long ldl, long long i, long long j) {
  return UP ? l[i * ldl + j] : l[j * ldl + i];
}

template <typename T, bool UP, bool DOWN>
__global__ void __launch_bounds__(RB) rank_update_kernel(T* __restrict__ l, long long ldl, long long n,
                                                         const T* __restrict__ v, T sigma, T* __restrict__ coef,
                                                         int* __restrict__ flags, int* __restrict__ counter,
                                                         int* __restrict__ fail, int* __restrict__ err) {
  __shared__ T sc[RB][CW];
  __shared__ int s_ticket, s_abort;
  const int t = threadIdx.x;
  if (t == 0) {
    s_ticket = atomicAdd(counter, 1);
    s_abort = 0;
  }
  __syncthreads();
  const int I = s_ticket;
  const long long I0 = (long long)I * RB, k = I0 + t;
  const bool own = k < n;
  T w = own ? (DOWN ? v[k] : T(sqrt((double)sigma)) * v[k]) : T(0);  // temp = sqrt(sigma) vec (LLT.h:259)
  T beta = T(1);
  // ---- columns of the earlier blocks
  for (int J = 0; J < I; ++J) {
    const long long J0 = (long long)J * RB;
    T xs[RB];
#pragma unroll
    for (int jj = 0; jj < RB; ++jj) xs[jj] = own ? lref<T, UP>(l, ldl, k, J0 + jj) : T(0);
    if (t == 0) {
      const volatile int* f = flags + J;
      const unsigned long long t0 = gtime();
      int fv;
      while ((fv = *f) == 0) {
        if (gtime() - t0 > WAIT_NS) {
          atomicExch(err, 1);
          fv = 2;
          break;
        }
      }
      __threadfence();
      if (fv != 1) s_abort = 1;
    }
    __syncthreads();
    if (s_abort) break;
    for (int idx = t; idx < RB * CW; idx += RB) sc[idx / CW][idx % CW] = __ldcg(coef + J0 * CW + idx);
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < RB; ++jj) {
      const T x = xs[jj];
      if (!DOWN) {
        const T c = sc[jj][0], s = sc[jj][1];
        const T msx = -s * x;
        xs[jj] = c * x + s * w;
        w = fma(c, w, msx);
      } else {
        w -= sc[jj][0] * x;
        if (sc[jj][3] != T(0)) xs[jj] = sc[jj][1] * x + sc[jj][2] * w;
      }
    }
    if (DOWN) beta = sc[RB - 1][4];
#pragma unroll
    for (int jj = 0; jj < RB; ++jj)
      if (own && J0 + jj < n) lref<T, UP>(l, ldl, k, J0 + jj) = xs[jj];
    __syncthreads();
  }
  if (s_abort) {  // an earlier block failed or timed out: pass the stop on
    __syncthreads();
    if (t == 0) atomicExch(flags + I, 2);
    return;
  }
  // ---- this block's own columns, one at a time
  const int nown = (int)(n - I0 < RB ? n - I0 : RB);
  for (int jj = 0; jj < nown; ++jj) {
    const long long j = I0 + jj;
    if (t == jj) {
      T* d = &lref<T, UP>(l, ldl, j, j);
      if (!DOWN) {
        // JacobiRotation::makeGivens(p, q, &r) for real scalars (Jacobi.h:231-267)
        const T p = *d, q = -w;
        T c, s, r;
        if (q == T(0)) {
          c = p < T(0) ? T(-1) : T(1);
          s = T(0);
          r = fabs(p);
        } else if (p == T(0)) {
          c = T(0);
          s = q < T(0) ? T(1) : T(-1);
          r = fabs(q);
        } else if (fabs(p) > fabs(q)) {
          const T tt = q / p;
          T u = sqrt(T(1) + tt * tt);
          if (p < T(0)) u = -u;
          c = T(1) / u;
          s = -tt * c;
          r = p * u;
        } else {
          const T tt = p / q;
          T u = sqrt(T(1) + tt * tt);
          if (q < T(0)) u = -u;
          s = -T(1) / u;
          c = -tt * s;
          r = q * u;
        }
        *d = r;
        sc[jj][0] = c;
        sc[jj][1] = s;
      } else {
        // the beta recurrence of LLT.h:281-303
        const T Ljj = *d, dj = Ljj * Ljj, wj = w, swj2 = sigma * wj * wj;
        const T gamma = dj * beta + swj2;
        const T x = dj + swj2 / beta;
        if (x <= T(0)) {
          atomicMin(fail, (int)j);
          s_abort = 1;
        } else {
          const T nLjj = sqrt(x);
          *d = nLjj;
          beta += swj2 / dj;
          sc[jj][0] = wj / Ljj;
          sc[jj][1] = nLjj / Ljj;
          sc[jj][2] = nLjj * sigma * wj / gamma;
          sc[jj][3] = gamma != T(0) ? T(1) : T(0);
          sc[jj][4] = beta;
        }
      }
    }
    __syncthreads();
    if (s_abort) break;
    if (DOWN) beta = sc[jj][4];
    if (own && t > jj) {
      T& xr = lref<T, UP>(l, ldl, k, j);
      const T x = xr;
      if (!DOWN) {
        const T c = sc[jj][0], s = sc[jj][1];
        const T msx = -s * x;
        xr = c * x + s * w;
        w = fma(c, w, msx);
      } else {
        w -= sc[jj][0] * x;
        if (sc[jj][3] != T(0)) xr = sc[jj][1] * x + sc[jj][2] * w;
      }
    }
  }
  // publish: the coefficients, then (after a fence) the block's flag (2 = stop)
  for (int idx = t; idx < RB * CW; idx += RB) coef[I0 * CW + idx] = sc[idx / CW][idx % CW];
  __threadfence();
  __syncthreads();
  if (t == 0) atomicExch(flags + I, s_abort ? 2 : 1);
}

// info = 0, the failing column + 1, or GBLLT_ERR_TIMEOUT when a bounded wait ran out
__global__ void rank_update_info_kernel(const int* fail, const int* err, int64_t* info) {
  *info = *err ? (int64_t)GBLLT_ERR_TIMEOUT : (*fail == INT_MAX ? 0 : (int64_t)*fail + 1);
}

__global__ void set_int_kernel(int* p, int v) { *p = v; }

}  // namespace

template <typename T>
int rank_update_dev(bool upper, int64_t n, T* l, int64_t ldl, const T* v, T sigma, int64_t* d_info, cudaStream_t s) {
  const int nb = (int)ceil_div(n, RB);
  const size_t cbytes = ((size_t)nb * RB * CW * sizeof(T) + 255) & ~(size_t)255;
  void* w = nullptr;
  if (dev_malloc_async((void**)&w, cbytes + (size_t)(nb + 4) * sizeof(int), s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("gbllt_?rank_update_dev: cudaMallocAsync failed");
    return GBLLT_ERR_ALLOC;
  }
  T* coef = (T*)w;
  int* flags = (int*)((char*)w + cbytes);
  int* counter = flags + nb;
  int* fail = counter + 1;
  int* err = counter + 2;
  int rc = GBLLT_SUCCESS;
  if (cudaMemsetAsync(flags, 0, (size_t)(nb + 4) * sizeof(int), s) != cudaSuccess) rc = GBLLT_ERR_CUDA;
  if (!rc) {
    set_int_kernel<<<1, 1, 0, s>>>(fail, INT_MAX);
    static const std::string kn = std::string("rank_update_") + tname<T>();
    ProfScope ps(kn.c_str(), s, 4.0 * (double)n * n, (double)n * n * sizeof(T));
    const bool down = !(sigma > T(0));
    if (upper) {
      if (down) rank_update_kernel<T, true, true><<<nb, RB, 0, s>>>(l, ldl, n, v, sigma, coef, flags, counter, fail, err);
      else rank_update_kernel<T, true, false><<<nb, RB, 0, s>>>(l, ldl, n, v, sigma, coef, flags, counter, fail, err);
    } else {
      if (down) rank_update_kernel<T, false, true><<<nb, RB, 0, s>>>(l, ldl, n, v, sigma, coef, flags, counter, fail, err);
      else rank_update_kernel<T, false, false><<<nb, RB, 0, s>>>(l, ldl, n, v, sigma, coef, flags, counter, fail, err);
    }
    rank_update_info_kernel<<<1, 1, 0, s>>>(fail, err, d_info);
    if (cudaGetLastError() != cudaSuccess) rc = GBLLT_ERR_CUDA;
  }
  cudaFreeAsync(w, s);
  return rc;
}

template int rank_update_dev<double>(bool, int64_t, double*, int64_t, const double*, double, int64_t*, cudaStream_t);
template int rank_update_dev<float>(bool, int64_t, float*, int64_t, const float*, float, int64_t*, cudaStream_t);

}  // namespace gbllt

using namespace gbllt;

namespace {

template <typename T>
int dev_rank_update(char uplo, int64_t n, T* d_l, int64_t ldl, const T* d_v, T sigma, int64_t* d_info, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (n > 0 && !d_l) return -3;
  if (ldl < (n > 1 ? n : 1)) return -4;
  if (n > 0 && !d_v) return -5;
  if (sigma != sigma) return -6;  // NaN
  if (!d_info) return -7;
  int rc = ensure_device();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    GB_CUDA_TRY(cudaMemsetAsync(d_info, 0, sizeof(int64_t), s));
    return GBLLT_SUCCESS;
  }
  return rank_update_dev<T>(uplo == 'U' || uplo == 'u', n, d_l, ldl, d_v, sigma, d_info, s);
}

template <typename T>
int host_rank_update(int layout, char uplo, int64_t n, T* l, int64_t ldl, const T* v, T sigma, int64_t* info) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (n > 0 && !l) return -4;
  if (ldl < (n > 1 ? n : 1)) return -5;
  if (n > 0 && !v) return -6;
  if (sigma != sigma) return -7;
  if (!info) return -8;
  *info = 0;
  if (n == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  // a row-major lower factor is a column-major upper one
  const bool upper = (uplo == 'U' || uplo == 'u') != (layout == GBLLT_ROW_MAJOR);
  cudaStream_t s = lib_stream();
  const size_t es = sizeof(T), lbytes = ((size_t)n * n * es + 255) & ~(size_t)255;
  void* w = nullptr;
  if (dev_malloc_async((void**)&w, lbytes + (size_t)n * es + 256 + sizeof(int64_t), s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("gbllt_?rank_update: cudaMallocAsync failed");
    return GBLLT_ERR_ALLOC;
  }
  T* d_l = (T*)w;
  T* d_v = (T*)((char*)w + lbytes);
  int64_t* d_info = (int64_t*)((char*)d_v + (((size_t)n * es + 255) & ~(size_t)255));
  int64_t h_info = 0;
  do {
    if (copy2d_async(d_l, n * es, l, ldl * es, n * es, n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d_v, v, n * es, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      set_last_error(cudaGetLastError(), "gbllt_?rank_update: copy to the device", __FILE__, __LINE__);
      rc = GBLLT_ERR_CUDA;
      break;
    }
    if ((rc = rank_update_dev<T>(upper, n, d_l, n, d_v, sigma, d_info, s))) break;
    if (copy2d_async(l, ldl * es, d_l, n * es, n * es, n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&h_info, d_info, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      set_last_error(cudaGetLastError(), "gbllt_?rank_update: copy to the host", __FILE__, __LINE__);
      rc = GBLLT_ERR_CUDA;
      break;
    }
  } while (false);
  cudaFreeAsync(w, s);
  if (rc) return rc;
  if (h_info == GBLLT_ERR_TIMEOUT) {
    set_error_message("gbllt_?rank_update: a bounded device wait ran out");
    return GBLLT_ERR_TIMEOUT;
  }
  *info = h_info;
  return GBLLT_SUCCESS;
}

}  // namespace

extern "C" {

int gbllt_drank_update_dev(char uplo, int64_t n, double* d_l, int64_t ldl, const double* d_v, double sigma,
                           int64_t* d_info, void* stream) {
  return dev_rank_update<double>(uplo, n, d_l, ldl, d_v, sigma, d_info, stream);
}
int gbllt_srank_update_dev(char uplo, int64_t n, float* d_l, int64_t ldl, const float* d_v, float sigma,
                           int64_t* d_info, void* stream) {
  return dev_rank_update<float>(uplo, n, d_l, ldl, d_v, sigma, d_info, stream);
}
int gbllt_drank_update(int layout, char uplo, int64_t n, double* l, int64_t ldl, const double* v, double sigma,
                       int64_t* info) {
  return host_rank_update<double>(layout, uplo, n, l, ldl, v, sigma, info);
}
int gbllt_srank_update(int layout, char uplo, int64_t n, float* l, int64_t ldl, const float* v, float sigma,
                       int64_t* info) {
  return host_rank_update<float>(layout, uplo, n, l, ldl, v, sigma, info);
}

}  // extern "C"
