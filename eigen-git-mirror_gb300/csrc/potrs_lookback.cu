// Single-pass blocked triangular sweeps for the solve L L^T X = B (LLT::_solve_impl_transposed,
// Eigen/src/Cholesky/LLT.h:490-498; TriangularSolverMatrix.h:38-184 / TriangularSolverVector.h:30-142).
//
// One kernel per sweep.  Row blocks of 64 are taken in ticket order from an atomic counter, so a
// CTA only ever waits on blocks whose CTAs started before it (no deadlock whatever the residency).
// CTA I (forward: Y_I = L_II^{-1} (B_I - sum_{J<I} L_IJ Y_J)):
//   - loads each off-diagonal 64 x 64 tile of L into shared memory with coalesced loads (the
//     loads do not depend on other blocks, so most CTAs stream L at HBM speed);
//   - waits for block J's flag (bounded: 2 s, then an error word is set and the CTA stops), reads
//     Y_J through L2 (ld.global.cg) and accumulates the tile product;
//   - applies the pre-inverted diagonal triangle (a 64 x 64 product instead of a 64-step
//     substitution on the critical path), stores Y_I, fences, and raises its flag.
// The backward sweep runs the same scheme on L^T from the last block up.  Right-hand sides are
// split into chunks of 16 that run as independent chains in the same launch (grid.y), so the FP64
// work of the last row blocks is spread over several SMs.
//
// The diagonal inverses come from trinv_kernel (one CTA per block, column-wise substitution).
//
// The same sweeps solve with the factor of LDL^T (LDLT::_solve_impl_transposed, LDLT.h:573-613):
// L has a unit diagonal (trinv_kernel<UNIT>) and the diagonal of the stored factor holds D; the
// backward sweep applies D's pseudo-inverse to each block's right-hand sides as it loads them
// (DSCALE: divide where |d| > the smallest normal number, else 0, LDLT.h:587-600).
#include <cfloat>

#include "internal.h"

namespace gbllt {

namespace {

constexpr int RB = 64;
constexpr int RC = 512;  // right-hand sides per launch (at most 32 chains of 16)
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <typename T, bool UP>
__device__ __forceinline__ T lget(const T* __restrict__ a, long long lda, long long i, long long j) {
  return UP ? a[i * lda + j] : a[j * lda + i];  // L(i, j)
}

// inv[blk] (64 x 64, column-major, lower) = L_blk^{-1}; identity padding beyond n.  UNIT: the
// diagonal of L is 1 and the stored diagonal (D of an LDL^T factor) is not read.
template <typename T, bool UP, bool UNIT>
__global__ void __launch_bounds__(128) trinv_kernel(const T* __restrict__ a, long long lda, long long n,
                                                    T* __restrict__ inv) {
  __shared__ T L[RB][RB + 1];  // L[i][p]
  const long long b0 = (long long)blockIdx.x * RB;
  const int bs = (int)(n - b0 < RB ? n - b0 : RB);
  for (int idx = threadIdx.x; idx < RB * RB; idx += 128) {
    int i, p;
    if (UP) { p = idx % RB; i = idx / RB; }
    else    { i = idx % RB; p = idx / RB; }
    T v = (i == p) ? T(1) : T(0);
    if (i < bs && p < bs && (UNIT ? i > p : i >= p)) v = lget<T, UP>(a, lda, b0 + i, b0 + p);
    L[i][p] = v;
  }
  __syncthreads();
  T* out = inv + (long long)blockIdx.x * RB * RB;
  if (threadIdx.x < RB) {
    const int c = threadIdx.x;  // column c of the inverse: L x = e_c
    T x[RB];
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      T v = (i == c) ? T(1) : T(0);
#pragma unroll
      for (int p = 0; p < i; ++p) v = fma(-L[i][p], x[p], v);
      x[i] = i < c ? T(0) : (UNIT ? v : v / L[i][i]);
    }
#pragma unroll
    for (int i = 0; i < RB; ++i) out[(long long)c * RB + i] = x[i];
  }
}

template <typename T, int RCT>
struct SweepSmem {
  T Ls[RB][RB + 1];    // Ls[p][r]: forward L(I0+r, J0+p); backward L(J0+p, I0+r)
  T Ds[RB][RB + 1];    // inverse of the diagonal triangle, Ds[i][p] = Linv(i, p)
  T Ys[RB][RCT + 1];   // the solved block J
  T Bs[RB][RCT + 1];   // this block's right-hand sides
};

// The pseudo-inverse of one entry of D (LDLT.h:594-600).
template <typename T>
__device__ __forceinline__ T dplus(T v, T d) {
  const T tiny = sizeof(T) == 8 ? (T)DBL_MIN : (T)FLT_MIN;
  return fabs(d) > tiny ? v / d : T(0);
}

// RCT right-hand sides per pass; thread (r, cq) owns row r and RCT/4 of them.  DSCALE (backward
// sweep of the LDL^T solve): the block's right-hand sides are multiplied by D^+ as they are loaded.
template <typename T, bool UP, bool BWD, int RCT, bool DSCALE>
__global__ void __launch_bounds__(256) sweep_kernel(const T* __restrict__ a, long long lda, long long n,
                                                    T* __restrict__ b, long long ldb, int nrhs, const T* __restrict__ inv,
                                                    int* __restrict__ flags, int* __restrict__ counter,
                                                    int* __restrict__ err) {
  constexpr int CPT = RCT / 4;
  // right-hand-side chunk: an independent chain with its own tickets and flags
  {
    const int chunk = blockIdx.y;
    b += (long long)chunk * RCT * ldb;
    nrhs -= chunk * RCT;
    flags += (long long)chunk * ((n + RB - 1) / RB);
    counter += chunk;
  }
  extern __shared__ __align__(16) unsigned char sweep_raw[];
  SweepSmem<T, RCT>& sm = *reinterpret_cast<SweepSmem<T, RCT>*>(sweep_raw);
  __shared__ int s_ticket, s_abort;
  const int tid = threadIdx.x, r = tid & 63, cq = tid >> 6;
  const int nb = (int)((n + RB - 1) / RB);
  if (tid == 0) {
    s_ticket = atomicAdd(counter, 1);
    s_abort = 0;
  }
  __syncthreads();
  const int I = BWD ? nb - 1 - s_ticket : s_ticket;
  const long long I0 = (long long)I * RB;
  // inputs that do not depend on other blocks are fetched first, off the critical path
  const T* Dinv = inv + (long long)I * RB * RB;
  for (int idx = tid; idx < RB * RB; idx += 256) {
    const int i = idx & 63, p = idx >> 6;
    sm.Ds[i][p] = Dinv[(long long)p * RB + i];
  }
  for (int idx = tid; idx < RB * RCT; idx += 256) {
    const int p = idx & 63, c = idx >> 6;
    T v = (I0 + p < n && c < nrhs) ? b[(long long)c * ldb + I0 + p] : T(0);
    if (DSCALE && I0 + p < n) v = dplus(v, a[(I0 + p) * (lda + 1)]);
    sm.Bs[p][c] = v;
  }
  T acc[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) acc[q] = T(0);
  // off-diagonal blocks in the order they become ready
  const int jfirst = BWD ? nb - 1 : 0;
  const int jstep = BWD ? -1 : 1;
  for (int J = jfirst; J != I; J += jstep) {
    const long long J0 = (long long)J * RB;
    constexpr bool r_fast = (!BWD && !UP) || (BWD && UP);
    for (int idx = tid; idx < RB * RB; idx += 256) {
      int rr, p;
      if (r_fast) { rr = idx & 63; p = idx >> 6; }
      else        { p = idx & 63; rr = idx >> 6; }
      T v = T(0);
      if (I0 + rr < n && J0 + p < n)
        v = BWD ? lget<T, UP>(a, lda, J0 + p, I0 + rr) : lget<T, UP>(a, lda, I0 + rr, J0 + p);
      sm.Ls[p][rr] = v;
    }
    if (tid == 0) {
      const volatile int* f = flags + J;
      const unsigned long long t0 = gtimer();
      while (*f == 0) {
        if (gtimer() - t0 > WAIT_NS) {
          s_abort = 1;
          atomicExch(err, 1);
          break;
        }
      }
      __threadfence();
    }
    __syncthreads();
    if (s_abort) return;
    for (int idx = tid; idx < RB * RCT; idx += 256) {
      const int p = idx & 63, c = idx >> 6;
      sm.Ys[p][c] = (J0 + p < n && c < nrhs) ? __ldcg(b + (long long)c * ldb + J0 + p) : T(0);
    }
    __syncthreads();
#pragma unroll 4
    for (int p = 0; p < RB; ++p) {
      const T l = sm.Ls[p][r];
#pragma unroll
      for (int q = 0; q < CPT; ++q) acc[q] = fma(l, sm.Ys[p][cq * CPT + q], acc[q]);
    }
    __syncthreads();
  }
  // V = B_I - acc, then X_I = Linv V (forward) or Linv^T V (backward).  The barrier orders the Ds/Bs
  // preload (written under another thread mapping) before these reads when the J loop ran no pass.
  __syncthreads();
#pragma unroll
  for (int q = 0; q < CPT; ++q) sm.Ys[r][cq * CPT + q] = sm.Bs[r][cq * CPT + q] - acc[q];
  __syncthreads();
  T x[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) x[q] = T(0);
#pragma unroll 4
  for (int p = 0; p < RB; ++p) {
    const T d = BWD ? sm.Ds[p][r] : sm.Ds[r][p];
#pragma unroll
    for (int q = 0; q < CPT; ++q) x[q] = fma(d, sm.Ys[p][cq * CPT + q], x[q]);
  }
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int c = cq * CPT + q;
    if (I0 + r < n && c < nrhs) b[(long long)c * ldb + I0 + r] = x[q];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) atomicExch(flags + I, 1);
}

template <typename T, bool UP, bool BWD, int RCT, bool DSCALE>
void launch_sweep_rc(int nb, const T* a, long long lda, long long n, T* b, long long ldb, int nrhs, const T* inv,
                     int* flags, int* counter, int* err, cudaStream_t s) {
  // set on every launch: cheap, and correct for every device and host thread
  const int smem = (int)sizeof(SweepSmem<T, RCT>);
  cudaFuncSetAttribute(sweep_kernel<T, UP, BWD, RCT, DSCALE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  dim3 grid((unsigned)nb, (unsigned)((nrhs + RCT - 1) / RCT));
  sweep_kernel<T, UP, BWD, RCT, DSCALE><<<grid, 256, smem, s>>>(a, lda, n, b, ldb, nrhs, inv, flags, counter, err);
}

// One launch per sweep: chunks of RCT right-hand sides run as parallel chains (grid.y); 4 columns
// per chunk for a single right-hand side, 16 otherwise (more chains spread the FP64 work of the
// last row blocks over more SMs).
template <typename T, bool UP, bool BWD, bool DSCALE = false>
void launch_sweep(int nb, const T* a, long long lda, long long n, T* b, long long ldb, int nrhs, const T* inv,
                  int* flags, int* counter, int* err, cudaStream_t s) {
  if (nrhs <= 4) launch_sweep_rc<T, UP, BWD, 4, DSCALE>(nb, a, lda, n, b, ldb, nrhs, inv, flags, counter, err, s);
  else launch_sweep_rc<T, UP, BWD, 16, DSCALE>(nb, a, lda, n, b, ldb, nrhs, inv, flags, counter, err, s);
}

}  // namespace

size_t potrs_ws_bytes(int64_t n, size_t elem) {
  const int64_t nb = (n + RB - 1) / RB;
  const int64_t nch = RC / 16;  // chains of one launch, at most
  return (size_t)nb * RB * RB * elem + (size_t)(2 * nch * nb + 2 * nch + 8) * sizeof(int) + 512;
}

// Both sweeps; ldl: the factor is the unit L of LDL^T with D on its diagonal.
template <typename T>
int sweeps_ws(bool upper, bool ldl, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, void* ws,
              cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
  static const std::string ki = std::string("trinv_diag_") + tname<T>();
  static const std::string kf = std::string("sweep_") + tname<T>();
  const int nb = (int)ceil_div(n, RB);
  T* inv = (T*)ws;
  int* base = (int*)((char*)ws + (((size_t)nb * RB * RB * sizeof(T) + 255) & ~(size_t)255));
  {
    ProfScope ps(ki.c_str(), s, (double)nb * RB * RB * RB / 3.0, (double)n * RB * sizeof(T) * 1.5);
    if (ldl) {
      if (upper) trinv_kernel<T, true, true><<<nb, 128, 0, s>>>(a, lda, n, inv);
      else trinv_kernel<T, false, true><<<nb, 128, 0, s>>>(a, lda, n, inv);
    } else {
      if (upper) trinv_kernel<T, true, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
      else trinv_kernel<T, false, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
    }
  }
  for (int64_t c0 = 0; c0 < nrhs; c0 += RC) {
    const int nc = (int)(nrhs - c0 < RC ? nrhs - c0 : RC);
    const int nch = nc <= 4 ? 1 : (nc + 15) / 16;  // chains in this launch
    int* fflags = base;                 // forward: nch x nb
    int* bflags = base + nch * nb;      // backward: nch x nb
    int* fctr = base + 2 * nch * nb;    // nch forward tickets, nch backward tickets, error word
    int* bctr = fctr + nch;
    int* err = bctr + nch;
    T* bc = b + c0 * ldb;
    GB_CUDA_TRY(cudaMemsetAsync(base, 0, (size_t)(2 * nch * nb + 2 * nch + 1) * sizeof(int), s));
    // algorithmic work per sweep: the lower triangle of L read once, 2 flops per entry and RHS
    const double fl = (double)n * (n + 1) * nc, by = (double)n * (n + 1) / 2.0 * sizeof(T) + 2.0 * n * nc * sizeof(T);
    {
      ProfScope ps(kf.c_str(), s, fl, by);
      if (upper) launch_sweep<T, true, false>(nb, a, lda, n, bc, ldb, nc, inv, fflags, fctr, err, s);
      else launch_sweep<T, false, false>(nb, a, lda, n, bc, ldb, nc, inv, fflags, fctr, err, s);
    }
    {
      ProfScope ps(kf.c_str(), s, fl, by);
      if (ldl) {
        if (upper) launch_sweep<T, true, true, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
        else launch_sweep<T, false, true, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
      } else {
        if (upper) launch_sweep<T, true, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
        else launch_sweep<T, false, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
      }
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int potrs_ws(bool upper, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, void* ws,
             cudaStream_t s) {
  return sweeps_ws<T>(upper, false, n, nrhs, a, lda, b, ldb, ws, s);
}

template <typename T>
int trsm_sweep_ws(bool upper, bool bwd, bool unit, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b,
                  int64_t ldb, void* ws, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
  static const std::string ki = std::string("trinv_diag_") + tname<T>();
  static const std::string kf = std::string("sweep_") + tname<T>();
  const int nb = (int)ceil_div(n, RB);
  T* inv = (T*)ws;
  int* base = (int*)((char*)ws + (((size_t)nb * RB * RB * sizeof(T) + 255) & ~(size_t)255));
  {
    ProfScope ps(ki.c_str(), s, (double)nb * RB * RB * RB / 3.0, (double)n * RB * sizeof(T) * 1.5);
    if (unit) {
      if (upper) trinv_kernel<T, true, true><<<nb, 128, 0, s>>>(a, lda, n, inv);
      else trinv_kernel<T, false, true><<<nb, 128, 0, s>>>(a, lda, n, inv);
    } else {
      if (upper) trinv_kernel<T, true, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
      else trinv_kernel<T, false, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
    }
  }
  for (int64_t c0 = 0; c0 < nrhs; c0 += RC) {
    const int nc = (int)(nrhs - c0 < RC ? nrhs - c0 : RC);
    const int nch = nc <= 4 ? 1 : (nc + 15) / 16;
    int* flags = base;
    int* ctr = base + nch * nb;
    int* err = ctr + nch;
    T* bc = b + c0 * ldb;
    GB_CUDA_TRY(cudaMemsetAsync(base, 0, (size_t)(nch * nb + nch + 1) * sizeof(int), s));
    const double fl = (double)n * (n + 1) * nc, by = (double)n * (n + 1) / 2.0 * sizeof(T) + 2.0 * n * nc * sizeof(T);
    ProfScope ps(kf.c_str(), s, fl, by);
    if (bwd) {
      if (upper) launch_sweep<T, true, true>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s);
      else launch_sweep<T, false, true>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s);
    } else {
      if (upper) launch_sweep<T, true, false>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s);
      else launch_sweep<T, false, false>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s);
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int ldlt_sweeps_ws(bool upper, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, void* ws,
                   cudaStream_t s) {
  return sweeps_ws<T>(upper, true, n, nrhs, a, lda, b, ldb, ws, s);
}

template int potrs_ws<double>(bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, void*, cudaStream_t);
template int potrs_ws<float>(bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, void*, cudaStream_t);
template int ldlt_sweeps_ws<double>(bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, void*,
                                    cudaStream_t);
template int ldlt_sweeps_ws<float>(bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, void*, cudaStream_t);
template int trsm_sweep_ws<double>(bool, bool, bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, void*,
                                   cudaStream_t);
template int trsm_sweep_ws<float>(bool, bool, bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, void*,
                                  cudaStream_t);

}  // namespace gbllt
