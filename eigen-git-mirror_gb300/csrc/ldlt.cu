// Pivoted LDL^T on the GPU: LDLT<MatrixXd|MatrixXf, UpLo>::compute and solve
// (Eigen/src/Cholesky/LDLT.h:497-530, 573-613).
//
// Eigen's factorisation (ldlt_inplace<Lower>::unblocked, LDLT.h:297-403) is left-looking and
// column by column: at step k it swaps the largest |diagonal entry| of the trailing corner into
// place, updates column k from the columns before it and divides it by the pivot.  The diagonal
// entries of the corner are never updated before their own step, so the whole pivot order is a
// function of the input's diagonal alone: it is the sequence of swaps that selection by largest
// |value| (first position on ties) makes on that diagonal.  The GPU path therefore splits the
// work into
//
//   1. the pivot order, on the host in O(n log n) (a tournament tree over the diagonal that
//      replays Eigen's swaps, so the transpositions are Eigen's bit for bit);
//   2. ldlt_gather_kernel: W = P A P^T, lower triangle, from the stored triangle of A;
//   3. a right-looking blocked LDL^T without pivoting on W, panels of 64:
//        ldlt_diag_kernel   one CTA factors the 64 x 64 diagonal block with Eigen's column step
//                           and its zero-pivot rules (a pivot with |d| = 0 leaves its column
//                           undivided and requires it to be zero, LDLT.h:366-387);
//        ldlt_panel_kernel  the rows below it: L21 = A21 L11^{-T} D1^{-1}, and T21 = L21 D1 (Eigen's
//                           temp, LDLT.h:358) as the second operand of the update, one thread per row;
//        syrk_lower_kernel  A22 -= L21 T21^T on the lower 64 x 64 tiles (shared with the Cholesky);
//   4. ldlt_finish_kernel: Eigen's sign (the signs of the pivots, LDLT.h:389-397) and success
//      flag (no nonzero column under a zero pivot, no nonzero pivot after a zero one);
//   5. ldlt_scatter_kernel: the factor back into the caller's triangle.
//
// The diagonal and panel kernels round every product and sum separately and in Eigen's order, so
// the first 64 columns of a lower factor are those of Eigen built without FMA contraction (its
// SSE2 build) bit for bit; the trailing update accumulates with FMAs in another order, and later
// columns agree to rounding.  A column whose pivot is zero contributes temp = 0 * l = 0 to later
// columns, as in Eigen.
// The solve permutes the right-hand sides, runs the single-pass sweeps of the Cholesky solve
// with a unit diagonal and D's pseudo-inverse between them (potrs_lookback.cu), and permutes back.
#include <cmath>
#include <vector>

#include "internal.h"

namespace gbllt {

namespace {

constexpr int NB = kNB;

// ---- pivot order (host) -------------------------------------------------------------------------

// Replays ldlt_inplace's pivot search (LDLT.h:323-346) on the diagonal: at step k the position of
// the largest |d| among positions k..n-1, the first one on ties, is swapped with position k.  A
// tournament tree over positions answers each search in O(1) and each swap in O(log n).  `perm`
// receives the composite permutation: perm[i] = the input row that ends at position i.
// A NaN diagonal entry never wins a comparison (Eigen's maxCoeff keeps the running maximum), except
// at the first position of the searched range, where Eigen's scan starts.
void pivot_order(int64_t n, const double* absd, int32_t* transp, int32_t* perm) {
  int64_t sz = 1;
  while (sz < n) sz <<= 1;
  std::vector<double> key(n);
  std::vector<int32_t> tree(2 * sz, -1);
  for (int64_t i = 0; i < n; ++i) {
    key[i] = std::isnan(absd[i]) ? -1.0 : absd[i];
    perm[i] = (int32_t)i;
  }
  auto better = [&](int32_t x, int32_t y) -> int32_t {  // positions (or -1 = empty)
    if (x < 0) return y;
    if (y < 0) return x;
    if (key[x] > key[y]) return x;
    if (key[y] > key[x]) return y;
    return x < y ? x : y;
  };
  for (int64_t i = 0; i < n; ++i) tree[sz + i] = (int32_t)i;
  for (int64_t v = sz - 1; v >= 1; --v) tree[v] = better(tree[2 * v], tree[2 * v + 1]);
  auto update = [&](int64_t pos) {
    for (int64_t v = (sz + pos) >> 1; v >= 1; v >>= 1) tree[v] = better(tree[2 * v], tree[2 * v + 1]);
  };
  std::vector<char> nan_at(n);
  for (int64_t i = 0; i < n; ++i) nan_at[i] = std::isnan(absd[i]) ? 1 : 0;
  for (int64_t k = 0; k < n; ++k) {
    int64_t p = nan_at[k] ? k : tree[1];
    transp[k] = (int32_t)p;
    if (p != k) {
      std::swap(key[k], key[p]);
      std::swap(nan_at[k], nan_at[p]);
      std::swap(perm[k], perm[p]);
      tree[sz + p] = (int32_t)p;
      update(p);
    }
    key[k] = -2.0;  // position k leaves the search
    tree[sz + k] = -1;
    update(k);
  }
}

// perm (composite) from a transposition sequence of any origin: apply the swaps in order.
int perm_from_transpositions(int64_t n, const int32_t* transp, std::vector<int32_t>& perm) {
  perm.resize(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
  for (int64_t k = 0; k < n; ++k) {
    const int64_t t = transp[k];
    if (t < 0 || t >= n) return -1;
    std::swap(perm[k], perm[t]);
  }
  return 0;
}

}  // namespace

namespace {

// ---- kernels ------------------------------------------------------------------------------------

// Stored triangle of the symmetric A: the entry (r, c) read from its lower (UP = false) or upper
// (UP = true) copy.
template <typename T, bool UP>
__device__ __forceinline__ T sym_at(const T* __restrict__ a, long long lda, long long r, long long c) {
  const long long lo = r < c ? r : c, hi = r < c ? c : r;
  return UP ? a[hi * lda + lo] : a[lo * lda + hi];
}

// W(i, j) = A(perm[i], perm[j]) for i >= j, one CTA per 64 x 64 lower tile of W.
template <typename T, bool UP>
__global__ void __launch_bounds__(256) ldlt_gather_kernel(const T* __restrict__ a, long long lda, long long n,
                                                          const int32_t* __restrict__ perm, T* __restrict__ w,
                                                          long long ldw) {
  __shared__ int32_t pr[64], pc[64];
  int ti, tj;
  lower_tile_coords(blockIdx.x, ti, tj);
  const long long i0 = (long long)ti * 64, j0 = (long long)tj * 64;
  if (threadIdx.x < 64) {
    const long long i = i0 + threadIdx.x, j = j0 + threadIdx.x;
    pr[threadIdx.x] = i < n ? perm[i] : 0;
    pc[threadIdx.x] = j < n ? perm[j] : 0;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int ii = idx & 63, jj = idx >> 6;
    const long long i = i0 + ii, j = j0 + jj;
    if (i < n && j <= i) w[j * ldw + i] = sym_at<T, UP>(a, lda, pr[ii], pc[jj]);
  }
}

// The caller's triangle from W: A(i, j) = W(i, j) (lower) or A(j, i) = W(i, j) (upper), i >= j,
// through a shared tile so that both sides are coalesced.
template <typename T, bool UP>
__global__ void __launch_bounds__(256) ldlt_scatter_kernel(const T* __restrict__ w, long long ldw, long long n,
                                                           T* __restrict__ a, long long lda) {
  __shared__ T tile[64][65];  // tile[jj][ii] = W(i0 + ii, j0 + jj)
  int ti, tj;
  lower_tile_coords(blockIdx.x, ti, tj);
  const long long i0 = (long long)ti * 64, j0 = (long long)tj * 64;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int ii = idx & 63, jj = idx >> 6;
    const long long i = i0 + ii, j = j0 + jj;
    if (i < n && j <= i) {
      if (UP) tile[jj][ii] = w[j * ldw + i];
      else a[j * lda + i] = w[j * ldw + i];
    }
  }
  if (!UP) return;
  __syncthreads();
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int jj = idx & 63, ii = idx >> 6;
    const long long i = i0 + ii, j = j0 + jj;
    if (i < n && j <= i) a[i * lda + j] = tile[jj][ii];
  }
}

// IEEE-rounded operations that the compiler may not fuse: Eigen's SSE2 build rounds every product
// and every sum, and the kernels below reproduce its order of operations.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// LDL^T of the bs x bs diagonal block at (k0, k0) of W, one thread per row, column by column in
// Eigen's left-looking order (LDLT.h:352-387).  For column k:
//   temp_j  = d_j * L(k, j), j < k                                          (LDLT.h:358)
//   d_k     = A(k, k) - (L(k,0) temp_0 + L(k,1) temp_1 + ...), summed left to right  (:359)
//   A(i, k) = A(i, k) - (0 + L(i,0) temp_0 + ...), i > k: the column-major GEMV's per-row
//             accumulation (GeneralMatrixVector.h), then divided by d_k if |d_k| > 0 (:372-375);
//             under a zero pivot the column must be zero (else *bad = 1).
// Every product and sum is rounded separately, so for the first diagonal block (k0 = 0) the
// factor is Eigen's to the bit.  Later blocks have already received the updates of earlier panels
// from syrk_lower_kernel.
template <typename T>
__global__ void __launch_bounds__(64) ldlt_diag_kernel(T* __restrict__ w, long long ldw, long long k0, int bs,
                                                       int* __restrict__ bad) {
  __shared__ T S[NB][NB + 1];  // S[i][j], i >= j
  __shared__ T temp[NB];
  const int i = threadIdx.x;
  T* blk = w + k0 * ldw + k0;
  for (int idx = i; idx < NB * NB; idx += 64) {
    const int r = idx & 63, c = idx >> 6;
    S[r][c] = (r < bs && c <= r) ? blk[(long long)c * ldw + r] : T(0);
  }
  int nz = 0;
  for (int k = 0; k < bs; ++k) {
    __syncthreads();
    if (i < k) temp[i] = mul_rn(S[i][i], S[k][i]);
    __syncthreads();
    if (i >= k && i < bs && k > 0) {
      T acc = i == k ? mul_rn(S[i][0], temp[0]) : add_rn(T(0), mul_rn(S[i][0], temp[0]));
      for (int j = 1; j < k; ++j) acc = add_rn(acc, mul_rn(S[i][j], temp[j]));
      S[i][k] = sub_rn(S[i][k], acc);
    }
    __syncthreads();
    const T d = S[k][k];
    if (i > k && i < bs) {
      const T v = S[i][k];
      if (fabs(d) > T(0)) S[i][k] = div_rn(v, d);
      else if (v != T(0)) nz = 1;
    }
  }
  __syncthreads();
  if (nz) atomicOr(bad, 1);
  for (int idx = i; idx < NB * NB; idx += 64) {
    const int r = idx & 63, c = idx >> 6;
    if (r < bs && c <= r) blk[(long long)c * ldw + r] = S[r][c];
  }
}

// Rows below the diagonal block, one thread per row, in the same order:
// x_jj = A21(r, jj) - (0 + L21(r,0) temp_0(jj) + ...), temp_p(jj) = d_p L11(jj, p), then divided by
// d_jj if it is nonzero (else required to be zero).  L21 is written over A21 and the trailing
// update's second operand tbuf(r, j) = d_j L21(r, j) -- Eigen's temp for row r -- to tbuf (rs x bs,
// leading dimension ldt).  The rows live in shared memory (xs[p][row], conflict-free): a division
// has a slow path that is a call, and 64 of them would spill a register-resident row.
constexpr int PANEL_ROWS = 64;
template <typename T>
struct PanelSmem {
  T Tm[NB][NB + 1];        // Tm[jj][p] = d_p L11(jj, p), p < jj
  T xs[NB][PANEL_ROWS];    // xs[p][row]
  T dv[NB];
};

template <typename T>
__global__ void __launch_bounds__(PANEL_ROWS) ldlt_panel_kernel(T* __restrict__ w, long long ldw, long long k0,
                                                                int bs, long long rs, T* __restrict__ tbuf,
                                                                long long ldt, int* __restrict__ bad) {
  extern __shared__ __align__(16) unsigned char panel_raw[];
  PanelSmem<T>& sm = *reinterpret_cast<PanelSmem<T>*>(panel_raw);
  const int t = threadIdx.x;
  const T* l11 = w + k0 * ldw + k0;
  sm.dv[t] = t < bs ? l11[(long long)t * (ldw + 1)] : T(0);
  __syncthreads();
  for (int idx = t; idx < NB * NB; idx += PANEL_ROWS) {
    const int jj = idx % NB, p = idx / NB;
    T v = T(0);
    if (jj < bs && p < jj) v = mul_rn(sm.dv[p], l11[(long long)p * ldw + jj]);
    sm.Tm[jj][p] = v;
  }
  const long long rbase = (long long)blockIdx.x * PANEL_ROWS;
  T* a21 = w + k0 * ldw + (k0 + bs);  // A21(r, p) at a21[p * ldw + r]
  for (int p = 0; p < NB; ++p) sm.xs[p][t] = (p < bs && rbase + t < rs) ? a21[(long long)p * ldw + rbase + t] : T(0);
  __syncthreads();
  const long long r = rbase + t;
  if (r >= rs) return;
  int nz = 0;
  for (int jj = 0; jj < bs; ++jj) {
    T v = sm.xs[jj][t];
    if (jj > 0) {
      T acc = add_rn(T(0), mul_rn(sm.xs[0][t], sm.Tm[jj][0]));
      for (int p = 1; p < jj; ++p) acc = add_rn(acc, mul_rn(sm.xs[p][t], sm.Tm[jj][p]));
      v = sub_rn(v, acc);
    }
    const T d = sm.dv[jj];
    if (fabs(d) > T(0)) v = div_rn(v, d);
    else if (v != T(0)) nz = 1;
    sm.xs[jj][t] = v;
  }
  for (int p = 0; p < bs; ++p) {
    const T v = sm.xs[p][t];
    a21[(long long)p * ldw + r] = v;
    tbuf[(long long)p * ldt + r] = mul_rn(sm.dv[p], v);
  }
  if (nz) atomicOr(bad, 1);
}

// Sign and success from the pivots (W's diagonal) and the zero-column flag.  One CTA.
template <typename T>
__global__ void __launch_bounds__(1024) ldlt_finish_kernel(const T* __restrict__ w, long long ldw, long long n,
                                                           const int* __restrict__ bad, int* __restrict__ out) {
  __shared__ int s_pos, s_neg;
  __shared__ unsigned long long s_first_zero, s_last_nonzero1;  // last nonzero pivot + 1 (0: none)
  if (threadIdx.x == 0) {
    s_pos = 0;
    s_neg = 0;
    s_first_zero = (unsigned long long)n;
    s_last_nonzero1 = 0;
  }
  __syncthreads();
  int pos = 0, neg = 0;
  long long fz = n, ln = -1;
  for (long long k = threadIdx.x; k < n; k += blockDim.x) {
    const T d = w[k * (ldw + 1)];
    if (d > T(0)) pos = 1;
    if (d < T(0)) neg = 1;
    if (fabs(d) > T(0)) ln = k;
    else if (fz == n) fz = k;
  }
  if (pos) atomicOr(&s_pos, 1);
  if (neg) atomicOr(&s_neg, 1);
  if (fz < n) atomicMin(&s_first_zero, (unsigned long long)fz);
  if (ln >= 0) atomicMax(&s_last_nonzero1, (unsigned long long)(ln + 1));
  __syncthreads();
  if (threadIdx.x == 0) {
    // LDLT.h:389-397: the first nonzero pivot fixes the semidefinite sign, a pivot of the other
    // sign makes it Indefinite; no nonzero pivot leaves ZeroSign
    out[0] = s_pos && s_neg ? 3 : s_pos ? 0 : s_neg ? 1 : 2;
    // LDLT.h:383-387: failure if a zero pivot had a nonzero column or a nonzero pivot followed it
    const bool ok = *bad == 0 && !(s_last_nonzero1 > 0 && s_first_zero + 1 < s_last_nonzero1);
    out[1] = ok ? 0 : 1;
  }
}

// Row permutation of an n x nrhs column-major block: GATHER dst(i) = src(perm[i]), else
// dst(perm[i]) = src(i).
template <typename T, bool GATHER>
__global__ void __launch_bounds__(256) permute_rows_kernel(long long n, int nrhs, const int32_t* __restrict__ perm,
                                                           const T* __restrict__ src, long long lds,
                                                           T* __restrict__ dst, long long ldd) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const long long p = perm[i];
  for (int c = blockIdx.y; c < nrhs; c += gridDim.y) {
    if (GATHER) dst[c * ldd + i] = src[c * lds + p];
    else dst[c * ldd + p] = src[c * lds + i];
  }
}

}  // namespace

namespace {

// Device memory from the stream-ordered pool, returned on scope exit.
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

}  // namespace

template <typename T>
int ldlt_factor_dev(bool upper, int64_t n, T* d_a, int64_t lda, int32_t* transp, int32_t* sign, int64_t* info,
                    cudaStream_t s) {
  if (n == 0) {
    *sign = 2;
    *info = 0;
    return GBLLT_SUCCESS;
  }
  const size_t es = sizeof(T);
  // 1. the pivot order from the diagonal
  std::vector<T> diag(n);
  GB_CUDA_TRY(copy2d_async(diag.data(), es, d_a, (size_t)(lda + 1) * es, es, (size_t)n, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<double> absd(n);
  for (int64_t i = 0; i < n; ++i) absd[i] = std::fabs((double)diag[i]);
  std::vector<int32_t> perm(n);
  pivot_order(n, absd.data(), transp, perm.data());

  // workspace: [W n x n | T21 n x 64 | perm | status | flags]
  const int64_t ldw = n, ldt = n;
  const size_t wb = up256((size_t)n * n * es), vb = up256((size_t)n * NB * es), pb = up256((size_t)n * 4);
  Scratch ws;
  int rc = ws.get(wb + vb + pb + 512, s);
  if (rc) return rc;
  T* W = (T*)ws.p;
  T* Tb = (T*)((char*)ws.p + wb);
  int32_t* d_perm = (int32_t*)((char*)ws.p + wb + vb);
  DevStatus* st = (DevStatus*)((char*)ws.p + wb + vb + pb);
  int* flags = (int*)((char*)st + 256);  // [bad, sign, info]
  GB_CUDA_TRY(cudaMemcpyAsync(d_perm, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(st, 0, 512, s));
  GB_CUDA_TRY(cudaMemsetAsync(&st->fail_col, 0xFF, sizeof(long long), s));

  static const std::string kg = std::string("ldlt_gather_") + tname<T>();
  static const std::string kd = std::string("ldlt_diag_") + tname<T>();
  static const std::string kp = std::string("ldlt_panel_") + tname<T>();
  static const std::string ks = std::string("ldlt_scatter_") + tname<T>();
  const int64_t mt = ceil_div(n, 64);
  const unsigned tiles = (unsigned)(mt * (mt + 1) / 2);
  {  // 2. W = P A P^T
    ProfScope ps(kg.c_str(), s, 0.0, (double)n * (n + 1) * es);
    if (upper) ldlt_gather_kernel<T, true><<<tiles, 256, 0, s>>>(d_a, lda, n, d_perm, W, ldw);
    else ldlt_gather_kernel<T, false><<<tiles, 256, 0, s>>>(d_a, lda, n, d_perm, W, ldw);
  }
  // 3. blocked LDL^T without pivoting.  FP64 from kTensorSyrkMinN on: the trailing update
  //    W22 -= L21 (L21 D)^T on the tensor cores, FP64-exact (both operands sliced, ozaki.cu)
  OzakiSyrk oz;
  bool use_oz = false;
  if constexpr (sizeof(T) == 8) {
    if (n >= kTensorSyrkMinN) {
      const int rc2 = oz.init(n, s, true);
      if (rc2 == GBLLT_SUCCESS) use_oz = true;
      else if (rc2 != GBLLT_ERR_ALLOC) return rc2;
    }
  }
  for (int64_t k0 = 0; k0 < n; k0 += NB) {
    const int bs = (int)(n - k0 < NB ? n - k0 : NB);
    const int64_t rs = n - k0 - bs;
    {
      ProfScope ps(kd.c_str(), s, (double)bs * bs * bs / 3.0, (double)bs * (bs + 1) * es);
      ldlt_diag_kernel<T><<<1, 64, 0, s>>>(W, ldw, k0, bs, flags);
    }
    if (rs > 0) {
      {
        ProfScope ps(kp.c_str(), s, (double)rs * bs * bs, (3.0 * rs * bs + 0.5 * bs * bs) * es);
        const int smem = (int)sizeof(PanelSmem<T>);
        cudaFuncSetAttribute(ldlt_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        ldlt_panel_kernel<T><<<(unsigned)ceil_div(rs, PANEL_ROWS), PANEL_ROWS, smem, s>>>(W, ldw, k0, bs, rs, Tb,
                                                                                         ldt, flags);
      }
      if constexpr (sizeof(T) == 8) {
        if (use_oz) {
          if ((rc = oz.update_pq(W, ldw, k0, bs, rs, Tb, ldt, st, s))) return rc;
          continue;
        }
      }
      launch_syrk_lower<T>(W, ldw, k0, bs, rs, rs, st, s, Tb, ldt);
    }
  }
  // 4. sign and success, 5. the factor back into the caller's triangle
  ldlt_finish_kernel<T><<<1, 1024, 0, s>>>(W, ldw, n, flags, flags + 1);
  {
    ProfScope ps(ks.c_str(), s, 0.0, (double)n * (n + 1) * es);
    if (upper) ldlt_scatter_kernel<T, true><<<tiles, 256, 0, s>>>(W, ldw, n, d_a, lda);
    else ldlt_scatter_kernel<T, false><<<tiles, 256, 0, s>>>(W, ldw, n, d_a, lda);
  }
  GB_CUDA_TRY(cudaGetLastError());
  int out[2] = {0, 0};
  DevStatus hst;
  GB_CUDA_TRY(cudaMemcpyAsync(out, flags + 1, sizeof out, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&hst, st, sizeof hst, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (hst.timeout) return GBLLT_ERR_TIMEOUT;  // a bounded wait of the tensor-core update ran out
  *sign = out[0];
  *info = out[1];
  return GBLLT_SUCCESS;
}

template <typename T>
int ldlt_solve_dev(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, const int32_t* transp, T* d_b,
                   int64_t ldb, cudaStream_t s) {
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  std::vector<int32_t> perm;
  if (perm_from_transpositions(n, transp, perm)) {
    set_error_message("transposition index out of range");
    return GBLLT_ERR_INTERNAL;
  }
  const size_t es = sizeof(T);
  const size_t pb = up256((size_t)n * 4), tb = up256((size_t)n * nrhs * es);
  Scratch ws;
  int rc = ws.get(pb + tb + potrs_ws_bytes(n, es), s);
  if (rc) return rc;
  int32_t* d_perm = (int32_t*)ws.p;
  T* tmp = (T*)((char*)ws.p + pb);
  void* sw = (char*)ws.p + pb + tb;
  GB_CUDA_TRY(cudaMemcpyAsync(d_perm, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
  const dim3 grid((unsigned)ceil_div(n, 256), (unsigned)(nrhs < 64 ? nrhs : 64));
  permute_rows_kernel<T, true><<<grid, 256, 0, s>>>(n, (int)nrhs, d_perm, d_b, ldb, tmp, n);
  if ((rc = ldlt_sweeps_ws<T>(upper, n, nrhs, d_a, lda, tmp, n, sw, s))) return rc;
  permute_rows_kernel<T, false><<<grid, 256, 0, s>>>(n, (int)nrhs, d_perm, tmp, n, d_b, ldb);
  // (a copy from pageable host memory has taken its data when cudaMemcpyAsync returns, so the
  // host perm vector may go)
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template int ldlt_factor_dev<double>(bool, int64_t, double*, int64_t, int32_t*, int32_t*, int64_t*, cudaStream_t);
template int ldlt_factor_dev<float>(bool, int64_t, float*, int64_t, int32_t*, int32_t*, int64_t*, cudaStream_t);
template int ldlt_solve_dev<double>(bool, int64_t, int64_t, const double*, int64_t, const int32_t*, double*, int64_t,
                                    cudaStream_t);
template int ldlt_solve_dev<float>(bool, int64_t, int64_t, const float*, int64_t, const int32_t*, float*, int64_t,
                                   cudaStream_t);

namespace {

inline bool upper_of(char uplo) { return uplo == 'U' || uplo == 'u'; }

template <typename T>
int host_ldlt(int layout, char uplo, int64_t n, T* a, int64_t lda, int32_t* transp, int32_t* sign, int64_t* info) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (n > 0 && !a) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (n > 0 && !transp) return -6;
  if (!sign) return -7;
  if (!info) return -8;
  if (n == 0) {
    *sign = 2;
    *info = 0;
    return GBLLT_SUCCESS;
  }
  int rc = ensure_device();
  if (rc) return rc;
  // a row-major lower triangle is a column-major upper one
  const bool upper = upper_of(uplo) != (layout == GBLLT_ROW_MAJOR);
  cudaStream_t s = lib_stream();
  const size_t es = sizeof(T);
  Scratch buf;
  if ((rc = buf.get((size_t)n * n * es, s))) return rc;
  T* d_a = (T*)buf.p;
  GB_CUDA_TRY(copy2d_async(d_a, n * es, a, lda * es, n * es, n, cudaMemcpyHostToDevice, s));
  if ((rc = ldlt_factor_dev<T>(upper, n, d_a, n, transp, sign, info, s))) return rc;
  GB_CUDA_TRY(copy2d_async(a, lda * es, d_a, n * es, n * es, n, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBLLT_SUCCESS;
}

template <typename T>
int dev_ldlt(char uplo, int64_t n, T* d_a, int64_t lda, int32_t* transp, int32_t* sign, int64_t* info, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (n > 0 && !d_a) return -3;
  if (lda < (n > 1 ? n : 1)) return -4;
  if (n > 0 && !transp) return -5;
  if (!sign) return -6;
  if (!info) return -7;
  if (n == 0) {
    *sign = 2;
    *info = 0;
    return GBLLT_SUCCESS;
  }
  int rc = ensure_device();
  if (rc) return rc;
  return ldlt_factor_dev<T>(upper_of(uplo), n, d_a, lda, transp, sign, info, (cudaStream_t)stream);
}

int check_transp(int64_t n, const int32_t* transp) {
  for (int64_t k = 0; k < n; ++k)
    if (transp[k] < 0 || transp[k] >= n) return -1;
  return 0;
}

template <typename T>
int host_ldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const T* a, int64_t lda, const int32_t* transp,
                    T* b, int64_t ldb) {
  if (layout != GBLLT_ROW_MAJOR && layout != GBLLT_COL_MAJOR) return -1;
  if (check_uplo(uplo)) return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (n > 0 && !a) return -5;
  if (lda < (n > 1 ? n : 1)) return -6;
  if (n > 0 && (!transp || check_transp(n, transp))) return -7;
  if (n > 0 && nrhs > 0 && !b) return -8;
  const bool rowmajor = layout == GBLLT_ROW_MAJOR;
  const int64_t minldb = rowmajor ? (nrhs > 1 ? nrhs : 1) : (n > 1 ? n : 1);
  if (ldb < minldb) return -9;
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  const bool upper = upper_of(uplo) != rowmajor;
  cudaStream_t s = lib_stream();
  const size_t es = sizeof(T);
  const size_t ab = up256((size_t)n * n * es), bb = up256((size_t)n * nrhs * es);
  Scratch buf;
  if ((rc = buf.get(ab + 2 * bb, s))) return rc;
  T* d_a = (T*)buf.p;
  T* d_b = (T*)((char*)buf.p + ab);
  T* d_t = (T*)((char*)buf.p + ab + bb);
  GB_CUDA_TRY(copy2d_async(d_a, n * es, a, lda * es, n * es, n, cudaMemcpyHostToDevice, s));
  if (!rowmajor) {
    GB_CUDA_TRY(copy2d_async(d_b, n * es, b, ldb * es, n * es, nrhs, cudaMemcpyHostToDevice, s));
  } else {  // row-major B (n x nrhs) seen column-major is B^T
    GB_CUDA_TRY(copy2d_async(d_t, nrhs * es, b, ldb * es, nrhs * es, n, cudaMemcpyHostToDevice, s));
    if ((rc = transpose_dev<T>(nrhs, n, d_t, nrhs, d_b, n, s))) return rc;
  }
  if ((rc = ldlt_solve_dev<T>(upper, n, nrhs, d_a, n, transp, d_b, n, s))) return rc;
  if (!rowmajor) {
    GB_CUDA_TRY(copy2d_async(b, ldb * es, d_b, n * es, n * es, nrhs, cudaMemcpyDeviceToHost, s));
  } else {
    if ((rc = transpose_dev<T>(n, nrhs, d_b, n, d_t, nrhs, s))) return rc;
    GB_CUDA_TRY(copy2d_async(b, ldb * es, d_t, nrhs * es, nrhs * es, n, cudaMemcpyDeviceToHost, s));
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBLLT_SUCCESS;
}

template <typename T>
int dev_ldlt_solve(char uplo, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, const int32_t* transp, T* d_b,
                   int64_t ldb, void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (n > 0 && !d_a) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (n > 0 && (!transp || check_transp(n, transp))) return -6;
  if (n > 0 && nrhs > 0 && !d_b) return -7;
  if (ldb < (n > 1 ? n : 1)) return -8;
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return ldlt_solve_dev<T>(upper_of(uplo), n, nrhs, d_a, lda, transp, d_b, ldb, (cudaStream_t)stream);
}

}  // namespace
}  // namespace gbllt

using namespace gbllt;

extern "C" {

int gbllt_dldlt(int layout, char uplo, int64_t n, double* a, int64_t lda, int32_t* transp, int32_t* sign,
                int64_t* info) {
  return host_ldlt<double>(layout, uplo, n, a, lda, transp, sign, info);
}
int gbllt_sldlt(int layout, char uplo, int64_t n, float* a, int64_t lda, int32_t* transp, int32_t* sign,
                int64_t* info) {
  return host_ldlt<float>(layout, uplo, n, a, lda, transp, sign, info);
}
int gbllt_dldlt_pivots(int64_t n, const double* diag, int64_t incd, int32_t* transp) {
  if (n < 0) return -1;
  if (n > 0 && !diag) return -2;
  if (incd < 1) return -3;
  if (n > 0 && !transp) return -4;
  std::vector<double> absd(n);
  std::vector<int32_t> perm(n);
  for (int64_t i = 0; i < n; ++i) absd[i] = std::fabs(diag[i * incd]);
  pivot_order(n, absd.data(), transp, perm.data());
  return GBLLT_SUCCESS;
}
int gbllt_sldlt_pivots(int64_t n, const float* diag, int64_t incd, int32_t* transp) {
  if (n < 0) return -1;
  if (n > 0 && !diag) return -2;
  if (incd < 1) return -3;
  if (n > 0 && !transp) return -4;
  std::vector<double> absd(n);
  std::vector<int32_t> perm(n);
  for (int64_t i = 0; i < n; ++i) absd[i] = std::fabs((double)diag[i * incd]);
  pivot_order(n, absd.data(), transp, perm.data());
  return GBLLT_SUCCESS;
}
int gbllt_dldlt_dev(char uplo, int64_t n, double* d_a, int64_t lda, int32_t* transp, int32_t* sign, int64_t* info,
                    void* stream) {
  return dev_ldlt<double>(uplo, n, d_a, lda, transp, sign, info, stream);
}
int gbllt_sldlt_dev(char uplo, int64_t n, float* d_a, int64_t lda, int32_t* transp, int32_t* sign, int64_t* info,
                    void* stream) {
  return dev_ldlt<float>(uplo, n, d_a, lda, transp, sign, info, stream);
}
int gbllt_dldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda,
                      const int32_t* transp, double* b, int64_t ldb) {
  return host_ldlt_solve<double>(layout, uplo, n, nrhs, a, lda, transp, b, ldb);
}
int gbllt_sldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda,
                      const int32_t* transp, float* b, int64_t ldb) {
  return host_ldlt_solve<float>(layout, uplo, n, nrhs, a, lda, transp, b, ldb);
}
int gbllt_dldlt_solve_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda, const int32_t* transp,
                          double* d_b, int64_t ldb, void* stream) {
  return dev_ldlt_solve<double>(uplo, n, nrhs, d_a, lda, transp, d_b, ldb, stream);
}
int gbllt_sldlt_solve_dev(char uplo, int64_t n, int64_t nrhs, const float* d_a, int64_t lda, const int32_t* transp,
                          float* d_b, int64_t ldb, void* stream) {
  return dev_ldlt_solve<float>(uplo, n, nrhs, d_a, lda, transp, d_b, ldb, stream);
}

}  // extern "C"
