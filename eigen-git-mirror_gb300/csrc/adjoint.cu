// Reverse mode (adjoint) of the Cholesky factorisation and of the two-sweep solve, FP64.
//
// Forward (what is differentiated): the blocked factorisation of llt_inplace::blocked
// (Eigen/src/Cholesky/LLT.h:338-368), written per block J (rows I below it, columns K left of it):
//     D' = A_JJ - L_JK L_JK^T ; L_JJ = chol(D') ; C' = A_IJ - L_IK L_JK^T ; L_IJ = C' L_JJ^{-T}
// and the solve x = L^{-T} L^{-1} b (LLT.h:483-498).
//
// Reverse of the factorisation, blocks J from last to first, in place on the adjoint array M
// (holding Lbar on entry, Abar on exit; only L and M are read -- panels are recomputed from L, no
// forward intermediates are stored):
//     Cbar  = M_IJ L_JJ^{-1}                       (right triangular solve)
//     M_JJ -= tril(Cbar^T L_IJ)                    (adjoint of L_JJ through L_IJ = C' L_JJ^{-T})
//     M_IJ  = Cbar / 2                             (= Abar_IJ: each off-diagonal entry of the
//                                                   symmetric A is shared by (i,j) and (j,i))
//     M_IK -= Cbar L_JK ;  M_JK -= Cbar^T L_IK      (adjoint of C' = A_IJ - L_IK L_JK^T)
//     Dbar  = 1/2 L_JJ^{-T} (P + P^T) L_JJ^{-1},  P = Phi(L_JJ^T M_JJ)   (diagonal block)
//     M_JJ  = Dbar ;  M_JK -= 2 Dbar L_JK          (adjoint of D' = A_JJ - L_JK L_JK^T)
// where Phi takes the lower triangle and halves the diagonal.  The result is the symmetric Abar
// with df = sum_ij Abar_ij dA_ij for symmetric perturbations dA (its lower triangle is stored).
// The symbolic form of the same result, Abar = 1/2 L^{-T} (P + P^T) L^{-1} with P = Phi(L^T Lbar),
// is Murray 2016 ("Differentiation of the Cholesky decomposition", arXiv:1602.07527); the blocked
// in-place order above does about 2n^3/3 flops (twice the forward factorisation), nearly all of them
// in the two products with the panel below each block (M_IK and M_JK updates).
//
// Reverse of the solve X = A^{-1} B:  Bbar = A^{-1} Xbar,  Abar -= sym(Bbar X^T).
#include <algorithm>

#include "internal.h"

namespace gbllt {

namespace {

constexpr int ANB = 32;  // block size of the adjoint

// ---- general FP64 GEMM:  C (m x n) += alpha * op(A) * op(B), column-major ----------------------
// opA: 0 = A (m x k), 1 = A^T (A stored k x m), 2 = A symmetric m x m stored in its lower triangle.
// opB: 0 = B (k x n), 1 = B^T (B stored n x k).
// lower_only: write only entries with global row >= column (row/col offsets applied by the caller).
// Tiles of TM x 64 (TM = 32 for the 32-row products of the block adjoint, else 64).  Split K: with
// gridDim.z > 1, CTA z covers k in [z*kc, (z+1)*kc) and stores alpha * its partial product densely
// in part[z] (m x n, leading dimension m); split_reduce_kernel then adds the partials into C in a
// fixed order, so the result does not depend on scheduling.
template <int OPA, int OPB, int TM>
__global__ void __launch_bounds__(256) gemm_f64_kernel(long long m, long long n, long long k, long long kc, double alpha,
                                                       const double* __restrict__ A, long long lda,
                                                       const double* __restrict__ B, long long ldb,
                                                       double* __restrict__ C, long long ldc, int lower_only,
                                                       double* __restrict__ part) {
  constexpr int KC = 32, RT = TM / 16;
  __shared__ double As[KC][TM + 1];  // As[p][i] = op(A)(i0 + i, p0 + p)
  __shared__ double Bs[KC][64 + 1];  // Bs[p][j] = op(B)(p0 + p, j0 + j)
  const long long i0 = (long long)blockIdx.x * TM, j0 = (long long)blockIdx.y * 64;
  if (lower_only && i0 + TM - 1 < j0) return;  // tile strictly above the diagonal
  const long long kb = (long long)blockIdx.z * kc;
  const long long ke = kb + kc < k ? kb + kc : k;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[RT][4];
#pragma unroll
  for (int u = 0; u < RT; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
  for (long long p0 = kb; p0 < ke; p0 += KC) {
    for (int idx = tid; idx < TM * KC; idx += 256) {
      int i, p;
      if (OPA == 1) { p = idx & 31; i = idx >> 5; }   // A^T: contiguous along p
      else          { i = idx % TM; p = idx / TM; }   // A: contiguous along i
      const long long gi = i0 + i, gp = p0 + p;
      double v = 0.0;
      if (gi < m && gp < ke) {
        if (OPA == 0) v = A[gp * lda + gi];
        else if (OPA == 1) v = A[gi * lda + gp];
        else v = gi >= gp ? A[gp * lda + gi] : A[gi * lda + gp];
      }
      As[p][i] = v;
    }
    for (int idx = tid; idx < 64 * KC; idx += 256) {
      int j, p;
      if (OPB == 0) { p = idx & 31; j = idx >> 5; }   // B: contiguous along p
      else          { j = idx & 63; p = idx >> 6; }   // B^T: contiguous along j
      const long long gj = j0 + j, gp = p0 + p;
      double v = 0.0;
      if (gj < n && gp < ke) v = OPB == 0 ? B[gj * ldb + gp] : B[gp * ldb + gj];
      Bs[p][j] = v;
    }
    __syncthreads();
    const int pe = (int)(ke - p0 < KC ? ke - p0 : KC);
    for (int p = 0; p < pe; ++p) {
      double av[RT], bv[4];
#pragma unroll
      for (int u = 0; u < RT; ++u) av[u] = As[p][tx + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = Bs[p][ty + 16 * v];
#pragma unroll
      for (int u = 0; u < RT; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(av[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
  double* P = part ? part + (long long)blockIdx.z * m * n : nullptr;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const long long j = j0 + ty + 16 * v;
#pragma unroll
    for (int u = 0; u < RT; ++u) {
      const long long i = i0 + tx + 16 * u;
      if (i < m && j < n && (!lower_only || i >= j)) {
        if (P) P[j * m + i] = alpha * acc[u][v];
        else C[j * ldc + i] += alpha * acc[u][v];
      }
    }
  }
}

// C(i, j) += sum_z part[z](i, j) over the nz partials, z ascending.
__global__ void split_reduce_kernel(long long m, long long n, int nz, const double* __restrict__ part,
                                    double* __restrict__ C, long long ldc, int lower_only) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  const long long i = idx % m, j = idx / m;
  if (lower_only && i < j) return;
  double s = 0.0;
  for (int z = 0; z < nz; ++z) s += part[(long long)z * m * n + idx];
  C[j * ldc + i] += s;
}

// X L = M for X, then M <- X / 2, in place (rows x ANB), L lower jb x jb: one thread per row,
// columns descending.  The halving converts the adjoint of the independent lower entries of A_IJ
// into the symmetric-gradient convention (each off-diagonal entry stands for two symmetric ones).
__global__ void __launch_bounds__(64) trsm_right_lower_kernel(const double* __restrict__ L, long long ldl, int jb,
                                                               double* __restrict__ M, long long ldm, long long rows) {
  __shared__ double Ls[ANB][ANB + 1];  // Ls[p][c] = L(p, c)
  for (int idx = threadIdx.x; idx < ANB * ANB; idx += 64) {
    const int p = idx % ANB, c = idx / ANB;
    Ls[p][c] = (p < jb && c < jb && p >= c) ? L[(long long)c * ldl + p] : (p == c ? 1.0 : 0.0);
  }
  __syncthreads();
  const long long r = (long long)blockIdx.x * 64 + threadIdx.x;
  if (r >= rows) return;
  double x[ANB];
#pragma unroll
  for (int c = 0; c < ANB; ++c) x[c] = c < jb ? M[(long long)c * ldm + r] : 0.0;
#pragma unroll
  for (int c = ANB - 1; c >= 0; --c) {
    double v = x[c];
#pragma unroll
    for (int p = c + 1; p < ANB; ++p) v = fma(-x[p], Ls[p][c], v);
    x[c] = v / Ls[c][c];
  }
#pragma unroll
  for (int c = 0; c < ANB; ++c)
    if (c < jb) M[(long long)c * ldm + r] = 0.5 * x[c];
}

// Diagonal block: Mjj (lower, holding Lbar_JJ) <- lower( 1/2 L^{-T} (P + P^T) L^{-1} ), P = Phi(L^T Lbar).
__global__ void __launch_bounds__(256) chol_adjoint_diag_kernel(const double* __restrict__ L, long long ldl, int jb,
                                                                double* __restrict__ Mjj, long long ldm) {
  __shared__ double Ls[ANB][ANB + 1];   // L(i, j)
  __shared__ double Lb[ANB][ANB + 1];   // Lbar(i, j), lower
  __shared__ double S[ANB][ANB + 1];    // work
  const int tid = threadIdx.x;
  for (int idx = tid; idx < ANB * ANB; idx += 256) {
    const int i = idx % ANB, j = idx / ANB;
    const bool in = i < jb && j < jb && i >= j;
    Ls[i][j] = in ? L[(long long)j * ldl + i] : (i == j ? 1.0 : 0.0);
    Lb[i][j] = in ? Mjj[(long long)j * ldm + i] : 0.0;
  }
  __syncthreads();
  // P = Phi(L^T Lbar): C(i, j) = sum_k L(k, i) Lbar(k, j), k >= max(i, j); keep i >= j, halve the diagonal
  for (int idx = tid; idx < ANB * ANB; idx += 256) {
    const int i = idx % ANB, j = idx / ANB;
    double c = 0.0;
    if (i >= j)
      for (int kk = i; kk < ANB; ++kk) c = fma(Ls[kk][i], Lb[kk][j], c);
    S[i][j] = i > j ? c : (i == j ? 0.5 * c : 0.0);
  }
  __syncthreads();
  // S <- P + P^T (symmetric)
  for (int idx = tid; idx < ANB * ANB; idx += 256) {
    const int i = idx % ANB, j = idx / ANB;
    if (i > j) S[j][i] = S[i][j];
    else if (i == j) S[i][i] = 2.0 * S[i][i];
  }
  __syncthreads();
  // Y = L^{-T} S: solve L^T Y = S column by column of S (thread per column), rows descending
  if (tid < ANB) {
    const int c = tid;
    for (int r = ANB - 1; r >= 0; --r) {
      double v = S[r][c];
      for (int p = r + 1; p < ANB; ++p) v = fma(-Ls[p][r], S[p][c], v);
      S[r][c] = v / Ls[r][r];
    }
  }
  __syncthreads();
  // D = 1/2 Y L^{-1}: solve D L = Y/2 row by row (thread per row), columns descending
  if (tid < ANB) {
    const int r = tid;
    for (int c = ANB - 1; c >= 0; --c) {
      double v = 0.5 * S[r][c];
      for (int p = c + 1; p < ANB; ++p) v = fma(-S[r][p], Ls[p][c], v);
      S[r][c] = v / Ls[c][c];
    }
  }
  __syncthreads();
  for (int idx = tid; idx < ANB * ANB; idx += 256) {
    const int i = idx % ANB, j = idx / ANB;
    if (i < jb && j < jb && i >= j) Mjj[(long long)j * ldm + i] = 0.5 * (S[i][j] + S[j][i]);
  }
}

// Split-K scratch: partial products of at most kSplitElems doubles.
constexpr long long kSplitElems = 1ll << 21;  // 16 MiB
constexpr int kTargetCtas = 2 * 152;          // two waves of CTAs over the 152 SMs

template <int OPA, int OPB>
void gemm(long long m, long long n, long long k, double alpha, const double* A, long long lda, const double* B,
          long long ldb, double* C, long long ldc, bool lower_only, double* part, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return;
  static const std::string kname = "adjoint_gemm_f64";
  ProfScope ps(kname.c_str(), s, 2.0 * m * n * k * (lower_only ? 0.5 : 1.0), 8.0 * (m * k + k * n + 2 * m * n));
  const int tm = m <= 32 ? 32 : 64;
  const long long tiles = ceil_div(m, tm) * ceil_div(n, 64);
  // split K when the output alone gives too few CTAs and each split keeps >= 64 of K
  long long nz = 1;
  if (part && tiles < kTargetCtas) {
    nz = std::min<long long>(kTargetCtas / tiles, k / 64);
    while (nz > 1 && nz * m * n > kSplitElems) --nz;
    if (nz < 1) nz = 1;
  }
  const long long kc = nz > 1 ? ceil_div(ceil_div(k, nz), 32) * 32 : k;
  nz = ceil_div(k, kc);
  double* P = nz > 1 ? part : nullptr;
  dim3 grid((unsigned)ceil_div(m, tm), (unsigned)ceil_div(n, 64), (unsigned)nz);
  const int lo = lower_only ? 1 : 0;
  if (tm == 32) gemm_f64_kernel<OPA, OPB, 32><<<grid, 256, 0, s>>>(m, n, k, kc, alpha, A, lda, B, ldb, C, ldc, lo, P);
  else gemm_f64_kernel<OPA, OPB, 64><<<grid, 256, 0, s>>>(m, n, k, kc, alpha, A, lda, B, ldb, C, ldc, lo, P);
  if (P) split_reduce_kernel<<<(unsigned)ceil_div(m * n, 256), 256, 0, s>>>(m, n, (int)nz, P, C, ldc, lo);
}

__global__ void sym_rank_update_kernel(long long n, long long nrhs, const double* __restrict__ X, long long ldx,
                                       const double* __restrict__ Bb, long long ldbb, double* __restrict__ Ab,
                                       long long ldab) {
  // Abar(i, j) -= 1/2 sum_c (Bbar(i,c) X(j,c) + X(i,c) Bbar(j,c)) for i >= j
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const long long i = idx % n, j = idx / n;
  if (i < j) return;
  double s = 0.0;
  for (long long c = 0; c < nrhs; ++c)
    s += Bb[c * ldbb + i] * X[c * ldx + j] + X[c * ldx + i] * Bb[c * ldbb + j];
  Ab[j * ldab + i] -= 0.5 * s;
}

// W (jb x (n - j0), row a contiguous over r, leading dimension ldw) = [sym(M_JJ); M_IJ]^T for the panel
// at j0: for r < jb the symmetric matrix whose lower triangle is M_JJ's, below it M_IJ.
__global__ void build_panel_w_kernel(const double* __restrict__ M, long long ldm, long long j0, int jb, long long n,
                                     double* __restrict__ W, long long ldw) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (r >= n - j0 || a >= jb) return;
  double v;
  if (r < jb) v = r >= a ? M[(j0 + a) * ldm + j0 + r] : M[(j0 + r) * ldm + j0 + a];
  else v = M[(j0 + a) * ldm + j0 + r];
  W[(long long)a * ldw + r] = v;
}

// A bounded wait of a tensor-core product ran out: the gradient is invalid, and its lower triangle
// becomes NaN so that a stream-ordered caller sees it.
__global__ void nan_if_error_kernel(const int* __restrict__ err, long long n, double* __restrict__ M, long long ldm) {
  if (*(volatile const int*)err == 0) return;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const long long i = idx % n, j = idx / n;
  if (i >= j) M[j * ldm + i] = __longlong_as_double(0x7ff8000000000000ll);
}

constexpr int APW = 64;      // panel width of the reverse sweep (two 32-wide blocks)
constexpr int64_t KC2 = 2048;  // rows of L per product of the panel-row update (bounds the slices)

}  // namespace

// The reverse sweep in 64-wide panels, last to first.  Inside a panel the 32-wide blocks run the
// per-block recurrences above with their column range K restricted to the panel; what each block
// would add into the columns left of the panel is linear in the panel's final values, and is added
// after the panel as two products on the tensor cores (OzakiGemm; nsl = 8: FP64-exact, nsl = 4: the
// 28-bit products of the mixed-precision adjoint):
//     M_IK -= 2 M_IJ L_JK                      (rows I below the panel; M_IJ holds Cbar / 2)
//     M_JK -= 2 W^T L_RK,  W = [sym(M_JJ); M_IJ] (the panel's rows; R = the rows from the panel down)
// where sym(M_JJ) collects, through the symmetric matrix whose lower triangle M_JJ holds, the
// products with the panel's own blocks: Cbar^T of the blocks below, Dbar on the diagonal, Cbar of the
// blocks above.  The in-panel work stays on the FP64 pipe (about 2 n^2 * 64 flops); the products with
// the panel (2 n^3 / 3) run on the tensor cores.
int potrf_adjoint_dev(int64_t n, const double* L, int64_t ldl, double* M, int64_t ldm, cudaStream_t s, int nsl) {
  static const std::string kt = "adjoint_trsm_f64", kd = "adjoint_diag_f64";
  const size_t pb = (size_t)kSplitElems * sizeof(double);
  const size_t g1b = (OzakiGemm::bytes(n, n, APW) + 255) & ~(size_t)255;
  const int64_t kc2 = n < KC2 ? n : KC2;
  const size_t g2b = (OzakiGemm::bytes(APW, n, kc2) + 255) & ~(size_t)255;
  const int64_t ldw = (n + 31) / 32 * 32;
  const size_t wb = (size_t)APW * ldw * sizeof(double);
  char* ws = nullptr;
  if (dev_malloc_async((void**)&ws, pb + g1b + g2b + wb + 256, s) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("gbllt_dpotrf_adjoint_dev: cudaMallocAsync of the workspace failed");
    return GBLLT_ERR_ALLOC;
  }
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{ws, s};
  double* part = (double*)ws;  // split-K partials of the long, narrow in-panel products
  OzakiGemm g1, g2;
  int rc;
  if ((rc = g1.attach(ws + pb, n, n, APW)) || (rc = g2.attach(ws + pb + g1b, APW, n, kc2))) return rc;
  double* W = (double*)(ws + pb + g1b + g2b);
  int* err = (int*)(ws + pb + g1b + g2b + wb);
  GB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  const int64_t last = ((n - 1) / APW) * APW;
  for (int64_t p0 = last; p0 >= 0; p0 -= APW) {
    const int pw = (int)(n - p0 < APW ? n - p0 : APW);
    // ---- the panel's blocks, last to first, columns K restricted to [p0, j0)
    for (int64_t j0 = p0 + ((pw - 1) / ANB) * ANB; j0 >= p0; j0 -= ANB) {
      const int jb = (int)(n - j0 < ANB ? n - j0 : ANB);
      const int64_t i0 = j0 + jb, ni = n - i0;  // rows below the block
      const int64_t kw = j0 - p0;               // columns of the panel left of the block
      const double* Ljj = L + j0 * ldl + j0;
      const double* Lij = L + j0 * ldl + i0;
      const double* Ljk = L + p0 * ldl + j0;   // rows J, columns p0 .. j0
      const double* Lik = L + p0 * ldl + i0;   // rows I, columns p0 .. j0
      double* Mjj = M + j0 * ldm + j0;
      double* Mij = M + j0 * ldm + i0;
      double* Mjk = M + p0 * ldm + j0;
      double* Mik = M + p0 * ldm + i0;
      if (ni > 0) {
        {
          ProfScope ps(kt.c_str(), s, (double)ni * jb * jb, 16.0 * ni * jb);
          trsm_right_lower_kernel<<<(unsigned)ceil_div(ni, 64), 64, 0, s>>>(Ljj, ldl, jb, Mij, ldm, ni);  // Cbar/2
        }
        // M_IJ now holds Cbar / 2 (its final, symmetric-convention value); the updates use Cbar = 2 M_IJ
        gemm<1, 0>(jb, jb, ni, -2.0, Mij, ldm, Lij, ldl, Mjj, ldm, true, part, s);        // M_JJ -= tril(Cbar^T L_IJ)
        if (kw > 0) {
          gemm<0, 0>(ni, kw, jb, -2.0, Mij, ldm, Ljk, ldl, Mik, ldm, false, part, s);     // M_IK -= Cbar L_JK
          gemm<1, 0>(jb, kw, ni, -2.0, Mij, ldm, Lik, ldl, Mjk, ldm, false, part, s);     // M_JK -= Cbar^T L_IK
        }
      }
      {
        ProfScope ps(kd.c_str(), s, 4.0 * jb * jb * jb, 24.0 * jb * jb);
        chol_adjoint_diag_kernel<<<1, 256, 0, s>>>(Ljj, ldl, jb, Mjj, ldm);          // Dbar
      }
      if (kw > 0) gemm<2, 0>(jb, kw, jb, -2.0, Mjj, ldm, Ljk, ldl, Mjk, ldm, false, part, s);  // M_JK -= 2 Dbar L_JK
    }
    if (p0 == 0) break;
    // ---- the columns left of the panel, on the tensor cores
    const int64_t r0 = p0 + pw, nr = n - r0;  // rows below the panel
    // M_IK -= 2 M_IJ L_JK: P = M_IJ (element (i, a) = M(r0 + i, p0 + a)), Q = L_JK^T (element
    // (k, a) = L(p0 + a, k))
    if (nr > 0 && (rc = g1.run(M + r0, ldm, nr, p0, pw, M + p0 * ldm + r0, 1, ldm, L + p0, ldl, 1, 1, err, s, nsl)))
      return rc;
    // M_JK -= 2 W^T L_RK in chunks of rows of R: P = W^T (element (a, r) = W[a ldw + r]), Q = L_RK^T
    // (element (k, r) = L(p0 + r, k))
    {
      const dim3 g((unsigned)ceil_div(n - p0, 256), (unsigned)pw);
      build_panel_w_kernel<<<g, 256, 0, s>>>(M, ldm, p0, pw, n, W, ldw);
    }
    for (int64_t c0 = 0; c0 < n - p0; c0 += kc2) {
      const int64_t kc = n - p0 - c0 < kc2 ? n - p0 - c0 : kc2;
      if ((rc = g2.run(M + p0, ldm, pw, p0, kc, W + c0, ldw, 1, L + p0 + c0, ldl, 1, 1, err, s, nsl))) return rc;
    }
  }
  nan_if_error_kernel<<<(unsigned)ceil_div(n * n, 256), 256, 0, s>>>(err, n, M, ldm);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

int potrs_adjoint_dev(int64_t n, int64_t nrhs, const double* L, int64_t ldl, const double* X, int64_t ldx,
                      const double* Xb, int64_t ldxb, double* Bb, int64_t ldbb, double* Ab, int64_t ldab,
                      cudaStream_t s) {
  // Bbar = A^{-1} Xbar (the same two sweeps as the forward solve)
  GB_CUDA_TRY(copy2d_async(Bb, ldbb * 8, Xb, ldxb * 8, n * 8, nrhs, cudaMemcpyDeviceToDevice, s));
  int rc = potrs_dev<double>(false, n, nrhs, L, ldl, Bb, ldbb, s);
  if (rc) return rc;
  if (Ab) {
    static const std::string kn = "adjoint_symupdate_f64";
    ProfScope ps(kn.c_str(), s, 2.0 * n * n * nrhs, 8.0 * (n * n + 2.0 * n * nrhs));
    sym_rank_update_kernel<<<(unsigned)ceil_div(n * n, 256), 256, 0, s>>>(n, nrhs, X, ldx, Bb, ldbb, Ab, ldab);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace gbllt

using namespace gbllt;

extern "C" {

int gbllt_dpotrf_adjoint_dev(int64_t n, const double* d_l, int64_t ldl, double* d_lbar, int64_t ldlb, void* stream) {
  if (n < 0) return -1;
  if (n > 0 && !d_l) return -2;
  if (ldl < (n > 1 ? n : 1)) return -3;
  if (n > 0 && !d_lbar) return -4;
  if (ldlb < (n > 1 ? n : 1)) return -5;
  if (n == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return potrf_adjoint_dev(n, d_l, ldl, d_lbar, ldlb, (cudaStream_t)stream, 8);
}

int gbllt_dpotrf_adjoint_mixed_dev(int64_t n, const double* d_l, int64_t ldl, double* d_lbar, int64_t ldlb,
                                   void* stream) {
  if (n < 0) return -1;
  if (n > 0 && !d_l) return -2;
  if (ldl < (n > 1 ? n : 1)) return -3;
  if (n > 0 && !d_lbar) return -4;
  if (ldlb < (n > 1 ? n : 1)) return -5;
  if (n == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return potrf_adjoint_dev(n, d_l, ldl, d_lbar, ldlb, (cudaStream_t)stream, 4);
}

int gbllt_dpotrs_adjoint_dev(int64_t n, int64_t nrhs, const double* d_l, int64_t ldl, const double* d_x, int64_t ldx,
                             const double* d_xbar, int64_t ldxb, double* d_bbar, int64_t ldbb, double* d_abar,
                             int64_t ldab, void* stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (n > 0 && !d_l) return -3;
  if (ldl < (n > 1 ? n : 1)) return -4;
  if (n > 0 && nrhs > 0 && d_abar && !d_x) return -5;
  if (ldx < (n > 1 ? n : 1)) return -6;
  if (n > 0 && nrhs > 0 && !d_xbar) return -7;
  if (ldxb < (n > 1 ? n : 1)) return -8;
  if (n > 0 && nrhs > 0 && !d_bbar) return -9;
  if (ldbb < (n > 1 ? n : 1)) return -10;
  if (d_abar && ldab < (n > 1 ? n : 1)) return -12;
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  int rc = ensure_device();
  if (rc) return rc;
  return potrs_adjoint_dev(n, nrhs, d_l, ldl, d_x, ldx, d_xbar, ldxb, d_bbar, ldbb, d_abar, ldab, (cudaStream_t)stream);
}

}  // extern "C"
