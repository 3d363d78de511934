// Host-side drivers shared by the C ABI translation units (not part of the public ABI).
#pragma once
#include <string>

#include "common.cuh"

namespace gbllt {

// A 2-D copy (cudaMemcpy2DAsync's arguments) issued as one linear copy when both pitches equal the
// row width, so a contiguous host matrix moves as one transfer.
inline cudaError_t copy2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                                size_t height, cudaMemcpyKind kind, cudaStream_t s) {
  if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * height, kind, s);
  return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, s);
}

// Copies the `upper ? upper : lower` triangle of a column-major n x n matrix (leading dimensions
// dld / sld in elements of es bytes) in column panels of 256: each panel is one 2-D copy of its
// diagonal block and the rows below it (above it for upper), so about half of the matrix moves.  The
// other triangle of dst is left as it was.
inline cudaError_t copy_triangle_async(bool upper, int64_t n, void* dst, size_t dld, const void* src, size_t sld,
                                       size_t es, cudaMemcpyKind kind, cudaStream_t s) {
  for (int64_t j0 = 0; j0 < n; j0 += 256) {
    const int64_t jb = n - j0 < 256 ? n - j0 : 256;
    const int64_t r0 = upper ? 0 : j0, rows = upper ? j0 + jb : n - j0;
    const cudaError_t e =
        cudaMemcpy2DAsync((char*)dst + ((size_t)j0 * dld + r0) * es, dld * es, (const char*)src + ((size_t)j0 * sld + r0) * es,
                          sld * es, (size_t)rows * es, (size_t)jb, kind, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Plain-path panel width: the diagonal block factored by one CTA and the depth of each
// trailing update.
constexpr int kNB = 64;

// Stream-ordered factorisation of the lower triangle of the column-major n x n matrix at
// d_a (device).  `st` is a device status word, initialised by the caller to fail_col = -1.
// For T = double and n of at least kTensorSyrkMinN, the trailing updates run on the tensor cores
// (OzakiSyrk) when may_allocate allows its workspace; otherwise, and for float, on the FP64/FP32 pipe.
constexpr int64_t kTensorSyrkMinN = 1024;
template <typename T>
int potrf_lower_dev(int64_t n, T* d_a, int64_t lda, DevStatus* st, cudaStream_t s, bool may_allocate = true);

// Kernel launchers of the blocked factorisation, shared with the mixed-precision path.
// Diagonal 64 x 64 block at (k0, k0): storage T, arithmetic TC.
template <typename T, typename TC>
void launch_potrf_diag(T* a, int64_t lda, int64_t k0, int bs, DevStatus* st, cudaStream_t s);
// FP32 diagonal block in FP32 arithmetic, 512 threads, one barrier per column (the mixed-precision
// factorisation).
// pk > 0: the block first receives A11 -= P P^T with P the pk columns from column pk0 in the block's
// rows (one panel step whose trailing update left the block out).
// linv: also write L11^{-1} there (64 x 64 FP32, row-major, identity beyond bs) for
// launch_trsm_panel_tc.
void launch_potrf_diag_f32s(float* a, int64_t lda, int64_t k0, int bs, DevStatus* st, cudaStream_t s,
                            int64_t pk0 = 0, int pk = 0, float* linv = nullptr);
// Rows below the block: A(k0+bs.., k0..k0+bs) <- A(...) L11^{-T}, rs rows.
template <typename T>
void launch_trsm_panel(T* a, int64_t lda, int64_t k0, int bs, int64_t rs, DevStatus* st, cudaStream_t s);
// The same FP32 solve as the product A21 L11^{-T} with the inverse from launch_potrf_diag_f32s, on
// the tensor cores (mma.sync, three-part BF16 split: FP32-accurate), also writing the solved rows as
// np split parts (BF16, or TF32 when tf32 is set; np = 0: none), K-major with 64 columns per row: the
// operand of the mixed-precision in-panel update.
void launch_trsm_panel_tc(float* a, int64_t lda, int64_t k0, int bs, int64_t rs, DevStatus* st, const float* linv,
                          int tf32, int np, void* const* parts, cudaStream_t s);
// Lower update of the first ncols columns of the rs x rs trailing matrix by the bs-wide panel:
// A22 -= A21 A21^T, or A22 -= A21 B^T with B the rs x bs array at bsrc (leading dimension ldb).
template <typename T>
void launch_syrk_lower(T* a, int64_t lda, int64_t k0, int bs, int64_t rs, int64_t ncols, DevStatus* st,
                       cudaStream_t s, const T* bsrc = nullptr, int64_t ldb = 0);

// Swap the strict lower and strict upper triangles of the n x n matrix at d_a in place
// (A <- A^T).  Used to run the lower algorithm on an upper-stored factor, the same trick as
// llt_inplace<Scalar,Upper> (Eigen/src/Cholesky/LLT.h:377-399).
template <typename T>
int transpose_inplace_dev(int64_t n, T* d_a, int64_t lda, cudaStream_t s);

// Out-of-place transpose: dst (cols x rows, ldd) = src^T, src rows x cols column-major.
template <typename T>
int transpose_dev(int64_t rows, int64_t cols, const T* src, int64_t lds, T* dst, int64_t ldd,
                  cudaStream_t s);

// Writes the LAPACK info (0, or fail_col + 1) from the status word into *d_info (device).
int finalize_info_dev(const DevStatus* st, int64_t* d_info, cudaStream_t s);

// Stream-ordered solve L L^T X = B (upper == false; L lower column-major at d_a) or
// U^T U X = B (upper == true; U upper column-major), B column-major n x nrhs, in place.
// host_err (optional): receives the solve's error word (copied in stream order; valid once the
// caller has synchronised s).
template <typename T>
int potrs_dev(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb,
              cudaStream_t s, int* host_err = nullptr);

// Brackets one kernel launch with profiling events when gbllt_profile_enable(1) is in effect.
struct ProfScope {
  int slot;
  cudaStream_t stream;
  ProfScope(const char* kind, cudaStream_t s, double flops, double bytes);
  ~ProfScope();
  ProfScope(const ProfScope&) = delete;
  ProfScope& operator=(const ProfScope&) = delete;
};

template <typename T>
constexpr const char* tname() {
  return sizeof(T) == 8 ? "f64" : "f32";
}

// The device error word of a solve on the workspace ws (elem = the solve's element size): 0, or 1
// when a bounded wait of one of its sweeps ran out (the rows it could not solve are then NaN).
// Cleared by each call; a caller that synchronises reads it to report GBLLT_ERR_TIMEOUT.
int* potrs_ws_error_word(int64_t n, size_t elem, void* ws);
// Failure-detection self-test of the sweeps' bounded waits (potrs_lookback.cu); *observed = the
// code the waits reported.
int sweep_wait_selftest(unsigned long long wait_ns, cudaStream_t s, int* observed);

// The same solve on a caller-supplied workspace of potrs_ws_bytes(n, sizeof(T)) bytes (allocates
// nothing).
size_t potrs_ws_bytes(int64_t n, size_t elem);
template <typename T>
int potrs_ws(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb, void* ws,
             cudaStream_t s);

// Mixed-precision solve with FP64 refinement (device pointers, column-major).
// Workspace layout of one solve: the FP32 working matrix (ldf x n), scaling, residuals, partial
// sums, split panel operands and the status word, in `bytes`; `fallback_bytes` more hold the FP64
// copy used by the FP64 fallback.
struct MixedLayout {
  int64_t ldf, ldk;
  int nb, zc, nparts, jpc, nsq;
  size_t es_k, bytes, fallback_bytes;
};
int resolve_mixed_opts(const gbllt_mixed_opts* in, gbllt_mixed_opts* out, int64_t n);  // defaults; -1 if invalid
// lookahead: room for the second set of panel operands that the two-stream schedule uses.
MixedLayout mixed_layout(int64_t n, int64_t nrhs, const gbllt_mixed_opts& o, bool lookahead);
// The solve on a caller-supplied workspace of ws_bytes (>= mixed_layout(.., may_allocate).bytes).
// With may_allocate false it creates no streams or events and allocates nothing: the factorisation
// runs without lookahead, the fallback runs only if the workspace also holds fallback_bytes, and the
// report's device times are 0.
int posv_mixed_core(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, const double* b, int64_t ldb,
                    double* x, int64_t ldx, const gbllt_mixed_opts& o, gbllt_mixed_report* rep, void* ws,
                    size_t ws_bytes, bool may_allocate, cudaStream_t s);
int posv_mixed_dev(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, const double* b, int64_t ldb,
                   double* x, int64_t ldx, const gbllt_mixed_opts* opts, gbllt_mixed_report* rep, cudaStream_t s);

// The LDL^T solve's two sweeps in place on b (already permuted): unit L from the factor at a, D^+
// from its diagonal; workspace of potrs_ws_bytes(n, sizeof(T)) bytes.
template <typename T>
int ldlt_sweeps_ws(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b, int64_t ldb, void* ws,
                   cudaStream_t s);

// One triangular sweep in place on b (n x nrhs): L X = B (forward) or L^T X = B (bwd), L lower
// column-major (upper == false) or stored as its transpose in an upper triangle (upper == true);
// unit: L's diagonal is 1 and not read.  Workspace of potrs_ws_bytes(n, sizeof(T)) bytes.  ext_err
// (optional): the device word the sweep's bounded waits report to, instead of the workspace's own
// (which each call clears); a caller chaining several sweeps keeps one word for all of them.
// pre_inv (optional, not with unit): the 64 x 64 inverses of L's diagonal blocks, as trinv_all
// leaves them; the sweep then forms none and runs chains of 4 right-hand sides (a panel of a
// blocked solve).
template <typename T>
int trsm_sweep_ws(bool upper, bool bwd, bool unit, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, T* d_b,
                  int64_t ldb, void* ws, cudaStream_t s, int* ext_err = nullptr, const T* pre_inv = nullptr);
// The inverses of the 64 x 64 diagonal blocks of the n x n triangle (block b at inv + b * 4096,
// column-major), one CTA per block.
template <typename T>
int trinv_all(bool upper, int64_t n, const T* d_a, int64_t lda, T* inv, cudaStream_t s);

// Pivoted LDL^T (LDLT::compute) of the symmetric matrix in the `upper ? upper : lower` triangle of
// the column-major device matrix d_a; transpositions, sign and info (0 Success, 1 NumericalIssue)
// are written to host memory.  Synchronises s.
template <typename T>
int ldlt_factor_dev(bool upper, int64_t n, T* d_a, int64_t lda, int32_t* transp, int32_t* sign, int64_t* info,
                    cudaStream_t s);
// x = A^{-1} b from the factor and host transpositions, b column-major n x nrhs on the device.
template <typename T>
int ldlt_solve_dev(bool upper, int64_t n, int64_t nrhs, const T* d_a, int64_t lda, const int32_t* transp, T* d_b,
                   int64_t ldb, cudaStream_t s);

// FP64 residual R = B - A X of a symmetric A on the BF16 tensor cores (error-free slicing of A and X,
// exact FP32 accumulation in 256-deep chunks, int64 combination; ozaki.cu).  setup() slices A once
// (n^2 * 16 bytes of device memory, stream-ordered); residual() slices X and forms R.  A non-finite
// input gives a NaN residual.  The object owns its device memory.
struct OzakiResidual {
  int64_t n = 0, nrhs = 0, lds = 0;
  void* buf = nullptr;
  cudaStream_t stream = nullptr;
  void* aslices = nullptr;
  void* xslices = nullptr;
  unsigned long long* rmax = nullptr;
  int* rexp = nullptr;
  int* xexp = nullptr;
  int* flags = nullptr;
  long long* part = nullptr;  // the K-split product's int64 sums
  OzakiResidual() = default;
  OzakiResidual(const OzakiResidual&) = delete;
  OzakiResidual& operator=(const OzakiResidual&) = delete;
  ~OzakiResidual();
  static size_t bytes(int64_t n, int64_t nrhs);
  // The device memory alone, stream-ordered on s (setup() reserves it itself when this was not called).
  int reserve(int64_t n, int64_t nrhs, cudaStream_t s);
  int setup(bool upper, int64_t n, int64_t nrhs, const double* a, int64_t lda, cudaStream_t s);
  int residual(const double* x, int64_t ldx, const double* b, int64_t ldb, double* r, int64_t ldr, cudaStream_t s);
  // copies the device timeout word (1 if a bounded wait of the product kernel ran out) to host memory
  int timeout_flag_into(int* host_flag, cudaStream_t s) const;
};

// The trailing updates of the FP64 factorisation on the BF16 tensor cores, FP64-exact (ozaki.cu):
// init() allocates panel slices for panels of up to nmax rows (about 5 nmax KB, stream-ordered) and
// encodes their tensor maps; update() slices the rs x pw panel below the diagonal block at (k0, k0)
// (pw <= 64, or up to kWide columns at once: one exact 256-deep chunk) and applies C -= L21 L21^T to
// the lower part of the rs x ncols block at (k0 + pw, k0 + pw).  A bounded wait that runs out sets
// st->timeout.
constexpr int kWide = 256;
struct OzakiSyrk {
  int64_t nmax = 0;
  int sms = 0;
  void* buf = nullptr;
  void* slices = nullptr;    // 64-wide sub-panel slices
  int* pexp = nullptr;
  void* slices_w = nullptr;  // kWide-wide panel slices
  int* pexp_w = nullptr;
  void* slices_b = nullptr;  // 64-wide slices of a second operand (two_sided)
  int* pexp_b = nullptr;
  void* maps = nullptr;
  cudaStream_t stream = nullptr;
  OzakiSyrk() = default;
  OzakiSyrk(const OzakiSyrk&) = delete;
  OzakiSyrk& operator=(const OzakiSyrk&) = delete;
  ~OzakiSyrk();
  int init(int64_t nmax, cudaStream_t s, bool two_sided = false);
  int update(double* a, int64_t lda, int64_t k0, int pw, int64_t rs, int64_t ncols, DevStatus* st, cudaStream_t s);
  // C -= P Q^T (lower) with Q given separately (the LDL^T update, Q = L21 D); needs two_sided, pw <= 64.
  int update_pq(double* a, int64_t lda, int64_t k0, int pw, int64_t rs, const double* q, int64_t ldq, DevStatus* st,
                cudaStream_t s);
  void release_maps();
};

// C (m x n, FP64, column-major ldc) -= 2^scale P Q^T on the BF16 tensor cores, exact to FP64 rounding of
// the result (ozaki.cu: the residual's error-free slicing in a rectangle mode).  P is m x k and Q is
// n x k; element (i, kk) of each lies at base[i * rstride + kk * kstride] (a column-major array has
// rstride 1 and kstride = its leading dimension; the transpose of one has rstride = the leading
// dimension and kstride 1).  attach() places the slices of both operands in a caller-supplied
// workspace of bytes(mmax, nmax, kmax); run() forms them and the product, stream-ordered.  A bounded
// wait that runs out sets *err.  nsl < 8 uses only the first nsl 7-bit slices of each operand and the
// slice pairs of weight below nsl: the product then carries about 7 nsl bits (nsl = 4: FP32 level)
// for (nsl (nsl + 1) / 2) / 36 of the tensor-core work.
struct OzakiGemm {
  int64_t mmax = 0, nmax = 0, kmax = 0;
  int sms = 0;
  void* pslices = nullptr;
  void* qslices = nullptr;
  int* pexp = nullptr;
  int* qexp = nullptr;
  unsigned long long* rmax = nullptr;  // row maxima of a column-major operand being sliced
  static size_t bytes(int64_t mmax, int64_t nmax, int64_t kmax);
  int attach(void* ws, int64_t mmax, int64_t nmax, int64_t kmax);
  int run(double* c, int64_t ldc, int64_t m, int64_t n, int64_t k, const double* p, int64_t p_rs, int64_t p_ks,
          const double* q, int64_t q_rs, int64_t q_ks, int scale, int* err, cudaStream_t s, int nsl = 8);
};

// Rank-1 update / downdate of the factor at l (device), L L^T + sigma v v^T; *d_info (device)
// receives 0, the failing column + 1 of a downdate, or GBLLT_ERR_TIMEOUT.
template <typename T>
int rank_update_dev(bool upper, int64_t n, T* l, int64_t ldl, const T* v, T sigma, int64_t* d_info, cudaStream_t s);

// Validates (uplo, n, lda) the way dpotrf_ does (lapack/cholesky.cpp:17-19); returns 0 or -argpos.
int check_uplo(char uplo);

// Ensures the current device can run the sm_103a kernels; GBLLT_SUCCESS or GBLLT_ERR_NO_DEVICE.
int ensure_device();

}  // namespace gbllt
