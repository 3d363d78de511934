/* gbllt.h -- C ABI of the GB300 (sm_103a) dense Cholesky (LLT) backend.
 *
 * This is the drop-in boundary for Eigen's dense Cholesky path.  Each entry point names the
 * reference interface it replaces (paths are inside the Eigen source tree):
 *   - the LAPACKE entry Eigen binds for its LAPACKE backend, LAPACKE_?potrf
 *     (Eigen/src/misc/lapacke.h:2821-2827), called by lapacke_llt<T>::potrf
 *     (Eigen/src/Cholesky/LLT_LAPACKE.h:47-61), which is the body of the explicit
 *     specialisation llt_inplace<T,Lower|Upper>::blocked (LLT_LAPACKE.h:64-92);
 *   - the Fortran-ABI routines Eigen itself exports, ?potrf_ / ?potrs_
 *     (lapack/cholesky.cpp:14-36 and :41-72);
 *   - the two triangular sweeps of LLT::_solve_impl_transposed (Eigen/src/Cholesky/LLT.h:490-498).
 *
 * Conventions (shared by every entry point)
 *   - Plain pointers and sizes only; no CUDA or C++ types cross this boundary.  A `stream`
 *     argument is a cudaStream_t passed as void* (NULL = the legacy default stream).
 *   - Host-pointer entry points are synchronous, like LAPACKE: they copy the inputs to the GPU,
 *     compute there, copy the results back and return.  `_dev` entry points take device
 *     pointers, are ordered on `stream` and return before the GPU work completes.
 *   - Storage: GBLLT_COL_MAJOR or GBLLT_ROW_MAJOR (the LAPACKE values), leading dimension
 *     `lda`.  Only the `uplo` triangle is read or written; the other strict triangle is left
 *     untouched (LLT.h keeps the strict upper part of m_matrix as it was).
 *   - Return value: GBLLT_SUCCESS, or -i when argument i (1-based) is illegal (the LAPACK
 *     convention, lapack/cholesky.cpp:17-24), or one of the GBLLT_ERR_* codes below.
 *   - `info` follows LAPACK: 0 on success, k > 0 when the leading minor of order k is not
 *     positive definite (the factorisation stopped at 0-based column k-1).  Eigen's
 *     llt_inplace::blocked returns k-1 for it and -1 for success (LLT_LAPACKE.h:60).
 *   - There is no CPU fallback: without a usable GPU every entry point returns
 *     GBLLT_ERR_NO_DEVICE.
 *   - Thread safety: entry points may be called from several host threads; each host thread
 *     uses its own library stream per device for the synchronous calls.
 */
#ifndef GBLLT_H
#define GBLLT_H

#include <stdint.h>

#if defined(__GNUC__)
#define GBLLT_API __attribute__((visibility("default")))
#else
#define GBLLT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBLLT_SUCCESS 0
#define GBLLT_ERR_CUDA (-1001)        /* a CUDA runtime call failed (see gbllt_last_error) */
#define GBLLT_ERR_ALLOC (-1002)       /* device or pinned memory could not be allocated */
#define GBLLT_ERR_TIMEOUT (-1003)     /* a bounded device-side wait ran out */
#define GBLLT_ERR_NO_DEVICE (-1004)   /* no CUDA device, or the device is not sm_103 */
#define GBLLT_ERR_INTERNAL (-1005)
#define GBLLT_ERR_NOT_CONVERGED (-1006) /* iterative refinement did not reach the tolerance */

#define GBLLT_ROW_MAJOR 101
#define GBLLT_COL_MAJOR 102

/* Library version (major*10000 + minor*100 + patch). */
GBLLT_API int gbllt_version(void);

/* Message of the last GBLLT_ERR_CUDA seen by the calling thread ("" if none). */
GBLLT_API const char* gbllt_last_error(void);

/* Workspaces come from a stream-ordered memory pool that the library creates for itself on first
 * use of a device (cudaMemPoolCreate; the device's default pool and its settings are left alone).
 * That pool keeps freed memory cached in the process instead of returning it at every
 * synchronisation (a large solve would otherwise map gigabytes again on each call).  This returns
 * the library's cached memory of the current device to the system. */
GBLLT_API int gbllt_release_cached_memory(void);

/* Factor A = L L^T ('L') or A = U^T U ('U') in place.
 * Replaces LAPACKE_dpotrf(matrix_layout, uplo, n, a, lda) as used by
 * Eigen/src/Cholesky/LLT_LAPACKE.h:59 and dpotrf_ (lapack/cholesky.cpp:14-36). */
GBLLT_API int gbllt_dpotrf(int layout, char uplo, int64_t n, double* a, int64_t lda, int64_t* info);
/* Single-precision twin: LAPACKE_spotrf / spotrf_ (LLT<MatrixXf>). */
GBLLT_API int gbllt_spotrf(int layout, char uplo, int64_t n, float* a, int64_t lda, int64_t* info);

/* Solve A X = B in place in B from a factor produced by ?potrf.
 * Replaces dpotrs_ (lapack/cholesky.cpp:41-72) and the two solveInPlace sweeps of
 * LLT::_solve_impl_transposed (Eigen/src/Cholesky/LLT.h:490-498). */
GBLLT_API int gbllt_dpotrs(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda,
                 double* b, int64_t ldb);
GBLLT_API int gbllt_spotrs(int layout, char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda,
                 float* b, int64_t ldb);

/* Factor and solve in one call (LAPACK ?posv semantics): A is overwritten by its factor and
 * B by X.  Equivalent to LLT::compute followed by LLT::solveInPlace (LLT.h:430-460, :514-522)
 * with a single upload of A. */
GBLLT_API int gbllt_dposv(int layout, char uplo, int64_t n, int64_t nrhs, double* a, int64_t lda, double* b,
                int64_t ldb, int64_t* info);
GBLLT_API int gbllt_sposv(int layout, char uplo, int64_t n, int64_t nrhs, float* a, int64_t lda, float* b,
                int64_t ldb, int64_t* info);

/* Device-pointer, stream-ordered variants (column-major).  d_info points to one int64_t in
 * device memory that receives the LAPACK info (or GBLLT_ERR_TIMEOUT if a bounded device-side wait
 * of the tensor-core trailing update ran out); it is written before the call's work on `stream`
 * completes.  FP64 factorisations of order >= 1024 run their trailing updates on the tensor cores
 * with FP64-exact error-free slicing (about 5 n KB of extra device memory; without it, or below that
 * order, on the FP64 pipe). */
GBLLT_API int gbllt_dpotrf_dev(char uplo, int64_t n, double* d_a, int64_t lda, int64_t* d_info, void* stream);
GBLLT_API int gbllt_spotrf_dev(char uplo, int64_t n, float* d_a, int64_t lda, int64_t* d_info, void* stream);
GBLLT_API int gbllt_dpotrs_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda, double* d_b,
                     int64_t ldb, void* stream);
GBLLT_API int gbllt_spotrs_dev(char uplo, int64_t n, int64_t nrhs, const float* d_a, int64_t lda, float* d_b,
                     int64_t ldb, void* stream);

/* ---- Mixed precision with FP64 iterative refinement ---------------------------------------
 * Solves A X = B to FP64 accuracy (normwise backward error <= tol) from a low-precision
 * factorisation: A is scaled by powers of two to a diagonal in [0.5, 2) and rounded to FP32, the
 * trailing updates of the blocked factorisation run on tensor cores in the chosen precision with
 * FP32 accumulation, the 64 x 64 diagonal blocks are factored in FP32, and residuals r = B - A X are
 * formed from the stored triangle of A in FP64 or FP64-exact on the tensor cores (the residual
 * method).  Replaces LLT<MatrixXd>::compute followed by solve
 * (Eigen/src/Cholesky/LLT.h:430-460, :483-498) for callers that need the solution, not the factor;
 * it is the counterpart of LAPACK's dsposv.  A and B are not modified. */
#define GBLLT_PREC_FP32 0   /* trailing update on FP32 CUDA cores (no tensor cores) */
#define GBLLT_PREC_TF32 1   /* one TF32 product per update */
#define GBLLT_PREC_TF32X3 2 /* three TF32 products (hi*hi + hi*lo + lo*hi): ~FP32 accuracy */
#define GBLLT_PREC_BF16 3   /* one BF16 product per update */
#define GBLLT_PREC_BF16X3 4 /* three BF16 products (two-way split) */
#define GBLLT_PREC_BF16X6 5 /* six BF16 products of a three-way split: ~FP32 accuracy at TF32X3 cost */

typedef struct {
  int precision;     /* GBLLT_PREC_*; default GBLLT_PREC_TF32X3 when opts == NULL */
  int max_steps;     /* refinement steps (solves with the low-precision factor); <= 0 -> 10, max 16 */
  double tol;        /* target normwise backward error; <= 0 -> 1e-14 */
  int fallback_fp64; /* when refinement fails, solve with the plain FP64 GPU factorisation */
  int panel;         /* outer panel width, a multiple of 64; <= 0 -> 256 below n = 16384, 384 from
                        there on (BF16X3: 512 from 16384, 640 from 32768) */
  int reserve_sms;   /* SMs left to the panel factorisation while the look-ahead update runs on the
                        others: 0 -> library default (32 for the first panels, growing to half the
                        SMs as the trailing matrix shrinks), < 0 -> none (the update may use every SM) */
  int residual;      /* how R = B - A X is formed: GBLLT_RESIDUAL_AUTO (0, default), _FP64 or
                        _TENSOR */
} gbllt_mixed_opts;

/* Residual methods.  TENSOR: A and X are split exactly into eight 7-bit BF16 slices (per-row and
 * per-column power-of-two scales) and the slice products run on the tensor cores with exact FP32
 * accumulation in 256-deep chunks and exact int64 combination; the result differs from the exact
 * B - A X by less than 2^-56 of the scaled magnitudes, i.e. at the FP64 rounding level.  It needs
 * n^2 * 16 bytes of device memory for A's slices (the no-allocation entry uses FP64).  FP64: the
 * product on the FP64 pipe, which is memory-bound for a few right-hand sides.  AUTO: TENSOR for
 * nrhs >= GBLLT_RESIDUAL_TENSOR_MIN_RHS, FP64 below. */
#define GBLLT_RESIDUAL_AUTO 0
#define GBLLT_RESIDUAL_FP64 1
#define GBLLT_RESIDUAL_TENSOR 2
#define GBLLT_RESIDUAL_TENSOR_MIN_RHS 4

/* R = B - A X for the symmetric A stored in the `uplo` triangle of d_a (column-major n x n), X, B
 * and R n x nrhs column-major, with one of the residual methods above; the residual that LAPACK's
 * dsposv forms with dsymm.  Stream-ordered; R may not overlap A, X or B. */
GBLLT_API int gbllt_dsyresid_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                 const double* d_x, int64_t ldx, const double* d_b, int64_t ldb, double* d_r,
                                 int64_t ldr, int method, void* stream);

typedef struct {
  int64_t info;          /* LAPACK info of the factorisation that produced X (0 = ok) */
  int steps;             /* refinement steps taken */
  int converged;         /* backward error of X <= tol */
  int used_fallback;     /* X came from the plain FP64 factorisation */
  double backward_error; /* ||B - A X||_F / (||A||_F ||X||_F) of the returned X */
  double factor_ms;      /* device time of scaling + low-precision factorisation */
  double refine_ms;      /* device time of the refinement loop */
  double history[16];    /* backward error after each refinement step */
} gbllt_mixed_report;

/* Device pointers, column-major; X is n x nrhs (ldx >= n).  Synchronises `stream` once per
 * refinement step to test convergence.  Returns GBLLT_ERR_NOT_CONVERGED (X = last iterate) when the
 * tolerance was not reached and no fallback was requested. */
GBLLT_API int gbllt_dposv_mixed_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                    const double* d_b, int64_t ldb, double* d_x, int64_t ldx,
                                    const gbllt_mixed_opts* opts, gbllt_mixed_report* report, void* stream);
/* Host pointers (LAPACKE-style layout), synchronous. */
GBLLT_API int gbllt_dposv_mixed(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda,
                                const double* b, int64_t ldb, double* x, int64_t ldx, const gbllt_mixed_opts* opts,
                                gbllt_mixed_report* report);

/* Same solve as gbllt_dposv_mixed_dev, for callers that cannot let the library allocate device
 * memory: their device memory is owned by their own caching allocator or a fixed budget, or they are
 * plug-ins handed only the buffers they work on.  No counterpart in the reference: Eigen's LLT
 * allocates on the host as it pleases.  This entry point calls no cudaMalloc / cudaMallocAsync /
 * cudaFree: its scratch is a fixed 64 MiB area inside the library image, held by every GPU that
 * loads the library until the process exits.  That is enough for n <= 2048 with up to 64
 * right-hand sides including the FP64 fallback, at the default panel width (opts->panel = 256; a
 * wider panel needs more); larger problems are rejected with GBLLT_ERR_SCRATCH_LIMIT
 * (gbllt_last_error() says how much scratch they need).  The first call on a device looks up the
 * area's device address; make that first call before any stream capture.  Like
 * gbllt_dposv_mixed_dev it synchronises `stream` once per refinement step.  All calls share the
 * area: calls whose GPU work overlaps race and must be serialised by the caller.  No device times
 * are reported (factor_ms = refine_ms = 0). */
#define GBLLT_ERR_SCRATCH_LIMIT (-1007)
GBLLT_API int gbllt_dposv_mixed_dev_noalloc(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                            const double* d_b, int64_t ldb, double* d_x, int64_t ldx,
                                            const gbllt_mixed_opts* opts, gbllt_mixed_report* report,
                                            void* stream);

/* ---- Batched factor + solve of many small systems of uneven sizes -------------------------
 * Replaces a loop of `LLT<MatrixXd> llt(A_s); x_s = llt.solve(b_s);` (Eigen/src/Cholesky/LLT.h:430-498)
 * over independent SPD systems, which Eigen runs one after another on the CPU.  A plan fixes the
 * sizes n_s (0 <= n_s <= 1024) and the packed layout: A_s is n_s x n_s column-major at element
 * offset aoff[s] = sum_{t<s} n_t^2 of one array, b_s (one right-hand side) at boff[s] =
 * sum_{t<s} n_t of another.  The solve overwrites the lower triangle of each A_s with L_s and b_s
 * with x_s, and writes the LAPACK info of each system.  All systems run in one persistent kernel
 * launch that pulls them from a largest-first work queue; the _dev entry points replay it as a
 * CUDA graph captured on first use for a given set of buffers. */
typedef struct gbllt_batch_plan gbllt_batch_plan;
/* elem_bytes: 8 (double) or 4 (float).  n is a host array of `count` sizes. */
GBLLT_API int gbllt_batch_plan_create(int64_t count, const int64_t* n, int elem_bytes, gbllt_batch_plan** plan);
GBLLT_API int gbllt_batch_plan_destroy(gbllt_batch_plan* plan);
/* Host copies of the offsets (arrays of `count`, may be NULL) and total element counts. */
GBLLT_API int gbllt_batch_plan_layout(const gbllt_batch_plan* plan, int64_t* aoff, int64_t* boff, int64_t* a_elems,
                                      int64_t* b_elems);
/* Number of batched kernel variants: algorithm (column at a time / panel-blocked) x panel width x
 * threads per CTA x the largest order staged in shared memory. */
#define GBLLT_BATCH_VARIANTS 16
/* Autotuner: times each kernel variant on synthetic SPD systems of the plan's sizes and keeps the
 * fastest; with cache_path, a previous choice for the same sizes is read from / a new one written
 * to that JSON file.  Returns the variant index (>= 0). */
GBLLT_API int gbllt_batch_plan_tune(gbllt_batch_plan* plan, const char* cache_path, void* stream);
/* Use kernel variant `variant` (0 .. GBLLT_BATCH_VARIANTS - 1) without tuning. */
GBLLT_API int gbllt_batch_plan_set_variant(gbllt_batch_plan* plan, int variant);
/* The variant in use: returns its index and its panel width, threads per CTA and the largest
 * order staged in shared memory. */
GBLLT_API int gbllt_batch_plan_variant(const gbllt_batch_plan* plan, int* panel, int* threads, int* smem_max_n);
/* Device pointers, stream-ordered (graph replay; no allocation, no host synchronisation). */
GBLLT_API int gbllt_dposv_batched_dev(gbllt_batch_plan* plan, double* d_a, double* d_b, int64_t* d_info,
                                      void* stream);
GBLLT_API int gbllt_sposv_batched_dev(gbllt_batch_plan* plan, float* d_a, float* d_b, int64_t* d_info,
                                      void* stream);
/* Host pointers, synchronous. */
GBLLT_API int gbllt_dposv_batched(gbllt_batch_plan* plan, double* a, double* b, int64_t* info);
GBLLT_API int gbllt_sposv_batched(gbllt_batch_plan* plan, float* a, float* b, int64_t* info);

/* Batched mixed-precision solve: every FP64 system of a plan (elem_bytes 8) solved to FP64
 * accuracy with an FP32 factorisation and FP64 iterative refinement -- the batched counterpart of
 * gbllt_dposv_mixed_dev, with no counterpart in the reference (Eigen solves each system in FP64).
 * A and b are read only (A's lower triangle); x receives the solutions, laid out like b.
 * Per system: A is rounded to FP32 and factored (the FP32 batched kernel, whose variant is tuned on
 * the first call), then x is refined with r = b - A x in FP64 until ||r||_F <= tol ||A||_F ||x||_F
 * or max_steps corrections were made; one launch per step for the whole batch.  Uses
 * opts->max_steps, ->tol and ->fallback_fp64 (precision, panel, reserve_sms and residual are not
 * used).  info[s]: 0 solved; k > 0: the FP64 factorisation (fallback) or, without fallback, the FP32
 * one failed at column k; GBLLT_BATCH_NOT_CONVERGED: no fallback and tol not reached (x holds the
 * last iterate).  With fallback_fp64, the systems that the FP32 factorisation or the refinement
 * failed are solved again by the FP64 batched kernel.  Synchronises `stream` once per step. */
#define GBLLT_BATCH_NOT_CONVERGED (-1)
typedef struct {
  int steps;                 /* refinement steps made (corrections of the slowest system) */
  int64_t converged;         /* systems that reached tol in mixed precision */
  int64_t fallback;          /* systems solved again in FP64 */
  double max_backward_error; /* the largest ||r||_F / (||A||_F ||x||_F) at the last check */
} gbllt_batch_mixed_report;
GBLLT_API int gbllt_batch_dposv_mixed_dev(gbllt_batch_plan* plan, const double* d_a, const double* d_b, double* d_x,
                                          int64_t* d_info, const gbllt_mixed_opts* opts,
                                          gbllt_batch_mixed_report* report, void* stream);

/* ---- Reverse mode (adjoints) of the factorisation and the solve, FP64, device pointers -------
 * Eigen has no derivative of LLT; these give the gradients of any scalar function of the factor
 * or of the solution, for A symmetric positive definite with A = L L^T (lower, column-major).
 * Gradients with respect to A are symmetric matrices G with df = sum_ij G_ij dA_ij for symmetric
 * dA; their lower triangle is stored. */
/* d_lbar holds Lbar = df/dL (lower triangle) on entry and Abar = df/dA on return.  Blocked, in
 * place, from L only (no stored intermediates): about 2 n^3 / 3 flops, twice the factorisation's;
 * the products with each 64-wide panel run FP64-exact on the tensor cores, the rest on the FP64
 * pipe.  A bounded wait that runs out leaves NaN in the gradient. */
GBLLT_API int gbllt_dpotrf_adjoint_dev(int64_t n, const double* d_l, int64_t ldl, double* d_lbar, int64_t ldlb,
                                       void* stream);
/* The same reverse sweep in mixed precision: the products with each panel carry 28 bits (four of
 * the eight 7-bit slices of each operand, 10 of the 36 slice products), everything else stays FP64.
 * The gradient is accurate to about FP32 level (relative error ~1e-7 or better on well-conditioned
 * problems). */
GBLLT_API int gbllt_dpotrf_adjoint_mixed_dev(int64_t n, const double* d_l, int64_t ldl, double* d_lbar,
                                             int64_t ldlb, void* stream);
/* For X = A^{-1} B (n x nrhs) with its adjoint Xbar: writes Bbar = A^{-1} Xbar and, when d_abar is
 * not NULL, accumulates Abar -= sym(Bbar X^T) into its lower triangle. */
GBLLT_API int gbllt_dpotrs_adjoint_dev(int64_t n, int64_t nrhs, const double* d_l, int64_t ldl, const double* d_x,
                                       int64_t ldx, const double* d_xbar, int64_t ldxb, double* d_bbar, int64_t ldbb,
                                       double* d_abar, int64_t ldab, void* stream);

/* ---- Rank-1 update / downdate (LLT::rankUpdate, Eigen/src/Cholesky/LLT.h:469-478) ----------
 * Given the factor of A in the `uplo` triangle, overwrite it with the factor of A + sigma v v^T:
 * llt_rank_update_lower (LLT.h:238-307) -- Givens rotations for sigma > 0, the beta recurrence for
 * sigma <= 0.  info = 0, or k + 1 when a downdate leaves A + sigma v v^T not positive definite at
 * column k (the factor's contents are then unspecified; LLT reports NumericalIssue). */
GBLLT_API int gbllt_drank_update(int layout, char uplo, int64_t n, double* l, int64_t ldl, const double* v,
                                 double sigma, int64_t* info);
GBLLT_API int gbllt_srank_update(int layout, char uplo, int64_t n, float* l, int64_t ldl, const float* v,
                                 float sigma, int64_t* info);
/* Device pointers (column-major), stream-ordered; *d_info is device memory and may also receive
 * GBLLT_ERR_TIMEOUT if a bounded device-side wait ran out. */
GBLLT_API int gbllt_drank_update_dev(char uplo, int64_t n, double* d_l, int64_t ldl, const double* d_v,
                                     double sigma, int64_t* d_info, void* stream);
GBLLT_API int gbllt_srank_update_dev(char uplo, int64_t n, float* d_l, int64_t ldl, const float* d_v, float sigma,
                                     int64_t* d_info, void* stream);

/* ---- Condition estimate (LLT::rcond, Eigen/src/Cholesky/LLT.h:166-171) ---------------------- */

/* 1-norm (max absolute column sum) of the symmetric n x n matrix stored in the `uplo` triangle of
 * the column-major d_a: the m_l1_norm loop of LLT::compute (LLT.h:443-453).  The result is written
 * to *d_norm (device), stream-ordered. */
GBLLT_API int gbllt_dlansy_l1_dev(char uplo, int64_t n, const double* d_a, int64_t lda, double* d_norm,
                                  void* stream);
GBLLT_API int gbllt_slansy_l1_dev(char uplo, int64_t n, const float* d_a, int64_t lda, float* d_norm, void* stream);
/* Reciprocal 1-norm condition estimate from a factor produced by ?potrf and anorm = ||A||_1:
 * rcond_estimate_helper + rcond_invmatrix_L1_norm_estimate (Eigen/src/Core/ConditionEstimator.h:
 * 56-171) with every solve on the device; the same role as LAPACK dpocon.  Returns after the
 * estimate is known (*rcond is host memory): +inf for n = 0, 0 for anorm = 0, 1 for n = 1. */
GBLLT_API int gbllt_dpocon_dev(char uplo, int64_t n, const double* d_l, int64_t ldl, double anorm, double* rcond,
                               void* stream);
GBLLT_API int gbllt_spocon_dev(char uplo, int64_t n, const float* d_l, int64_t ldl, float anorm, float* rcond,
                               void* stream);
/* Host-pointer form (the factor is copied to the device once for all the solves). */
GBLLT_API int gbllt_dpocon(int layout, char uplo, int64_t n, const double* l, int64_t ldl, double anorm,
                           double* rcond);
GBLLT_API int gbllt_spocon(int layout, char uplo, int64_t n, const float* l, int64_t ldl, float anorm, float* rcond);

/* ---- Diagnostics (no counterpart in the reference; Eigen has no built-in timers) ----------- */

/* Per-kernel-class totals: launches, device time (CUDA events on the launch stream) and the
 * algorithmic work of those launches (flops and bytes implied by the launch shapes). */
typedef struct {
  char name[40];
  int64_t launches;
  double ms;
  double flops;
  double bytes;
} gbllt_kernel_stat;

/* ---- Pivoted LDL^T (LDLT<MatrixXd|MatrixXf, UpLo>, Eigen/src/Cholesky/LDLT.h) -----------------
 * Factorisation, replacing LDLT::compute (LDLT.h:497-530 -> ldlt_inplace<Lower>::unblocked,
 * LDLT.h:297-403; Upper runs on the transpose, LDLT.h:460-466): P A P^T = L D L^T with Eigen's
 * symmetric pivoting (largest remaining |diagonal entry|, first on ties).  On return the `uplo`
 * triangle holds L (unit diagonal, not stored) and D on the diagonal -- LDLT::matrixLDLT() -- and
 * the other triangle is untouched; transp[k] (n entries, host memory) is the row swapped with row k
 * at step k -- LDLT::transpositionsP().indices(); *sign is one of the GBLLT_SIGN_* values below
 * (Eigen's internal::SignMatrix, LDLT.h:31); *info = 0 (Success) or 1 (NumericalIssue: a zero
 * pivot with a nonzero column below it, or a nonzero pivot after a zero one, LDLT.h:383-387).
 * The pivot order is computed on the host from the diagonal, so the _dev entry synchronises its
 * stream (once to read the diagonal, once for sign and info); transp, sign and info are host
 * memory in both entries. */
#define GBLLT_SIGN_POSITIVE_SEMIDEF 0
#define GBLLT_SIGN_NEGATIVE_SEMIDEF 1
#define GBLLT_SIGN_ZERO 2
#define GBLLT_SIGN_INDEFINITE 3
GBLLT_API int gbllt_dldlt(int layout, char uplo, int64_t n, double* a, int64_t lda, int32_t* transp, int32_t* sign,
                          int64_t* info);
GBLLT_API int gbllt_sldlt(int layout, char uplo, int64_t n, float* a, int64_t lda, int32_t* transp, int32_t* sign,
                          int64_t* info);
GBLLT_API int gbllt_dldlt_dev(char uplo, int64_t n, double* d_a, int64_t lda, int32_t* transp, int32_t* sign,
                              int64_t* info, void* stream);
GBLLT_API int gbllt_sldlt_dev(char uplo, int64_t n, float* d_a, int64_t lda, int32_t* transp, int32_t* sign,
                              int64_t* info, void* stream);
/* The transpositions that LDLT::compute chooses for a matrix whose diagonal is diag[0], diag[incd],
 * ... (the pivot order depends on nothing else): host computation, no device needed.  The
 * factorisation entries above compute the same order. */
GBLLT_API int gbllt_dldlt_pivots(int64_t n, const double* diag, int64_t incd, int32_t* transp);
GBLLT_API int gbllt_sldlt_pivots(int64_t n, const float* diag, int64_t incd, int32_t* transp);
/* X = A^{-1} B in place in B from that factor and its transpositions (host memory), replacing
 * LDLT::_solve_impl_transposed (LDLT.h:573-613): P, the unit-L solve, D's pseudo-inverse (entries
 * with |d| <= the smallest normal number give 0), the L^T solve, P^T.  The _dev entry is
 * stream-ordered. */
GBLLT_API int gbllt_dldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda,
                                const int32_t* transp, double* b, int64_t ldb);
GBLLT_API int gbllt_sldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda,
                                const int32_t* transp, float* b, int64_t ldb);
GBLLT_API int gbllt_dldlt_solve_dev(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                    const int32_t* transp, double* d_b, int64_t ldb, void* stream);
GBLLT_API int gbllt_sldlt_solve_dev(char uplo, int64_t n, int64_t nrhs, const float* d_a, int64_t lda,
                                    const int32_t* transp, float* d_b, int64_t ldb, void* stream);

/* ---- BLAS level 3 of the Cholesky path (Eigen's Fortran BLAS, blas/level3_impl.h) -------------
 * SYRK replaces dsyrk_ / ssyrk_ (blas/level3_impl.h:355-417): C = alpha op(A) op(A)^T + beta C on
 * the `uplo` triangle of the n x n C, op(A) = A (n x k) for trans 'N', A^T (A k x n) for 'T'/'C'.
 * beta is applied first (0 clears the triangle without reading it), then alpha times the product;
 * the other triangle of C is untouched.  Argument errors return -i with i the argument's position
 * (the _dev forms have no layout argument). */
GBLLT_API int gbllt_dsyrk(int layout, char uplo, char trans, int64_t n, int64_t k, double alpha, const double* a,
                          int64_t lda, double beta, double* c, int64_t ldc);
GBLLT_API int gbllt_ssyrk(int layout, char uplo, char trans, int64_t n, int64_t k, float alpha, const float* a,
                          int64_t lda, float beta, float* c, int64_t ldc);
GBLLT_API int gbllt_dsyrk_dev(char uplo, char trans, int64_t n, int64_t k, double alpha, const double* d_a,
                              int64_t lda, double beta, double* d_c, int64_t ldc, void* stream);
GBLLT_API int gbllt_ssyrk_dev(char uplo, char trans, int64_t n, int64_t k, float alpha, const float* d_a,
                              int64_t lda, float beta, float* d_c, int64_t ldc, void* stream);
/* TRSM replaces dtrsm_ / strsm_ (blas/level3_impl.h:78-160): B (m x n) = alpha op(A)^{-1} B for
 * side 'L' (A m x m) or alpha B op(A)^{-1} for side 'R' (A n x n); A upper or lower triangular
 * (`uplo`), op 'N' or 'T'/'C', diag 'U' (unit, not read) or 'N'.  As in the reference the solve
 * comes first and alpha scales its result. */
GBLLT_API int gbllt_dtrsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n,
                          double alpha, const double* a, int64_t lda, double* b, int64_t ldb);
GBLLT_API int gbllt_strsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n,
                          float alpha, const float* a, int64_t lda, float* b, int64_t ldb);
GBLLT_API int gbllt_dtrsm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
                              const double* d_a, int64_t lda, double* d_b, int64_t ldb, void* stream);
GBLLT_API int gbllt_strsm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n, float alpha,
                              const float* d_a, int64_t lda, float* d_b, int64_t ldb, void* stream);

/* Turn per-launch event timing on (1) or off (0); either call discards earlier records. */
GBLLT_API int gbllt_profile_enable(int on);
/* Wait for the recorded launches and return up to max_entries classes; *n_entries = classes seen. */
GBLLT_API int gbllt_profile_read(gbllt_kernel_stat* out, int max_entries, int* n_entries);

/* One recorded launch: its kernel class, the stream it ran on, and its start and end on the device,
 * in ms after the first launch recorded since gbllt_profile_enable (events on the launch's stream,
 * so concurrent launches on different streams overlap in time). */
typedef struct {
  char name[40];
  uint64_t stream;
  double start_ms;
  double end_ms;
  double flops;
  double bytes;
} gbllt_launch_record;
/* Wait for the recorded launches and return the first max_entries of them in launch order;
 * *n_entries = launches recorded.  No counterpart in the reference (a tracing aid). */
GBLLT_API int gbllt_profile_trace(gbllt_launch_record* out, int max_entries, int* n_entries);

/* Failure-detection self-test of the device-side bounded waits.  No counterpart in the reference
 * (Eigen's LLT runs on one CPU thread and never waits on another).  Every wait of the library's
 * kernels (the solve's look-back flags, the tensor-core pipelines' mbarriers, the rank update's
 * block flags) gives up after a time limit, sets an error word and returns, so that a lost signal
 * ends in GBLLT_ERR_TIMEOUT instead of a hung GPU; host-pointer entries then return that code, and
 * a triangular sweep that gave up writes NaN into the rows it could not solve.  This runs one
 * FP64 and one FP32 sweep of order 256 in which block 0 is never solved, with the wait limited to
 * wait_us microseconds (1000 .. 2000000), on the calling thread's library stream.  *observed
 * receives the code the waits reported (GBLLT_ERR_TIMEOUT); the return value is GBLLT_SUCCESS when
 * every wait gave up as designed, both error words were set, the unsolved rows are NaN and the
 * solved ones untouched, and GBLLT_ERR_INTERNAL otherwise.  The device stays usable. */
GBLLT_API int gbllt_selftest_wait_timeout(int64_t wait_us, int* observed);

/* Self-test of the FP64-to-FP32 rounding that forms the mixed solve's FP32 working copy (integer
 * arithmetic on the bits, round to nearest even; the FP32 conversion of the GPU otherwise runs on
 * its narrow FP64 pipe): d_out[i] receives that rounding of d_in[i] and d_ref[i] the hardware
 * conversion, n device values each, stream-ordered on `stream`.  The two agree bit for bit. */
GBLLT_API int gbllt_selftest_f64_to_f32(const double* d_in, float* d_out, float* d_ref, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBLLT_H */
