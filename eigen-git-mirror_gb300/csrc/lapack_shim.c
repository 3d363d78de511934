/* Fortran-ABI LAPACK Cholesky and BLAS level-3 entry points over the gbllt C ABI
 * (libgbllt_lapack.so).
 *
 * Eigen's own LAPACK build exports dpotrf_/spotrf_ and dpotrs_/spotrs_ from lapack/cholesky.cpp
 * (:14-36 and :41-72): arguments by reference, column-major storage, argument errors reported
 * through xerbla_ with a negative info, and a failed factorisation reported as info = k + 1 for
 * the first non-positive pivot at column k.  These functions keep that interface, so a program
 * linked against a LAPACK library can be relinked against this one, and run the factorisation and
 * solve on the GPU through gbllt_?potrf / gbllt_?potrs (host pointers, synchronous).
 *
 * The BLAS routines dsyrk_/ssyrk_ and dtrsm_/strsm_ of Eigen's BLAS build (blas/level3_impl.h:355-417
 * and :78-160) are here too, with the reference's argument checks in its order and its xerbla_
 * names ("DSYRK ", "DTRSM "), over gbllt_?syrk / gbllt_?trsm.
 *
 * One difference is documented rather than hidden: a GPU-side failure (no usable device, an
 * allocation or a CUDA error) has no LAPACK code.  It is reported as *info = the gbllt error code
 * (GBLLT_ERR_*, all <= -1001, a range no argument error can take); gbllt_last_error() gives the
 * message.  There is no CPU fallback.
 */
#include <stdint.h>
#include <stdio.h>

#include "gbllt.h"
#include "gbllt_lapack.h"

#define SHIM_API __attribute__((visibility("default")))

/* Default error handler with the reference's message format (blas/xerbla.cpp:15-19).  It is weak,
 * so an application's or a LAPACK library's own xerbla_ takes precedence. */
SHIM_API __attribute__((weak)) int xerbla_(const char* msg, int* info, int len) {
  (void)len;
  printf("Eigen BLAS ERROR #%i: %s\n", *info, msg);
  fflush(stdout);  /* visible at once, also when stdout is a pipe */
  return 0;
}

/* 'U'/'u' -> 'U', 'L'/'l' -> 'L', anything else -> 0 (blas/common.h:56-58). */
static char uplo_of(const char* uplo) {
  if (!uplo) return 0;
  if (*uplo == 'U' || *uplo == 'u') return 'U';
  if (*uplo == 'L' || *uplo == 'l') return 'L';
  return 0;
}

static int max1(int n) { return n > 1 ? n : 1; }

static int arg_error(const char* name, int info) {
  int e = -info;
  return xerbla_(name, &e, 6);
}

/* Argument checks of lapack/cholesky.cpp:16-24 (potrf) */
static int potrf_args(const char* uplo, const int* n, const int* lda, int* info) {
  *info = 0;
  if (!uplo_of(uplo)) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < max1(*n)) *info = -4;
  return *info;
}

/* Argument checks of lapack/cholesky.cpp:43-53 (potrs) */
static int potrs_args(const char* uplo, const int* n, const int* nrhs, const int* lda, const int* ldb, int* info) {
  *info = 0;
  if (!uplo_of(uplo)) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < max1(*n)) *info = -5;
  else if (*ldb < max1(*n)) *info = -7;
  return *info;
}

SHIM_API int dpotrf_(char* uplo, int* n, double* a, int* lda, int* info) {
  if (potrf_args(uplo, n, lda, info)) return arg_error("DPOTRF", *info);
  int64_t inf = 0;
  const int rc = gbllt_dpotrf(GBLLT_COL_MAJOR, uplo_of(uplo), *n, a, *lda, &inf);
  *info = rc ? rc : (int)inf;
  return 0;
}

SHIM_API int spotrf_(char* uplo, int* n, float* a, int* lda, int* info) {
  if (potrf_args(uplo, n, lda, info)) return arg_error("SPOTRF", *info);
  int64_t inf = 0;
  const int rc = gbllt_spotrf(GBLLT_COL_MAJOR, uplo_of(uplo), *n, a, *lda, &inf);
  *info = rc ? rc : (int)inf;
  return 0;
}

SHIM_API int dpotrs_(char* uplo, int* n, int* nrhs, double* a, int* lda, double* b, int* ldb, int* info) {
  if (potrs_args(uplo, n, nrhs, lda, ldb, info)) return arg_error("DPOTRS", *info);
  *info = gbllt_dpotrs(GBLLT_COL_MAJOR, uplo_of(uplo), *n, *nrhs, a, *lda, b, *ldb);
  return 0;
}

SHIM_API int spotrs_(char* uplo, int* n, int* nrhs, float* a, int* lda, float* b, int* ldb, int* info) {
  if (potrs_args(uplo, n, nrhs, lda, ldb, info)) return arg_error("SPOTRS", *info);
  *info = gbllt_spotrs(GBLLT_COL_MAJOR, uplo_of(uplo), *n, *nrhs, a, *lda, b, *ldb);
  return 0;
}

/* ---- BLAS level 3 ------------------------------------------------------------------------------ */

/* blas/common.h:47-62: the character codes the reference accepts */
static int op_ok(const char* c) { return c && (*c == 'N' || *c == 'n' || *c == 'T' || *c == 't' || *c == 'C' || *c == 'c'); }
static int op_is_n(const char* c) { return *c == 'N' || *c == 'n'; }
static int side_ok(const char* c) { return c && (*c == 'L' || *c == 'l' || *c == 'R' || *c == 'r'); }
static int side_is_left(const char* c) { return *c == 'L' || *c == 'l'; }
static int diag_ok(const char* c) { return c && (*c == 'N' || *c == 'n' || *c == 'U' || *c == 'u'); }

static int gpu_error(const char* name, int rc) {
  fprintf(stderr, "%s: GPU call failed with %d: %s\n", name, rc, gbllt_last_error());
  return rc;
}

/* Argument checks of blas/level3_impl.h:381-388 (syrk): positive position of the first bad one */
static int syrk_args(const char* uplo, const char* op, const int* n, const int* k, const int* lda, const int* ldc) {
  if (!uplo_of(uplo)) return 1;
  if (!op_ok(op)) return 2;
  if (*n < 0) return 3;
  if (*k < 0) return 4;
  if (*lda < max1(op_is_n(op) ? *n : *k)) return 7;
  if (*ldc < max1(*n)) return 10;
  return 0;
}

/* Argument checks of blas/level3_impl.h:136-146 (trsm) */
static int trsm_args(const char* side, const char* uplo, const char* op, const char* diag, const int* m, const int* n,
                     const int* lda, const int* ldb) {
  if (!side_ok(side)) return 1;
  if (!uplo_of(uplo)) return 2;
  if (!op_ok(op)) return 3;
  if (!diag_ok(diag)) return 4;
  if (*m < 0) return 5;
  if (*n < 0) return 6;
  if (*lda < max1(side_is_left(side) ? *m : *n)) return 9;
  if (*ldb < max1(*m)) return 11;
  return 0;
}

SHIM_API int dsyrk_(const char* uplo, const char* op, const int* n, const int* k, const double* alpha, const double* a,
                    const int* lda, const double* beta, double* c, const int* ldc) {
  int info = syrk_args(uplo, op, n, k, lda, ldc);
  if (info) return xerbla_("DSYRK ", &info, 6);
  const int rc = gbllt_dsyrk(GBLLT_COL_MAJOR, uplo_of(uplo), *op, *n, *k, *alpha, a, *lda, *beta, c, *ldc);
  return rc ? gpu_error("DSYRK", rc) : 0;
}

SHIM_API int ssyrk_(const char* uplo, const char* op, const int* n, const int* k, const float* alpha, const float* a,
                    const int* lda, const float* beta, float* c, const int* ldc) {
  int info = syrk_args(uplo, op, n, k, lda, ldc);
  if (info) return xerbla_("SSYRK ", &info, 6);
  const int rc = gbllt_ssyrk(GBLLT_COL_MAJOR, uplo_of(uplo), *op, *n, *k, *alpha, a, *lda, *beta, c, *ldc);
  return rc ? gpu_error("SSYRK", rc) : 0;
}

SHIM_API int dtrsm_(const char* side, const char* uplo, const char* op, const char* diag, const int* m, const int* n,
                    const double* alpha, const double* a, const int* lda, double* b, const int* ldb) {
  int info = trsm_args(side, uplo, op, diag, m, n, lda, ldb);
  if (info) return xerbla_("DTRSM ", &info, 6);
  const int rc = gbllt_dtrsm(GBLLT_COL_MAJOR, *side, uplo_of(uplo), *op, *diag, *m, *n, *alpha, a, *lda, b, *ldb);
  return rc ? gpu_error("DTRSM", rc) : 0;
}

SHIM_API int strsm_(const char* side, const char* uplo, const char* op, const char* diag, const int* m, const int* n,
                    const float* alpha, const float* a, const int* lda, float* b, const int* ldb) {
  int info = trsm_args(side, uplo, op, diag, m, n, lda, ldb);
  if (info) return xerbla_("STRSM ", &info, 6);
  const int rc = gbllt_strsm(GBLLT_COL_MAJOR, *side, uplo_of(uplo), *op, *diag, *m, *n, *alpha, a, *lda, b, *ldb);
  return rc ? gpu_error("STRSM", rc) : 0;
}
