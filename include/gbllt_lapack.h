/* Fortran-ABI LAPACK Cholesky routines and the BLAS level-3 routines of the Cholesky path
 * (dsyrk_, dtrsm_ and their single-precision twins) backed by the GB300 kernels (libgbllt_lapack.so).
 *
 * Same names, argument order and meaning as Eigen's LAPACK build of the Cholesky routines
 * (lapack/cholesky.cpp:14 potrf, :41 potrs; prototypes in Eigen/src/misc/lapack.h), which are the
 * reference LAPACK interface:
 *   - all arguments by reference, matrices column-major with leading dimension lda / ldb;
 *   - uplo 'L'/'l' or 'U'/'u';
 *   - *info = 0 on success, -i when argument i is illegal (after a call to xerbla_), and for potrf
 *     k + 1 when the leading minor of order k + 1 is not positive definite.
 * Beyond LAPACK: a GPU-side failure sets *info to a gbllt error code (GBLLT_ERR_*, <= -1001);
 * gbllt_last_error() describes it.  The return value is always 0, as in the reference, except that
 * the BLAS routines, which have no info argument, return the gbllt error code (and print the
 * message to stderr) after a GPU-side failure.
 */
#ifndef GBLLT_LAPACK_H
#define GBLLT_LAPACK_H

#include "gbllt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* replaces dpotrf_ / spotrf_ (lapack/cholesky.cpp:14-36) */
GBLLT_API int dpotrf_(char* uplo, int* n, double* a, int* lda, int* info);
GBLLT_API int spotrf_(char* uplo, int* n, float* a, int* lda, int* info);

/* replaces dpotrs_ / spotrs_ (lapack/cholesky.cpp:41-72) */
GBLLT_API int dpotrs_(char* uplo, int* n, int* nrhs, double* a, int* lda, double* b, int* ldb, int* info);
GBLLT_API int spotrs_(char* uplo, int* n, int* nrhs, float* a, int* lda, float* b, int* ldb, int* info);

/* replaces dsyrk_ / ssyrk_ (blas/level3_impl.h:355-417): C = alpha op(A) op(A)^T + beta C, `uplo` triangle */
GBLLT_API int dsyrk_(const char* uplo, const char* op, const int* n, const int* k, const double* alpha,
                     const double* a, const int* lda, const double* beta, double* c, const int* ldc);
GBLLT_API int ssyrk_(const char* uplo, const char* op, const int* n, const int* k, const float* alpha,
                     const float* a, const int* lda, const float* beta, float* c, const int* ldc);

/* replaces dtrsm_ / strsm_ (blas/level3_impl.h:78-160): B = alpha op(A)^{-1} B or alpha B op(A)^{-1} */
GBLLT_API int dtrsm_(const char* side, const char* uplo, const char* op, const char* diag, const int* m,
                     const int* n, const double* alpha, const double* a, const int* lda, double* b, const int* ldb);
GBLLT_API int strsm_(const char* side, const char* uplo, const char* op, const char* diag, const int* m,
                     const int* n, const float* alpha, const float* a, const int* lda, float* b, const int* ldb);

/* weak default error handler with the reference's message (blas/xerbla.cpp:15-19) */
GBLLT_API int xerbla_(const char* msg, int* info, int len);

#ifdef __cplusplus
}
#endif

#endif /* GBLLT_LAPACK_H */
