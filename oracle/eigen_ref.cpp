// C shim over Eigen's own dense Cholesky, compiled against the reference headers in place
// (oracle/Makefile, target `ref`).  TEST INFRASTRUCTURE ONLY: it produces the golden vectors
// that pin the oracle and lets the oracle be timed against Eigen on the same machine.
//
// Every function goes through Eigen's public LLT API (Eigen/src/Cholesky/LLT.h):
// LLT<Matrix,UpLo>::compute (:430-460), matrixLLT, info (:191-195) and solve (:483-498).
#include <Eigen/Cholesky>
#include <Eigen/Dense>
#include <chrono>
#include <cstdint>

using namespace Eigen;

template <typename T, int UpLo>
static int64_t factor_solve(int64_t n, int64_t nrhs, T* a, int64_t lda, T* b, int64_t ldb, double* seconds) {
  typedef Matrix<T, Dynamic, Dynamic> M;
  Map<M, 0, OuterStride<>> A(a, n, n, OuterStride<>(lda));
  auto t0 = std::chrono::steady_clock::now();
  LLT<M, UpLo> llt(A);                       // copies A, L1 norm, blocked factorisation
  auto t1 = std::chrono::steady_clock::now();
  int64_t info = llt.info() == Success ? 0 : 1;
  if (nrhs > 0 && info == 0) {
    Map<M, 0, OuterStride<>> B(b, n, nrhs, OuterStride<>(ldb));
    M X = llt.solve(B);
    B = X;
  }
  auto t2 = std::chrono::steady_clock::now();
  // write the factor back (only the UpLo triangle is meaningful)
  A.template triangularView<UpLo>() = llt.matrixLLT().template triangularView<UpLo>();
  if (seconds) {
    seconds[0] = std::chrono::duration<double>(t1 - t0).count();
    seconds[1] = std::chrono::duration<double>(t2 - t1).count();
  }
  return info;
}

// Failing column as returned by llt_inplace<T,UpLo>::blocked (LLT.h:338-368): -1 on success.
template <typename T, int UpLo>
static int64_t blocked(int64_t n, T* a, int64_t lda) {
  typedef Matrix<T, Dynamic, Dynamic> M;
  Map<M, 0, OuterStride<>> A(a, n, n, OuterStride<>(lda));
  return (int64_t)internal::llt_inplace<T, UpLo>::blocked(A);
}

// LLT<Matrix,UpLo>(A).rcond() (LLT.h:166-171): Eigen's own 1-norm and condition estimate.
template <typename T, int UpLo>
static double rcond(int64_t n, const T* a, int64_t lda) {
  typedef Matrix<T, Dynamic, Dynamic> M;
  Map<const M, 0, OuterStride<>> A(a, n, n, OuterStride<>(lda));
  LLT<M, UpLo> llt(A);
  if (llt.info() != Success) return -1.0;
  return (double)llt.rcond();
}

// LLT<Matrix,UpLo>::rankUpdate(v, sigma) (LLT.h:469-478) on the factor of A; the updated factor
// is written back to a (its UpLo triangle), returns 0 on success, 1 when Eigen reports
// NumericalIssue.
template <typename T, int UpLo>
static int64_t rank_update(int64_t n, T* a, int64_t lda, const T* v, T sigma) {
  typedef Matrix<T, Dynamic, Dynamic> M;
  typedef Matrix<T, Dynamic, 1> V;
  Map<M, 0, OuterStride<>> A(a, n, n, OuterStride<>(lda));
  LLT<M, UpLo> llt(A);
  if (llt.info() != Success) return 2;
  llt.rankUpdate(Map<const V>(v, n), sigma);
  A.template triangularView<UpLo>() = llt.matrixLLT().template triangularView<UpLo>();
  return llt.info() == Success ? 0 : 1;
}

// LDLT<Matrix,UpLo>(A) (LDLT.h:497-530): the factor (UpLo triangle of matrixLDLT()) is written back
// to a, the transpositions to transp, Eigen's sign (0 PositiveSemiDef, 1 NegativeSemiDef, 2 ZeroSign,
// 3 Indefinite, recovered from isPositive()/isNegative(), LDLT.h:178-190) to *sign; returns 0 for
// Success, 1 for NumericalIssue.
template <typename T, int UpLo>
static int64_t ldlt(int64_t n, T* a, int64_t lda, int32_t* transp, int32_t* sign) {
  typedef Matrix<T, Dynamic, Dynamic> M;
  Map<M, 0, OuterStride<>> A(a, n, n, OuterStride<>(lda));
  LDLT<M, UpLo> f(A);
  A.template triangularView<UpLo>() = f.matrixLDLT().template triangularView<UpLo>();
  for (int64_t k = 0; k < n; ++k) transp[k] = (int32_t)f.transpositionsP().indices()(k);
  const bool pos = f.isPositive(), neg = f.isNegative();
  *sign = pos && neg ? 2 : pos ? 0 : neg ? 1 : 3;
  return f.info() == Success ? 0 : 1;
}

// x = LDLT<Matrix,UpLo>(A).solve(b) (LDLT.h:573-613), b overwritten by x.
template <typename T, int UpLo>
static void ldlt_solve(int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb) {
  typedef Matrix<T, Dynamic, Dynamic> M;
  Map<const M, 0, OuterStride<>> A(a, n, n, OuterStride<>(lda));
  Map<M, 0, OuterStride<>> B(b, n, nrhs, OuterStride<>(ldb));
  LDLT<M, UpLo> f(A);
  M X = f.solve(B);
  B = X;
}

extern "C" {

int64_t ref_drank_update(char uplo, int64_t n, double* a, int64_t lda, const double* v, double sigma) {
  return uplo == 'U' ? rank_update<double, Upper>(n, a, lda, v, sigma) : rank_update<double, Lower>(n, a, lda, v, sigma);
}
int64_t ref_srank_update(char uplo, int64_t n, float* a, int64_t lda, const float* v, float sigma) {
  return uplo == 'U' ? rank_update<float, Upper>(n, a, lda, v, sigma) : rank_update<float, Lower>(n, a, lda, v, sigma);
}

double ref_drcond(char uplo, int64_t n, const double* a, int64_t lda) {
  return uplo == 'U' ? rcond<double, Upper>(n, a, lda) : rcond<double, Lower>(n, a, lda);
}
double ref_srcond(char uplo, int64_t n, const float* a, int64_t lda) {
  return uplo == 'U' ? rcond<float, Upper>(n, a, lda) : rcond<float, Lower>(n, a, lda);
}

int64_t ref_dllt(char uplo, int64_t n, int64_t nrhs, double* a, int64_t lda, double* b, int64_t ldb, double* sec) {
  return uplo == 'U' ? factor_solve<double, Upper>(n, nrhs, a, lda, b, ldb, sec)
                     : factor_solve<double, Lower>(n, nrhs, a, lda, b, ldb, sec);
}
int64_t ref_sllt(char uplo, int64_t n, int64_t nrhs, float* a, int64_t lda, float* b, int64_t ldb, double* sec) {
  return uplo == 'U' ? factor_solve<float, Upper>(n, nrhs, a, lda, b, ldb, sec)
                     : factor_solve<float, Lower>(n, nrhs, a, lda, b, ldb, sec);
}
int64_t ref_dblocked(char uplo, int64_t n, double* a, int64_t lda) {
  return uplo == 'U' ? blocked<double, Upper>(n, a, lda) : blocked<double, Lower>(n, a, lda);
}
int64_t ref_sblocked(char uplo, int64_t n, float* a, int64_t lda) {
  return uplo == 'U' ? blocked<float, Upper>(n, a, lda) : blocked<float, Lower>(n, a, lda);
}

int64_t ref_dldlt(char uplo, int64_t n, double* a, int64_t lda, int32_t* transp, int32_t* sign) {
  return uplo == 'U' ? ldlt<double, Upper>(n, a, lda, transp, sign) : ldlt<double, Lower>(n, a, lda, transp, sign);
}
int64_t ref_sldlt(char uplo, int64_t n, float* a, int64_t lda, int32_t* transp, int32_t* sign) {
  return uplo == 'U' ? ldlt<float, Upper>(n, a, lda, transp, sign) : ldlt<float, Lower>(n, a, lda, transp, sign);
}
void ref_dldlt_solve(char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda, double* b, int64_t ldb) {
  if (uplo == 'U') ldlt_solve<double, Upper>(n, nrhs, a, lda, b, ldb);
  else ldlt_solve<double, Lower>(n, nrhs, a, lda, b, ldb);
}
void ref_sldlt_solve(char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda, float* b, int64_t ldb) {
  if (uplo == 'U') ldlt_solve<float, Upper>(n, nrhs, a, lda, b, ldb);
  else ldlt_solve<float, Lower>(n, nrhs, a, lda, b, ldb);
}

}  // extern "C"
