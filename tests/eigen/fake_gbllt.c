/* Test double of libgbllt for checking include/eigen_gb300/LLT_GB300.h on a machine without a GPU.
 *
 * TEST INFRASTRUCTURE ONLY.  It implements the entry points the Eigen header calls by
 * forwarding to the oracle (oracle/llt_oracle.c), applying the same layout rule as the real
 * library (a row-major factor with uplo 'L' is a column-major one with uplo 'U'), and counts the
 * calls so that a test can prove the specialisations were selected.  It never ships. */
#include <stdint.h>
#include <stdio.h>

#include "../../include/gbllt.h"

int oracle_dpotrf(char uplo, int64_t n, double* a, int64_t lda, int64_t* info);
int oracle_spotrf(char uplo, int64_t n, float* a, int64_t lda, int64_t* info);
int oracle_dpotrs(char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda, double* b, int64_t ldb);
int oracle_spotrs(char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda, float* b, int64_t ldb);
int64_t oracle_drank_update(char uplo, int64_t n, double* l, int64_t ldl, const double* v, double sigma);
int64_t oracle_srank_update(char uplo, int64_t n, float* l, int64_t ldl, const float* v, float sigma);
double oracle_drcond(char uplo, int64_t n, const double* l, int64_t ldl, double anorm);
double oracle_srcond(char uplo, int64_t n, const float* l, int64_t ldl, double anorm);
int oracle_dldlt(char uplo, int64_t n, double* a, int64_t lda, int* transp, int* sign);
int oracle_sldlt(char uplo, int64_t n, float* a, int64_t lda, int* transp, int* sign);
void oracle_dldlt_solve(char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda, const int* transp, double* b,
                        int64_t ldb);
void oracle_sldlt_solve(char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda, const int* transp, float* b,
                        int64_t ldb);

void oracle_dtrsm(char side, char uplo, char op, char diag, int64_t m, int64_t n, double alpha, const double* a,
                  int64_t lda, double* b, int64_t ldb);
void oracle_strsm(char side, char uplo, char op, char diag, int64_t m, int64_t n, float alpha, const float* a,
                  int64_t lda, float* b, int64_t ldb);

long fake_calls[14];

static char eff_uplo(int layout, char uplo) {
  const int up = uplo == 'U' || uplo == 'u';
  return (layout == GBLLT_ROW_MAJOR) ? (up ? 'L' : 'U') : (up ? 'U' : 'L');
}

const char* gbllt_last_error(void) { return "fake"; }
int gbllt_dpotrf(int layout, char uplo, int64_t n, double* a, int64_t lda, int64_t* info) {
  ++fake_calls[0];
  return oracle_dpotrf(eff_uplo(layout, uplo), n, a, lda, info);
}
int gbllt_spotrf(int layout, char uplo, int64_t n, float* a, int64_t lda, int64_t* info) {
  ++fake_calls[1];
  return oracle_spotrf(eff_uplo(layout, uplo), n, a, lda, info);
}
int gbllt_dpotrs(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda, double* b, int64_t ldb) {
  ++fake_calls[2];
  if (layout != GBLLT_COL_MAJOR) return -1;
  return oracle_dpotrs(uplo, n, nrhs, a, lda, b, ldb);
}
int gbllt_spotrs(int layout, char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda, float* b, int64_t ldb) {
  ++fake_calls[3];
  if (layout != GBLLT_COL_MAJOR) return -1;
  return oracle_spotrs(uplo, n, nrhs, a, lda, b, ldb);
}

int gbllt_dpocon(int layout, char uplo, int64_t n, const double* l, int64_t ldl, double anorm, double* rcond) {
  ++fake_calls[4];
  *rcond = oracle_drcond(eff_uplo(layout, uplo), n, l, ldl, anorm);
  return 0;
}
int gbllt_spocon(int layout, char uplo, int64_t n, const float* l, int64_t ldl, float anorm, float* rcond) {
  ++fake_calls[5];
  *rcond = (float)oracle_srcond(eff_uplo(layout, uplo), n, l, ldl, anorm);
  return 0;
}

int gbllt_drank_update(int layout, char uplo, int64_t n, double* l, int64_t ldl, const double* v, double sigma,
                       int64_t* info) {
  ++fake_calls[6];
  const int64_t r = oracle_drank_update(eff_uplo(layout, uplo), n, l, ldl, v, sigma);
  *info = r < 0 ? 0 : r + 1;
  return 0;
}
int gbllt_srank_update(int layout, char uplo, int64_t n, float* l, int64_t ldl, const float* v, float sigma,
                       int64_t* info) {
  ++fake_calls[7];
  const int64_t r = oracle_srank_update(eff_uplo(layout, uplo), n, l, ldl, v, sigma);
  *info = r < 0 ? 0 : r + 1;
  return 0;
}

int gbllt_dldlt(int layout, char uplo, int64_t n, double* a, int64_t lda, int32_t* transp, int32_t* sign,
                int64_t* info) {
  ++fake_calls[8];
  *info = oracle_dldlt(eff_uplo(layout, uplo), n, a, lda, transp, sign) ? 0 : 1;
  return 0;
}
int gbllt_sldlt(int layout, char uplo, int64_t n, float* a, int64_t lda, int32_t* transp, int32_t* sign,
                int64_t* info) {
  ++fake_calls[9];
  *info = oracle_sldlt(eff_uplo(layout, uplo), n, a, lda, transp, sign) ? 0 : 1;
  return 0;
}
int gbllt_dldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const double* a, int64_t lda,
                      const int32_t* transp, double* b, int64_t ldb) {
  ++fake_calls[10];
  if (layout != GBLLT_COL_MAJOR) return -1;
  oracle_dldlt_solve(uplo, n, nrhs, a, lda, transp, b, ldb);
  return 0;
}
int gbllt_sldlt_solve(int layout, char uplo, int64_t n, int64_t nrhs, const float* a, int64_t lda,
                      const int32_t* transp, float* b, int64_t ldb) {
  ++fake_calls[11];
  if (layout != GBLLT_COL_MAJOR) return -1;
  oracle_sldlt_solve(uplo, n, nrhs, a, lda, transp, b, ldb);
  return 0;
}

int gbllt_dtrsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n, double alpha,
                const double* a, int64_t lda, double* b, int64_t ldb) {
  ++fake_calls[12];
  if (layout != GBLLT_COL_MAJOR) return -1;
  oracle_dtrsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
  return 0;
}
int gbllt_strsm(int layout, char side, char uplo, char transa, char diag, int64_t m, int64_t n, float alpha,
                const float* a, int64_t lda, float* b, int64_t ldb) {
  ++fake_calls[13];
  if (layout != GBLLT_COL_MAJOR) return -1;
  oracle_strsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
  return 0;
}

/* Prints the call counts at exit so that the test can check the backend was used. */
__attribute__((destructor)) static void fake_report(void) {
  fprintf(stderr,
          "fake_gbllt calls: dpotrf=%ld spotrf=%ld dpotrs=%ld spotrs=%ld dpocon=%ld spocon=%ld drankupd=%ld "
          "srankupd=%ld dldlt=%ld sldlt=%ld dldlts=%ld sldlts=%ld dtrsm=%ld strsm=%ld\n",
          fake_calls[0], fake_calls[1], fake_calls[2], fake_calls[3], fake_calls[4], fake_calls[5], fake_calls[6],
          fake_calls[7], fake_calls[8], fake_calls[9], fake_calls[10], fake_calls[11], fake_calls[12],
          fake_calls[13]);
}
