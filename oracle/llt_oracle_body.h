/* Scalar-generic body of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Included twice by llt_oracle.c, once with T=double / P(x)=oracle_d##x and once with
 * T=float / P(x)=oracle_s##x.  Every routine restates the algorithm of the Eigen source it
 * cites; the arithmetic is done in T, like Eigen's LLT<Matrix<T,...>>.
 *
 * A matrix is addressed through (rs, cs) strides: element (i, j) lives at p[i*rs + j*cs].
 * A column-major lower factor uses (1, lda); a column-major UPPER factor is the lower factor
 * of the transpose, i.e. (lda, 1) -- the same trick as llt_inplace<Scalar,Upper> in
 * Eigen/src/Cholesky/LLT.h:377-399, which runs the Lower algorithm on Transpose<MatrixType>.
 */

#define EL(p, i, j) (p)[(int64_t)(i) * rs + (int64_t)(j) * cs]

/* Left-looking unblocked factorisation of one diagonal block.
 * Restates llt_inplace<Scalar,Lower>::unblocked, Eigen/src/Cholesky/LLT.h:312-336:
 *   x = a_kk - ||A10||^2 ; x <= 0 -> return k ; a_kk = sqrt(x) ;
 *   A21 -= A20 * A10^T (a GEMV) ; A21 /= a_kk.
 * Returns -1 on success, else the failing column. */
int64_t P(llt_unblocked)(int64_t n, T* a, int64_t rs, int64_t cs) {
  for (int64_t k = 0; k < n; ++k) {
    const int64_t r = n - k - 1;
    T x = EL(a, k, k);
    T ss = 0;
    for (int64_t p = 0; p < k; ++p) ss += EL(a, k, p) * EL(a, k, p);
    x -= ss;
    if (x <= (T)0) return k;   /* same test as LLT.h:329: a NaN pivot does not stop it */
    x = (T)sqrt((double)x);   /* correctly rounded in T for both float and double */
    EL(a, k, k) = x;
    if (r > 0) {
      /* GEMV A21 -= A20 * A10^T, column-oriented (axpy per column of A20) */
      for (int64_t p = 0; p < k; ++p) {
        const T akp = EL(a, k, p);
        for (int64_t i = k + 1; i < n; ++i) EL(a, i, k) -= EL(a, i, p) * akp;
      }
      for (int64_t i = k + 1; i < n; ++i) EL(a, i, k) /= x;
    }
  }
  return -1;
}

/* Panel triangular solve A21 <- A21 * L11^{-T}, L11 lower bs x bs, A21 m x bs.
 * Restates the OnTheRight solve that LLT.h:364 issues
 * (triangular_solve_matrix<...,OnTheRight,...>, Eigen/src/Core/products/TriangularSolverMatrix.h:188-329):
 * column j of X is (A21(:,j) - sum_{p<j} X(:,p) L11(j,p)) / L11(j,j).
 * Rows are independent, so the row range is split over threads; each element sees the same
 * operation order whatever the thread count. */
static void P(trsm_right_lt)(int64_t m, int64_t bs, const T* l11, int64_t lrs, int64_t lcs,
                             T* a21, int64_t rs, int64_t cs) {
  const int64_t RB = 256;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int64_t r0 = 0; r0 < m; r0 += RB) {
    const int64_t r1 = r0 + RB < m ? r0 + RB : m;
    for (int64_t j = 0; j < bs; ++j) {
      for (int64_t p = 0; p < j; ++p) {
        const T ljp = l11[j * lrs + p * lcs];
        for (int64_t i = r0; i < r1; ++i) EL(a21, i, j) -= EL(a21, i, p) * ljp;
      }
      const T ljj = l11[j * lrs + j * lcs];
      for (int64_t i = r0; i < r1; ++i) EL(a21, i, j) /= ljj;
    }
  }
}

/* Lower SYRK  C -= A * A^T  (C m x m lower, A m x k).
 * Restates the rankUpdate issued at LLT.h:365 (SelfadjointProduct.h:82-117 ->
 * general_matrix_matrix_triangular_product, GeneralMatrixMatrixTriangular.h:57-194):
 * A is packed once into row strips of MR and column strips of NR (the role of
 * gemm_pack_lhs / gemm_pack_rhs, GeneralBlockPanelKernel.h:2236+, 2524+), and an MR x NR
 * register-blocked micro-kernel (the role of gebp_kernel, :1548+) accumulates over the full
 * depth k before subtracting from C.  Only tiles on or below the diagonal are touched, and
 * inside a diagonal tile only the lower half is written (the role of tribb_kernel, :138-194).
 * Per element, the sum runs over p = 0..k-1 in order and is then subtracted: the result does not
 * depend on the thread count. */
#define ORC_MR 8
#define ORC_NR 4
static void P(syrk_lower_sub)(int64_t m, int64_t k, const T* a, int64_t ars, int64_t acs,
                              T* c, int64_t rs, int64_t cs) {
  if (m <= 0 || k <= 0) return;
  const int64_t mp = (m + ORC_MR - 1) / ORC_MR * ORC_MR;
  const int64_t np = (m + ORC_NR - 1) / ORC_NR * ORC_NR;
  T* pa = (T*)calloc((size_t)(mp * k), sizeof(T));   /* [m/MR][k][MR] */
  T* pb = (T*)calloc((size_t)(np * k), sizeof(T));   /* [m/NR][k][NR] */
  for (int64_t i = 0; i < m; ++i)
    for (int64_t p = 0; p < k; ++p) {
      const T v = a[i * ars + p * acs];
      pa[(i / ORC_MR) * k * ORC_MR + p * ORC_MR + (i % ORC_MR)] = v;
      pb[(i / ORC_NR) * k * ORC_NR + p * ORC_NR + (i % ORC_NR)] = v;
    }
  const int64_t nstrips = np / ORC_NR;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t js = 0; js < nstrips; ++js) {
    const int64_t j0 = js * ORC_NR;
    const T* bp = pb + js * k * ORC_NR;
    for (int64_t i0 = (j0 / ORC_MR) * ORC_MR; i0 < m; i0 += ORC_MR) {
      const T* ap = pa + (i0 / ORC_MR) * k * ORC_MR;
      T acc[ORC_NR][ORC_MR];
      for (int jj = 0; jj < ORC_NR; ++jj)
        for (int ii = 0; ii < ORC_MR; ++ii) acc[jj][ii] = 0;
      for (int64_t p = 0; p < k; ++p) {
        const T* av = ap + p * ORC_MR;
        const T* bv = bp + p * ORC_NR;
        for (int jj = 0; jj < ORC_NR; ++jj)
          for (int ii = 0; ii < ORC_MR; ++ii) acc[jj][ii] += av[ii] * bv[jj];
      }
      for (int jj = 0; jj < ORC_NR; ++jj) {
        const int64_t j = j0 + jj;
        if (j >= m) break;
        for (int ii = 0; ii < ORC_MR; ++ii) {
          const int64_t i = i0 + ii;
          if (i >= m) break;
          if (i >= j) EL(c, i, j) -= acc[jj][ii];
        }
      }
    }
  }
  free(pa);
  free(pb);
}

/* Right-looking blocked factorisation.
 * Restates llt_inplace<Scalar,Lower>::blocked, Eigen/src/Cholesky/LLT.h:338-368:
 * n < 32 -> unblocked; blockSize = clamp((n/8)/16*16, 8, 128); per panel:
 * unblocked(A11), A21 <- A21 L11^{-T}, A22 -= A21 A21^T (lower).
 * Returns -1 on success, else the failing column (k + ret, :363). */
int64_t P(llt_blocked)(int64_t n, T* a, int64_t rs, int64_t cs) {
  if (n < 32) return P(llt_unblocked)(n, a, rs, cs);
  int64_t bsz = n / 8;
  bsz = (bsz / 16) * 16;
  if (bsz < 8) bsz = 8;
  if (bsz > 128) bsz = 128;
  for (int64_t k = 0; k < n; k += bsz) {
    const int64_t bs = bsz < n - k ? bsz : n - k;
    const int64_t r = n - k - bs;
    T* a11 = &EL(a, k, k);
    int64_t ret = P(llt_unblocked)(bs, a11, rs, cs);
    if (ret >= 0) return k + ret;
    if (r > 0) {
      T* a21 = &EL(a, k + bs, k);
      P(trsm_right_lt)(r, bs, a11, rs, cs, a21, rs, cs);
      P(syrk_lower_sub)(r, bs, a21, rs, cs, &EL(a, k + bs, k + bs), rs, cs);
    }
  }
  return -1;
}

/* LAPACK-shaped wrapper: the mapping lapack/cholesky.cpp:14-36 performs around
 * llt_inplace::blocked (argument checks -1/-2/-4, then info = ret + 1).
 * uplo 'L'/'l' or 'U'/'u'; column-major storage with leading dimension lda. */
int P(potrf)(char uplo, int64_t n, T* a, int64_t lda, int64_t* info) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int lo = (uplo == 'L' || uplo == 'l');
  *info = 0;
  if (!up && !lo) { *info = -1; return -1; }
  if (n < 0) { *info = -2; return -2; }
  if (lda < (n > 1 ? n : 1)) { *info = -4; return -4; }
  if (n == 0) return 0;
  const int64_t ret = up ? P(llt_blocked)(n, a, lda, 1) : P(llt_blocked)(n, a, 1, lda);
  if (ret >= 0) *info = ret + 1;
  return 0;
}

/* Solve A X = B in place in B from the factor, restating LLT::_solve_impl_transposed
 * (Eigen/src/Cholesky/LLT.h:483-498) = matrixL().solveInPlace then matrixU().solveInPlace, and
 * the potrs wrapper lapack/cholesky.cpp:41-72.  Both sweeps walk the columns of L, which are
 * contiguous for a lower column-major factor (the forward sweep is an axpy per column, the
 * backward sweep a dot per column, cf. TriangularSolverVector.h:88-142 and :30-85). */
int P(potrs)(char uplo, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int lo = (uplo == 'L' || uplo == 'l');
  if (!up && !lo) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (ldb < (n > 1 ? n : 1)) return -7;
  const int64_t rs = up ? lda : 1, cs = up ? 1 : lda;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int64_t c = 0; c < nrhs; ++c) {
    T* x = b + c * ldb;
    for (int64_t j = 0; j < n; ++j) {          /* L y = b */
      const T yj = x[j] / EL(a, j, j);
      x[j] = yj;
      for (int64_t i = j + 1; i < n; ++i) x[i] -= EL(a, i, j) * yj;
    }
    for (int64_t j = n - 1; j >= 0; --j) {     /* L^T x = y */
      T s = x[j];
      for (int64_t i = j + 1; i < n; ++i) s -= EL(a, i, j) * x[i];
      x[j] = s / EL(a, j, j);
    }
  }
  return 0;
}

/* Normwise backward error ||A X - B||_F / (||A||_F ||X||_F) with A symmetric, of which only
 * the `uplo` triangle is read (the same triangle LLT::compute reads).  The residual is
 * accumulated in double-double (error-free TwoSum / TwoProduct via fma; Dekker 1971,
 * Ogita-Rump-Oishi 2005), so that values around 1e-17 are resolved. */
double P(backward_error)(char uplo, int64_t n, int64_t nrhs, const T* a, int64_t lda,
                         const T* x, int64_t ldx, const T* b, int64_t ldb) {
  const int up = (uplo == 'U' || uplo == 'u');
  double na = 0, nx = 0, nr = 0;
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) {
      const double v = (i >= j) != up || i == j ? (double)a[i + j * lda] : (double)a[j + i * lda];
      na += v * v;
    }
  for (int64_t c = 0; c < nrhs; ++c)
    for (int64_t i = 0; i < n; ++i) nx += (double)x[i + c * ldx] * (double)x[i + c * ldx];
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : nr) schedule(static)
#endif
  for (int64_t c = 0; c < nrhs; ++c) {
    for (int64_t i = 0; i < n; ++i) {
      double hi = -(double)b[i + c * ldb], lo = 0;
      for (int64_t j = 0; j < n; ++j) {
        const int lower_el = i >= j;
        const double aij = (lower_el != up || i == j) ? (double)a[i + j * lda] : (double)a[j + i * lda];
        const double xv = (double)x[j + c * ldx];
        const double ph = aij * xv;
        const double pl = fma(aij, xv, -ph);
        const double s = hi + ph;
        const double bb = s - hi;
        const double e = (hi - (s - bb)) + (ph - bb);
        hi = s;
        lo += e + pl;
      }
      const double r = hi + lo;
      nr += r * r;
    }
  }
  if (na == 0 || nx == 0) return nr == 0 ? 0.0 : INFINITY;
  return sqrt(nr) / (sqrt(na) * sqrt(nx));
}


/* 1-norm of the symmetric matrix of which only the `uplo` triangle of the column-major a is read:
 * the m_l1_norm loop of LLT::compute (Eigen/src/Cholesky/LLT.h:443-453), column by column, the
 * stored part of column j plus the stored part of row j. */
T P(sym_l1_norm)(char uplo, int64_t n, const T* a, int64_t lda) {
  const int up = (uplo == 'U' || uplo == 'u');
  T best = 0;
  for (int64_t j = 0; j < n; ++j) {
    T s = 0;
    if (!up) {
      for (int64_t i = j; i < n; ++i) s += (T)fabs((double)a[i + j * lda]);   /* col(j).tail(n-j) */
      for (int64_t k = 0; k < j; ++k) s += (T)fabs((double)a[j + k * lda]);   /* row(j).head(j)   */
    } else {
      for (int64_t i = 0; i < j; ++i) s += (T)fabs((double)a[i + j * lda]);   /* col(j).head(j)   */
      for (int64_t k = j; k < n; ++k) s += (T)fabs((double)a[j + k * lda]);   /* row(j).tail(n-j) */
    }
    if (s > best) best = s;
  }
  return best;
}

static T P(vec_l1)(int64_t n, const T* v) {
  T s = 0;
  for (int64_t i = 0; i < n; ++i) s += (T)fabs((double)v[i]);
  return s;
}

/* Reciprocal condition estimate from the factor: rcond_estimate_helper and
 * rcond_invmatrix_L1_norm_estimate (Eigen/src/Core/ConditionEstimator.h:56-171), restated step by
 * step over this oracle's potrs (the LLT solve; A is symmetric, so dec.adjoint().solve is the same
 * solve).  Returns +inf for n = 0, 0 for anorm = 0, 1 for n = 1 (:165-167). */
double P(rcond)(char uplo, int64_t n, const T* l, int64_t ldl, double anorm) {
  if (n == 0) return INFINITY;
  if (anorm == 0) return 0.0;
  if (n == 1) return 1.0;
  T* v = (T*)malloc(sizeof(T) * n);
  T* sign = (T*)malloc(sizeof(T) * n);
  T* old_sign = (T*)malloc(sizeof(T) * n);
  for (int64_t i = 0; i < n; ++i) v[i] = (T)1 / (T)n;                 /* :79 */
  P(potrs)(uplo, n, 1, l, ldl, v, n);
  T lower = P(vec_l1)(n, v);                                            /* :88 */
  T old_lower = lower;
  int64_t old_idx = -1;
  for (int k = 0; k < 4; ++k) {                                         /* :100-128 */
    int same = k > 0;
    for (int64_t i = 0; i < n; ++i) {
      sign[i] = v[i] < (T)0 ? (T)-1 : (T)1;                            /* :29-35 */
      if (k > 0 && sign[i] != old_sign[i]) same = 0;
    }
    if (k > 0 && same) break;
    for (int64_t i = 0; i < n; ++i) v[i] = sign[i];
    P(potrs)(uplo, n, 1, l, ldl, v, n);
    int64_t idx = 0;                                                    /* first max |v| */
    T mx = (T)fabs((double)v[0]);
    for (int64_t i = 1; i < n; ++i)
      if ((T)fabs((double)v[i]) > mx) { mx = (T)fabs((double)v[i]); idx = i; }
    if (idx == old_idx) break;
    for (int64_t i = 0; i < n; ++i) v[i] = (T)(i == idx ? 1 : 0);
    P(potrs)(uplo, n, 1, l, ldl, v, n);
    lower = P(vec_l1)(n, v);
    if (lower <= old_lower) break;
    for (int64_t i = 0; i < n; ++i) old_sign[i] = sign[i];
    old_idx = idx;
    old_lower = lower;
  }
  T alt_sign = (T)1;                                                    /* :141-147 */
  for (int64_t i = 0; i < n; ++i) {
    v[i] = alt_sign * ((T)1 + (T)i / (T)(n - 1));
    alt_sign = -alt_sign;
  }
  P(potrs)(uplo, n, 1, l, ldl, v, n);
  const T alt = ((T)2 * P(vec_l1)(n, v)) / ((T)3 * (T)n);
  const T est = lower > alt ? lower : alt;
  free(v);
  free(sign);
  free(old_sign);
  return est == (T)0 ? 0.0 : ((double)((T)1 / est) / anorm);
}

/* Rank-1 update / downdate of a Cholesky factor, A + sigma v v^T = L' L'^T: the restatement of
 * llt_rank_update_lower (Eigen/src/Cholesky/LLT.h:238-307) on the `uplo` triangle of the
 * column-major l (Upper runs the same steps on the transpose, LLT.h:394-398; real scalars, so the
 * vector's conjugate is itself).  sigma > 0: Givens rotations, with JacobiRotation::makeGivens
 * (Eigen/src/Jacobi/Jacobi.h:231-267) and the plane rotation of Jacobi.h:327-335; sigma <= 0: the
 * beta recurrence, which returns the column j at which x <= 0 (the factor is then partly updated).
 * Returns -1 on success, like llt_rank_update_lower. */
int64_t P(rank_update)(char uplo, int64_t n, T* l, int64_t ldl, const T* v, T sigma) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int64_t rs = up ? ldl : 1, cs = up ? 1 : ldl;  /* EL(l, i, j) = L(i, j) of the lower view */
  T* temp = (T*)malloc(sizeof(T) * (n > 0 ? n : 1));
  int64_t ret = -1;
  if (sigma > 0) {
    const T ss = (T)sqrt((double)sigma);
    for (int64_t i = 0; i < n; ++i) temp[i] = ss * v[i];
    for (int64_t i = 0; i < n; ++i) {
      const T p = EL(l, i, i), q = -temp[i];
      T c, s, r;
      if (q == 0) {
        c = p < 0 ? (T)-1 : (T)1;
        s = 0;
        r = (T)fabs((double)p);
      } else if (p == 0) {
        c = 0;
        s = q < 0 ? (T)1 : (T)-1;
        r = (T)fabs((double)q);
      } else if (fabs((double)p) > fabs((double)q)) {
        const T t = q / p;
        T u = (T)sqrt((double)((T)1 + t * t));
        if (p < 0) u = -u;
        c = (T)1 / u;
        s = -t * c;
        r = p * u;
      } else {
        const T t = p / q;
        T u = (T)sqrt((double)((T)1 + t * t));
        if (q < 0) u = -u;
        s = -(T)1 / u;
        c = -t * s;
        r = q * u;
      }
      EL(l, i, i) = r;
      for (int64_t k = i + 1; k < n; ++k) {
        const T xk = EL(l, k, i), yk = temp[k];
        EL(l, k, i) = c * xk + s * yk;
        temp[k] = -s * xk + c * yk;
      }
    }
  } else {
    for (int64_t i = 0; i < n; ++i) temp[i] = v[i];
    T beta = 1;
    for (int64_t j = 0; j < n; ++j) {
      const T Ljj = EL(l, j, j);
      const T dj = Ljj * Ljj;
      const T wj = temp[j];
      const T swj2 = sigma * wj * wj;
      const T gamma = dj * beta + swj2;
      const T x = dj + swj2 / beta;
      if (x <= 0) {
        ret = j;
        break;
      }
      const T nLjj = (T)sqrt((double)x);
      EL(l, j, j) = nLjj;
      beta += swj2 / dj;
      const T f = wj / Ljj;
      const T a = nLjj / Ljj;
      const T b = nLjj * sigma * wj / gamma;
      for (int64_t k = j + 1; k < n; ++k) {
        temp[k] -= f * EL(l, k, j);
        if (gamma != 0) EL(l, k, j) = a * EL(l, k, j) + b * temp[k];
      }
    }
  }
  free(temp);
  return ret;
}


/* LDL^T with Eigen's symmetric pivoting: the restatement of ldlt_inplace<Lower>::unblocked
 * (Eigen/src/Cholesky/LDLT.h:297-403) on the `uplo` triangle of the column-major a (Upper runs the
 * same steps on the transpose, LDLT.h:460-466).  On return the lower view holds L (unit diagonal
 * not stored) and D on the diagonal; transp[k] is the row swapped with row k at step k; *sign is
 * Eigen's SignMatrix (0 PositiveSemiDef, 1 NegativeSemiDef, 2 ZeroSign, 3 Indefinite).  Returns 1
 * for success (Eigen's `ret`), 0 for NumericalIssue.  The column update is left-looking, as in the
 * reference: A11 -= A10 D A10^T, A21 -= A20 D A10^T, then A21 /= A11 unless the pivot is 0. */
int P(ldlt)(char uplo, int64_t n, T* a, int64_t lda, int* transp, int* sign) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int64_t rs = up ? lda : 1, cs = up ? 1 : lda;
  int ret = 1, found_zero = 0;
  *sign = 2; /* ZeroSign */
  if (n <= 1) {
    for (int64_t i = 0; i < n; ++i) transp[i] = (int)i;
    if (n == 1) {
      const T a00 = EL(a, 0, 0);
      *sign = a00 > 0 ? 0 : (a00 < 0 ? 1 : 2);
    }
    return 1;
  }
  T* temp = (T*)malloc(sizeof(T) * n);
  for (int64_t k = 0; k < n; ++k) {
    /* largest |diagonal| in the corner, first index on ties (LDLT.h:323-326) */
    int64_t p = k;
    T best = (T)fabs((double)EL(a, k, k));
    for (int64_t i = k + 1; i < n; ++i) {
      const T v = (T)fabs((double)EL(a, i, i));
      if (v > best) { best = v; p = i; }
    }
    transp[k] = (int)p;
    if (p != k) { /* the swap of LDLT.h:329-345, lower triangle only */
      for (int64_t j = 0; j < k; ++j) { const T t = EL(a, k, j); EL(a, k, j) = EL(a, p, j); EL(a, p, j) = t; }
      for (int64_t i = p + 1; i < n; ++i) { const T t = EL(a, i, k); EL(a, i, k) = EL(a, i, p); EL(a, i, p) = t; }
      { const T t = EL(a, k, k); EL(a, k, k) = EL(a, p, p); EL(a, p, p) = t; }
      for (int64_t i = k + 1; i < p; ++i) { const T t = EL(a, i, k); EL(a, i, k) = EL(a, p, i); EL(a, p, i) = t; }
    }
    if (k > 0) { /* LDLT.h:356-362 */
      for (int64_t j = 0; j < k; ++j) temp[j] = EL(a, j, j) * EL(a, k, j);
      T s = 0;
      for (int64_t j = 0; j < k; ++j) s += EL(a, k, j) * temp[j];
      EL(a, k, k) -= s;
      for (int64_t i = k + 1; i < n; ++i) {
        T t = 0;
        for (int64_t j = 0; j < k; ++j) t += EL(a, i, j) * temp[j];
        EL(a, i, k) -= t;
      }
    }
    const T akk = EL(a, k, k);
    const int valid = fabs((double)akk) > 0;
    if (k == 0 && !valid) { /* LDLT.h:371-382: the diagonal is entirely zero */
      *sign = 2;
      for (int64_t j = 0; j < n; ++j) {
        transp[j] = (int)j;
        for (int64_t i = j + 1; i < n; ++i) if (EL(a, i, j) != 0) ret = 0;
      }
      free(temp);
      return ret;
    }
    if (valid) {
      for (int64_t i = k + 1; i < n; ++i) EL(a, i, k) /= akk;
    } else {
      for (int64_t i = k + 1; i < n; ++i) if (EL(a, i, k) != 0) ret = 0;
    }
    if (found_zero && valid) ret = 0;
    else if (!valid) found_zero = 1;
    if (*sign == 0) { if (akk < 0) *sign = 3; }
    else if (*sign == 1) { if (akk > 0) *sign = 3; }
    else if (*sign == 2) { if (akk > 0) *sign = 0; else if (akk < 0) *sign = 1; }
  }
  free(temp);
  return ret;
}

/* x = A^{-1} b from the LDL^T factor (LDLT::_solve_impl_transposed, LDLT.h:573-613): P b, L^{-1},
 * the pseudo-inverse of D (|d| > the smallest normal number, else 0), L^{-T}, P^T. */
void P(ldlt_solve)(char uplo, int64_t n, int64_t nrhs, const T* a, int64_t lda, const int* transp, T* b, int64_t ldb) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int64_t rs = up ? lda : 1, cs = up ? 1 : lda;
  const T tiny = sizeof(T) == 8 ? (T)2.2250738585072014e-308 : (T)1.17549435e-38f;
  for (int64_t c = 0; c < nrhs; ++c) {
    T* x = b + c * ldb;
    for (int64_t k = 0; k < n; ++k) { const int64_t p = transp[k]; const T t = x[k]; x[k] = x[p]; x[p] = t; }
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = j + 1; i < n; ++i) x[i] -= EL(a, i, j) * x[j];
    for (int64_t i = 0; i < n; ++i) {
      const T d = EL(a, i, i);
      x[i] = fabs((double)d) > (double)tiny ? x[i] / d : (T)0;
    }
    for (int64_t j = n - 1; j >= 0; --j) {
      T s = x[j];
      for (int64_t i = j + 1; i < n; ++i) s -= EL(a, i, j) * x[i];
      x[j] = s;
    }
    for (int64_t k = n - 1; k >= 0; --k) { const int64_t p = transp[k]; const T t = x[k]; x[k] = x[p]; x[p] = t; }
  }
}

/* C = alpha op(A) op(A)^T + beta C on the `uplo` triangle (Eigen's BLAS syrk,
 * blas/level3_impl.h:355-417): beta first (0 clears, 1 leaves), then the product times alpha. */
void P(syrk)(char uplo, char op, int64_t n, int64_t k, T alpha, const T* a, int64_t lda, T beta, T* c, int64_t ldc) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int tr = !(op == 'N' || op == 'n');
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = up ? 0 : j; i < (up ? j + 1 : n); ++i) {
      T* cij = c + j * ldc + i;
      if (beta == (T)0) *cij = 0;
      else if (beta != (T)1) *cij *= beta;
    }
  if (n == 0 || k == 0) return;
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = up ? 0 : j; i < (up ? j + 1 : n); ++i) {
      T s = 0;
      for (int64_t p = 0; p < k; ++p) {
        const T x = tr ? a[i * lda + p] : a[p * lda + i];
        const T y = tr ? a[j * lda + p] : a[p * lda + j];
        s += x * y;
      }
      c[j * ldc + i] += alpha * s;
    }
}

/* B = alpha op(A)^{-1} B (side 'L') or alpha B op(A)^{-1} (side 'R') (Eigen's BLAS trsm,
 * blas/level3_impl.h:78-160): substitution, then the scaling by alpha. */
void P(trsm)(char side, char uplo, char op, char diag, int64_t m, int64_t n, T alpha, const T* a, int64_t lda, T* b,
             int64_t ldb) {
  const int left = (side == 'L' || side == 'l');
  const int up = (uplo == 'U' || uplo == 'u');
  const int tr = !(op == 'N' || op == 'n');
  const int unit = (diag == 'U' || diag == 'u');
  if (m == 0 || n == 0) return;
  /* the system matrix S: op(A) (left) or op(A)^T (right, solving for rows of B) */
  const int st = left ? tr : !tr;           /* S(r, q) = st ? A(q, r) : A(r, q) */
  const int slower = (!up) != st;           /* S is lower triangular */
  const int64_t ns = left ? m : n, nv = left ? n : m;
  for (int64_t v = 0; v < nv; ++v) {
    /* the v-th right-hand side: column v of B (left) or row v of B (right) */
    const int64_t inc = left ? 1 : ldb;
    T* x = left ? b + v * ldb : b + v;
    for (int64_t t = 0; t < ns; ++t) {
      const int64_t r = slower ? t : ns - 1 - t;
      const int64_t q0 = slower ? 0 : r + 1, q1 = slower ? r : ns;
      T s = x[r * inc];
      for (int64_t q = q0; q < q1; ++q) s -= (st ? a[r * lda + q] : a[q * lda + r]) * x[q * inc];
      x[r * inc] = unit ? s : s / a[r * lda + r];
    }
  }
  if (alpha != (T)1)
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < m; ++i) b[j * ldb + i] *= alpha;
}

#undef EL
