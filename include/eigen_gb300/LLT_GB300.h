// LLT_GB300.h -- Eigen backend that runs LLT<MatrixXd> / LLT<MatrixXf> on a GB300 GPU.
//
// Selected by a preprocessor macro, like Eigen's LAPACKE backend (Eigen/Cholesky:34-41 includes
// Eigen/src/Cholesky/LLT_LAPACKE.h under EIGEN_USE_LAPACKE).  Existing code picks it up unchanged
// when compiled with
//
//     -DEIGEN_USE_GB300 -include eigen_gb300/LLT_GB300.h      (and linked with -lgbllt)
//
// What is routed to the GPU (through the C ABI of gbllt.h):
//   - the factorisation: full specialisations of internal::llt_inplace<T, Lower|Upper> for
//     T = double, float, whose blocked() calls gbllt_?potrf -- the same boundary and the same
//     info mapping (0 -> -1, i > 0 -> i - 1) as LLT_LAPACKE.h:42-93.  Their rankUpdate (which
//     LLT_LAPACKE.h:71-73 leaves to llt_rank_update_lower on the CPU) calls gbllt_?rank_update, the
//     same algorithm (LLT.h:238-307) on the GPU;
//   - the solve: partial specialisations of internal::Assignment<Dst, Solve<LLT<...>, Rhs>, ...>
//     (dst = llt.solve(b), Solve.h:137-149) and internal::evaluator<Solve<LLT<...>, Rhs>>
//     (dst += / -= / noalias, Solve.h:114-131) call gbllt_?potrs on the current host factor
//     (matrixLLT()), so a modified factor changes the result as Eigen's own solve does.
//   - the condition estimate: explicit specialisations of internal::rcond_estimate_helper for the
//     dynamic-size LLTs (called by LLT::rcond, LLT.h:166-171) call gbllt_?pocon, which runs
//     Eigen's estimator (ConditionEstimator.h:56-171) with the factor resident on the device.
//   - LDLT<MatrixXd|MatrixXf> (and LDLT<Ref<...>>): the pivoted factorisation, through explicit
//     specialisations of internal::ldlt_inplace<Lower>::unblocked (LDLT.h:297-403) that call
//     gbllt_?ldlt; ldlt.solve(b) through Solve<LDLT<...>> specialisations calling gbllt_?ldlt_solve.
//   - triangular solves with a dynamic number of right-hand sides, triangularView<Mode>()
//     .solveInPlace(B) and .solve(B) (SolveTriangular.h:49-104): partial specialisations of
//     internal::triangular_solve_matrix for double and float, the hook that
//     TriangularSolverMatrix_BLAS.h:41-161 uses for ?trsm_, call gbllt_?trsm; and
//     internal::triangular_solve_vector for a single right-hand-side vector.  LLT::solveInPlace
//     (LLT.h:514-522), which calls the two triangular views directly, therefore runs on the GPU too.
// What stays on Eigen's CPU code: the L1 norm that LLT::compute keeps for rcond
// (LLT.h:443-453; gbllt_?lansy_l1_dev is its device form for callers outside Eigen); fixed-size
// LDLTs; LDLT::rankUpdate (ldlt_inplace::update, LDLT.h:405-456); LDLT::rcond, whose estimator
// (ConditionEstimator.h) runs its solves through the GPU solve above; triangular solves of complex
// scalars, of right-hand sides with an inner stride, and of fixed-size vectors of at most 8
// entries (SolveTriangular.h's compile-time unrolled path).
//
// Errors: a failing library call (no usable GPU, CUDA error) trips eigen_assert; with assertions
// disabled the factorisation reports NumericalIssue and a solve leaves NaN in its result.
#ifndef EIGEN_LLT_GB300_H
#define EIGEN_LLT_GB300_H

#ifdef EIGEN_USE_LAPACKE
#error "EIGEN_USE_GB300 and EIGEN_USE_LAPACKE both specialise llt_inplace<double|float>; define only one"
#endif
#ifndef EIGEN_USE_GB300
#define EIGEN_USE_GB300
#endif

#include <Eigen/Cholesky>
#include <cstdio>
#include <limits>

#include "gbllt.h"  // found through -I <repo>/include

namespace Eigen {
namespace internal {

inline bool gb300_check(const char* fn, int rc) {
  if (rc == GBLLT_SUCCESS) return true;
  std::fprintf(stderr, "%s failed with %d: %s\n", fn, rc, gbllt_last_error());
  eigen_assert(false && "gbllt call failed");
  return false;
}

template <typename Scalar>
struct gb300_llt;

#define EIGEN_GB300_LLT(EIGTYPE, POTRF, POTRS, RANKUPD)                                                 \
  template <>                                                                                          \
  struct gb300_llt<EIGTYPE> {                                                                          \
    template <typename MatrixType>                                                                     \
    static Index potrf(MatrixType& m, char uplo) {                                                     \
      eigen_assert(m.rows() == m.cols());                                                              \
      const int64_t n = (int64_t)m.rows();                                                             \
      if (n == 0) return -1;                                                                           \
      const int layout = (MatrixType::Flags & RowMajorBit) ? GBLLT_ROW_MAJOR : GBLLT_COL_MAJOR;       \
      int64_t info = 0;                                                                                \
      const int rc = POTRF(layout, uplo, n, &m.coeffRef(0, 0), (int64_t)m.outerStride(), &info);       \
      if (!gb300_check(#POTRF, rc)) return 0;                                                          \
      return info == 0 ? -1 : (Index)(info - 1);                                                       \
    }                                                                                                  \
    /* Solves in place in the column-major n x k array x (leading dimension n) from the factor */      \
    /* `fac` stored in the UpLo triangle of a matrix with the given storage order. */                 \
    static void potrs(const EIGTYPE* fac, int64_t ldf, bool rowmajor, int uplo_lower, int64_t n,       \
                      int64_t k, EIGTYPE* x) {                                                         \
      if (n == 0 || k == 0) return;                                                                    \
      /* a row-major lower factor is a column-major upper one (and vice versa) */                      \
      const char uplo = ((uplo_lower != 0) != rowmajor) ? 'L' : 'U';                                   \
      const int rc = POTRS(GBLLT_COL_MAJOR, uplo, n, k, fac, ldf, x, n);                               \
      if (!gb300_check(#POTRS, rc))                                                                    \
        for (int64_t i = 0; i < n * k; ++i) x[i] = std::numeric_limits<EIGTYPE>::quiet_NaN();          \
    }                                                                                                  \
    /* llt_rank_update_lower (LLT.h:238-307) on the `uplo` triangle: -1 or the failing column */     \
    template <typename MatrixType, typename VectorType>                                                \
    static Index rank_update(MatrixType& m, const VectorType& vec, EIGTYPE sigma, char uplo) {         \
      eigen_assert(m.rows() == m.cols() && vec.size() == m.rows());                                   \
      const int64_t n = (int64_t)m.rows();                                                             \
      if (n == 0) return -1;                                                                           \
      const int layout = (MatrixType::Flags & RowMajorBit) ? GBLLT_ROW_MAJOR : GBLLT_COL_MAJOR;       \
      const Matrix<EIGTYPE, Dynamic, 1> v = vec;                                                       \
      int64_t info = 0;                                                                                \
      const int rc = RANKUPD(layout, uplo, n, &m.coeffRef(0, 0), (int64_t)m.outerStride(), v.data(),   \
                             sigma, &info);                                                            \
      if (!gb300_check(#RANKUPD, rc)) return 0;                                                        \
      return info == 0 ? -1 : (Index)(info - 1);                                                       \
    }                                                                                                  \
  };                                                                                                   \
  template <>                                                                                          \
  struct llt_inplace<EIGTYPE, Lower> {                                                                 \
    template <typename MatrixType>                                                                     \
    static Index blocked(MatrixType& m) {                                                              \
      return gb300_llt<EIGTYPE>::potrf(m, 'L');                                                        \
    }                                                                                                  \
    template <typename MatrixType, typename VectorType>                                                \
    static Index rankUpdate(MatrixType& mat, const VectorType& vec,                                    \
                            const typename MatrixType::RealScalar& sigma) {                            \
      return gb300_llt<EIGTYPE>::rank_update(mat, vec, sigma, 'L');                                    \
    }                                                                                                  \
  };                                                                                                   \
  template <>                                                                                          \
  struct llt_inplace<EIGTYPE, Upper> {                                                                 \
    template <typename MatrixType>                                                                     \
    static Index blocked(MatrixType& m) {                                                              \
      return gb300_llt<EIGTYPE>::potrf(m, 'U');                                                        \
    }                                                                                                  \
    template <typename MatrixType, typename VectorType>                                                \
    static Index rankUpdate(MatrixType& mat, const VectorType& vec,                                    \
                            const typename MatrixType::RealScalar& sigma) {                            \
      return gb300_llt<EIGTYPE>::rank_update(mat, vec, sigma, 'U');                                    \
    }                                                                                                  \
  };

EIGEN_GB300_LLT(double, gbllt_dpotrf, gbllt_dpotrs, gbllt_drank_update)
EIGEN_GB300_LLT(float, gbllt_spotrf, gbllt_spotrs, gbllt_srank_update)

#undef EIGEN_GB300_LLT

// The GPU solve of an LLT in place in the column-major n x k array x (leading dimension n).
template <typename MatrixType, int UpLo, typename Scalar>
void gb300_run_solve(const LLT<MatrixType, UpLo>& dec, int64_t n, int64_t k, Scalar* x) {
  const auto& f = dec.matrixLLT();
  gb300_llt<Scalar>::potrs(f.data(), (int64_t)f.outerStride(), (MatrixType::Flags & RowMajorBit) != 0,
                           UpLo == Lower ? 1 : 0, n, k, x);
}

template <typename Scalar>
struct gb300_ldlt;
template <typename MatrixType, int UpLo, typename Scalar>
void gb300_run_solve(const LDLT<MatrixType, UpLo>& dec, int64_t n, int64_t k, Scalar* x);

// dst = dec.solve(rhs).  A plain column-major destination is solved in its own storage (no
// temporary, so `x = dec.solve(x)` allocates nothing, as Eigen's in-place solve does); any other
// destination goes through a column-major temporary.
template <typename DecType, typename RhsType, typename Scalar, int Rows, int Cols, int MaxRows, int MaxCols>
void gb300_solve_assign(const DecType& dec, const RhsType& rhs, Matrix<Scalar, Rows, Cols, ColMajor, MaxRows, MaxCols>& dst) {
  dst = rhs;  // no-op when rhs is dst itself
  gb300_run_solve(dec, (int64_t)dst.rows(), (int64_t)dst.cols(), dst.data());
}
template <typename DecType, typename RhsType, typename DstType>
void gb300_solve_assign(const DecType& dec, const RhsType& rhs, DstType& dst) {
  Matrix<typename DstType::Scalar, Dynamic, Dynamic, ColMajor> x = rhs;
  gb300_run_solve(dec, (int64_t)x.rows(), (int64_t)x.cols(), x.data());
  dst = x;
}

#define EIGEN_GB300_SOLVE(EIGTYPE)                                                                     \
  /* dst = llt.solve(rhs) */                                                                           \
  template <typename DstXprType, int Options, int MaxRows, int MaxCols, int UpLo, typename RhsType>    \
  struct Assignment<DstXprType,                                                                        \
                    Solve<LLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType>, \
                    assign_op<EIGTYPE, EIGTYPE>, Dense2Dense> {                                        \
    typedef Solve<LLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType> SrcXprType; \
    static void run(DstXprType& dst, const SrcXprType& src, const assign_op<EIGTYPE, EIGTYPE>&) {      \
      if ((dst.rows() != src.rows()) || (dst.cols() != src.cols())) dst.resize(src.rows(), src.cols()); \
      gb300_solve_assign(src.dec(), src.rhs(), dst);                                                   \
    }                                                                                                  \
  };                                                                                                   \
  /* llt.solve(rhs) used inside a larger expression (+=, -=, noalias): evaluated into a temporary */  \
  template <int Options, int MaxRows, int MaxCols, int UpLo, typename RhsType>                         \
  struct evaluator<Solve<LLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType> > \
      : public evaluator<typename Solve<LLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, \
                                        RhsType>::PlainObject> {                                       \
    typedef Solve<LLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType> SolveType; \
    typedef typename SolveType::PlainObject PlainObject;                                               \
    typedef evaluator<PlainObject> Base;                                                               \
    enum { Flags = Base::Flags | EvalBeforeNestingBit };                                               \
    explicit evaluator(const SolveType& solve) : m_result(solve.rows(), solve.cols()) {                \
      ::new (static_cast<Base*>(this)) Base(m_result);                                                 \
      Matrix<EIGTYPE, Dynamic, Dynamic, ColMajor> x = solve.rhs();                                     \
      gb300_run_solve(solve.dec(), (int64_t)x.rows(), (int64_t)x.cols(), x.data());                   \
      m_result = x;                                                                                    \
    }                                                                                                  \
                                                                                                       \
   protected:                                                                                          \
    PlainObject m_result;                                                                              \
  };

EIGEN_GB300_SOLVE(double)
EIGEN_GB300_SOLVE(float)

#undef EIGEN_GB300_SOLVE

// llt.rcond(): LLT::rcond (LLT.h:166-171) returns rcond_estimate_helper(m_l1_norm, *this)
// (ConditionEstimator.h:161-171), whose estimator runs up to 11 solves.  These explicit
// specialisations for the dynamic-size double/float LLTs hand the whole estimate to gbllt_?pocon,
// which copies the factor to the device once and runs the same algorithm there.
#define EIGEN_GB300_RCOND(EIGTYPE, POCON, OPT, UPLO)                                                    \
  template <>                                                                                          \
  inline EIGTYPE rcond_estimate_helper<LLT<Matrix<EIGTYPE, Dynamic, Dynamic, OPT>, UPLO> >(             \
      EIGTYPE matrix_norm, const LLT<Matrix<EIGTYPE, Dynamic, Dynamic, OPT>, UPLO>& dec) {              \
    eigen_assert(dec.rows() == dec.cols());                                                            \
    const int64_t n = (int64_t)dec.rows();                                                             \
    const auto& f = dec.matrixLLT();                                                                   \
    const int layout = (OPT & RowMajor) ? GBLLT_ROW_MAJOR : GBLLT_COL_MAJOR;                          \
    EIGTYPE r = 0;                                                                                     \
    const int rc = POCON(layout, UPLO == Lower ? 'L' : 'U', n, n ? f.data() : nullptr,                 \
                         n ? (int64_t)f.outerStride() : 1, matrix_norm, &r);                            \
    if (!gb300_check(#POCON, rc)) return std::numeric_limits<EIGTYPE>::quiet_NaN();                   \
    return r;                                                                                          \
  }

EIGEN_GB300_RCOND(double, gbllt_dpocon, ColMajor, Lower)
EIGEN_GB300_RCOND(double, gbllt_dpocon, ColMajor, Upper)
EIGEN_GB300_RCOND(double, gbllt_dpocon, RowMajor, Lower)
EIGEN_GB300_RCOND(double, gbllt_dpocon, RowMajor, Upper)
EIGEN_GB300_RCOND(float, gbllt_spocon, ColMajor, Lower)
EIGEN_GB300_RCOND(float, gbllt_spocon, ColMajor, Upper)
EIGEN_GB300_RCOND(float, gbllt_spocon, RowMajor, Lower)
EIGEN_GB300_RCOND(float, gbllt_spocon, RowMajor, Upper)

#undef EIGEN_GB300_RCOND

// ---- LDLT ---------------------------------------------------------------------------------------
// LDLT::compute (LDLT.h:497-530) calls ldlt_inplace<UpLo>::unblocked; Upper passes a Transpose<> of
// its matrix to ldlt_inplace<Lower> (LDLT.h:460-466).  These explicit specialisations of that member
// template for the dynamic-size double/float matrices (plain and Ref<>, either storage order, and
// their transposes) call gbllt_?ldlt, which returns Eigen's transpositions, sign and success flag.
#define EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN, MTYPE, LAYOUT, UPLO, BASE)                               \
  template <>                                                                                          \
  inline bool ldlt_inplace<Lower>::unblocked<MTYPE, Transpositions<Dynamic, Dynamic, int>,              \
                                             Matrix<EIGTYPE, Dynamic, 1> >(                            \
      MTYPE & mat, Transpositions<Dynamic, Dynamic, int> & transpositions, Matrix<EIGTYPE, Dynamic, 1> & temp, \
      SignMatrix & sign) {                                                                             \
    EIGEN_UNUSED_VARIABLE(temp);                                                                       \
    eigen_assert(mat.rows() == mat.cols());                                                            \
    const int64_t n = (int64_t)mat.rows();                                                             \
    if (n == 0) {                                                                                      \
      sign = ZeroSign;                                                                                 \
      return true;                                                                                     \
    }                                                                                                  \
    int32_t sg = 2;                                                                                    \
    int64_t info = 0;                                                                                  \
    const int rc = LDLTFN(LAYOUT, UPLO, n, &mat.coeffRef(0, 0), (int64_t)BASE.outerStride(),           \
                          transpositions.indices().data(), &sg, &info);                                \
    if (!gb300_check(#LDLTFN, rc)) return false;                                                       \
    sign = static_cast<SignMatrix>(sg);                                                                \
    return info == 0;                                                                                  \
  }

#define EIGEN_GB300_LDLT_TYPES(EIGTYPE, LDLTFN)                                                          \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN, Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA ColMajor>, \
                          GBLLT_COL_MAJOR, 'L', mat)                                                   \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN, Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA RowMajor>, \
                          GBLLT_ROW_MAJOR, 'L', mat)                                                   \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN,                                                             \
                          Transpose<Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA ColMajor> >, \
                          GBLLT_COL_MAJOR, 'U', mat.nestedExpression())                                \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN,                                                             \
                          Transpose<Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA RowMajor> >, \
                          GBLLT_ROW_MAJOR, 'U', mat.nestedExpression())                                \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN,                                                             \
                          Ref<Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA ColMajor> >, \
                          GBLLT_COL_MAJOR, 'L', mat)                                                   \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN,                                                             \
                          Ref<Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA RowMajor> >, \
                          GBLLT_ROW_MAJOR, 'L', mat)                                                   \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN,                                                             \
                          Transpose<Ref<Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA ColMajor> > >, \
                          GBLLT_COL_MAJOR, 'U', mat.nestedExpression())                                \
  EIGEN_GB300_LDLT_FACTOR(EIGTYPE, LDLTFN,                                                             \
                          Transpose<Ref<Matrix<EIGTYPE EIGEN_COMMA Dynamic EIGEN_COMMA Dynamic EIGEN_COMMA RowMajor> > >, \
                          GBLLT_ROW_MAJOR, 'U', mat.nestedExpression())

EIGEN_GB300_LDLT_TYPES(double, gbllt_dldlt)
EIGEN_GB300_LDLT_TYPES(float, gbllt_sldlt)

#undef EIGEN_GB300_LDLT_TYPES
#undef EIGEN_GB300_LDLT_FACTOR

#define EIGEN_GB300_LDLT_SOLVER(EIGTYPE, SOLVEFN)                                                        \
  template <>                                                                                          \
  struct gb300_ldlt<EIGTYPE> {                                                                         \
    static void solve(const EIGTYPE* fac, int64_t ldf, bool rowmajor, int uplo_lower, const int* transp, \
                      int64_t n, int64_t k, EIGTYPE* x) {                                              \
      if (n == 0 || k == 0) return;                                                                    \
      const char uplo = ((uplo_lower != 0) != rowmajor) ? 'L' : 'U';                                   \
      const int rc = SOLVEFN(GBLLT_COL_MAJOR, uplo, n, k, fac, ldf, transp, x, n);                     \
      if (!gb300_check(#SOLVEFN, rc))                                                                  \
        for (int64_t i = 0; i < n * k; ++i) x[i] = std::numeric_limits<EIGTYPE>::quiet_NaN();          \
    }                                                                                                  \
  };
EIGEN_GB300_LDLT_SOLVER(double, gbllt_dldlt_solve)
EIGEN_GB300_LDLT_SOLVER(float, gbllt_sldlt_solve)
#undef EIGEN_GB300_LDLT_SOLVER

// The GPU solve of an LDLT in place in x (LDLT::_solve_impl_transposed, LDLT.h:573-613: P, L, D^+,
// L^T, P^T).
template <typename MatrixType, int UpLo, typename Scalar>
void gb300_run_solve(const LDLT<MatrixType, UpLo>& dec, int64_t n, int64_t k, Scalar* x) {
  const auto& f = dec.matrixLDLT();
  gb300_ldlt<Scalar>::solve(f.data(), (int64_t)f.outerStride(), (MatrixType::Flags & RowMajorBit) != 0,
                            UpLo == Lower ? 1 : 0, dec.transpositionsP().indices().data(), n, k, x);
}

#define EIGEN_GB300_LDLT_SOLVE(EIGTYPE)                                                                \
  /* dst = ldlt.solve(rhs) */                                                                          \
  template <typename DstXprType, int Options, int MaxRows, int MaxCols, int UpLo, typename RhsType>    \
  struct Assignment<DstXprType,                                                                        \
                    Solve<LDLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType>, \
                    assign_op<EIGTYPE, EIGTYPE>, Dense2Dense> {                                        \
    typedef Solve<LDLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType> SrcXprType; \
    static void run(DstXprType& dst, const SrcXprType& src, const assign_op<EIGTYPE, EIGTYPE>&) {      \
      if ((dst.rows() != src.rows()) || (dst.cols() != src.cols())) dst.resize(src.rows(), src.cols()); \
      gb300_solve_assign(src.dec(), src.rhs(), dst);                                                   \
    }                                                                                                  \
  };                                                                                                   \
  /* ldlt.solve(rhs) inside a larger expression (+=, -=, noalias): evaluated into a temporary */      \
  template <int Options, int MaxRows, int MaxCols, int UpLo, typename RhsType>                         \
  struct evaluator<Solve<LDLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType> > \
      : public evaluator<typename Solve<LDLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, \
                                        RhsType>::PlainObject> {                                       \
    typedef Solve<LDLT<Matrix<EIGTYPE, Dynamic, Dynamic, Options, MaxRows, MaxCols>, UpLo>, RhsType> SolveType; \
    typedef typename SolveType::PlainObject PlainObject;                                               \
    typedef evaluator<PlainObject> Base;                                                               \
    enum { Flags = Base::Flags | EvalBeforeNestingBit };                                               \
    explicit evaluator(const SolveType& solve) : m_result(solve.rows(), solve.cols()) {                \
      ::new (static_cast<Base*>(this)) Base(m_result);                                                 \
      Matrix<EIGTYPE, Dynamic, Dynamic, ColMajor> x = solve.rhs();                                     \
      gb300_run_solve(solve.dec(), (int64_t)x.rows(), (int64_t)x.cols(), x.data());                   \
      m_result = x;                                                                                    \
    }                                                                                                  \
                                                                                                       \
   protected:                                                                                          \
    PlainObject m_result;                                                                              \
  };

EIGEN_GB300_LDLT_SOLVE(double)
EIGEN_GB300_LDLT_SOLVE(float)

#undef EIGEN_GB300_LDLT_SOLVE

// ---- triangular solves --------------------------------------------------------------------------
// SolveTriangular.h:85-104 hands a matrix right-hand side to triangular_solve_matrix<Scalar, Index,
// Side, Mode, Conjugate, TriStorageOrder, OtherStorageOrder, OtherInnerStride>; a row-major right-hand
// side is first turned into the transposed problem on the other side
// (TriangularSolverMatrix.h:17-34), so the column-major cases below see every layout.  As in
// TriangularSolverMatrix_BLAS.h, a row-major triangle is the transpose of a column-major one with
// the other uplo, and Conjugate is immaterial for real scalars.
template <typename Scalar>
struct gb300_trsm;

#define EIGEN_GB300_TRSM(EIGTYPE, TRSM)                                                                    template <>                                                                                            struct gb300_trsm<EIGTYPE> {                                                                             /* B (m x n, column-major, leading dimension ldb) <- op(T)^-1 B (side 'L') or B op(T)^-1 ('R') */      static void run(char side, int mode, bool tri_rowmajor, int64_t m, int64_t n, const EIGTYPE* tri,                       int64_t ldt, EIGTYPE* b, int64_t ldb) {                                                  if (m == 0 || n == 0) return;                                                                          const bool lower = (mode & Lower) == Lower;                                                            const char uplo = (lower != tri_rowmajor) ? 'L' : 'U';                                                 const char trans = tri_rowmajor ? 'T' : 'N';                                                           const char diag = (mode & UnitDiag) ? 'U' : 'N';                                                       const int rc = TRSM(GBLLT_COL_MAJOR, side, uplo, trans, diag, m, n, EIGTYPE(1), tri, ldt, b, ldb);       if (!gb300_check(#TRSM, rc))                                                                             for (int64_t j = 0; j < n; ++j)                                                                          for (int64_t i = 0; i < m; ++i) b[i + j * ldb] = std::numeric_limits<EIGTYPE>::quiet_NaN();      }                                                                                                    };                                                                                                     /* op(T)^-1 B, B column-major with unit inner stride */                                               template <typename Index, int Mode, bool Conjugate, int TriStorageOrder>                               struct triangular_solve_matrix<EIGTYPE, Index, OnTheLeft, Mode, Conjugate, TriStorageOrder, ColMajor, 1> {     static void run(Index size, Index otherSize, const EIGTYPE* tri, Index triStride, EIGTYPE* other,                      Index otherIncr, Index otherStride, level3_blocking<EIGTYPE, EIGTYPE>&) {                EIGEN_ONLY_USED_FOR_DEBUG(otherIncr);                                                                  eigen_assert(otherIncr == 1);                                                                          gb300_trsm<EIGTYPE>::run('L', Mode, TriStorageOrder == RowMajor, (int64_t)size, (int64_t)otherSize,                                tri, (int64_t)triStride, other, (int64_t)otherStride);                      }                                                                                                    };                                                                                                     /* B op(T)^-1 */                                                                                       template <typename Index, int Mode, bool Conjugate, int TriStorageOrder>                               struct triangular_solve_matrix<EIGTYPE, Index, OnTheRight, Mode, Conjugate, TriStorageOrder, ColMajor, 1> {     static void run(Index size, Index otherSize, const EIGTYPE* tri, Index triStride, EIGTYPE* other,                      Index otherIncr, Index otherStride, level3_blocking<EIGTYPE, EIGTYPE>&) {                EIGEN_ONLY_USED_FOR_DEBUG(otherIncr);                                                                  eigen_assert(otherIncr == 1);                                                                          gb300_trsm<EIGTYPE>::run('R', Mode, TriStorageOrder == RowMajor, (int64_t)otherSize, (int64_t)size,                                tri, (int64_t)triStride, other, (int64_t)otherStride);                      }                                                                                                    };                                                                                                     /* one right-hand-side vector (TriangularSolverVector.h:30-142); OnTheRight reduces to these */        template <typename Index, int Mode, bool Conjugate>                                                    struct triangular_solve_vector<EIGTYPE, EIGTYPE, Index, OnTheLeft, Mode, Conjugate, ColMajor> {          static void run(Index size, const EIGTYPE* lhs, Index lhsStride, EIGTYPE* rhs) {                         gb300_trsm<EIGTYPE>::run('L', Mode, false, (int64_t)size, 1, lhs, (int64_t)lhsStride, rhs,                                       (int64_t)(size > 0 ? size : 1));                                            }                                                                                                    };                                                                                                     template <typename Index, int Mode, bool Conjugate>                                                    struct triangular_solve_vector<EIGTYPE, EIGTYPE, Index, OnTheLeft, Mode, Conjugate, RowMajor> {          static void run(Index size, const EIGTYPE* lhs, Index lhsStride, EIGTYPE* rhs) {                         gb300_trsm<EIGTYPE>::run('L', Mode, true, (int64_t)size, 1, lhs, (int64_t)lhsStride, rhs,                                        (int64_t)(size > 0 ? size : 1));                                            }                                                                                                    };

EIGEN_GB300_TRSM(double, gbllt_dtrsm)
EIGEN_GB300_TRSM(float, gbllt_strsm)

#undef EIGEN_GB300_TRSM

}  // namespace internal
}  // namespace Eigen

#endif  // EIGEN_LLT_GB300_H
