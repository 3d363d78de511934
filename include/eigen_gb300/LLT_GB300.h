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
// What stays on Eigen's CPU code: LLT::solveInPlace (LLT.h:514-522) calls the triangular views
// directly and bypasses Solve<>; the L1 norm that LLT::compute keeps for rcond
// (LLT.h:443-453; gbllt_?lansy_l1_dev is its device form for callers outside Eigen).
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

// Runs the GPU solve of `dec` against `rhs` into the column-major temporary `x`.
template <typename DecType, typename RhsType, typename Scalar>
void gb300_solve(const DecType& dec, const RhsType& rhs, Matrix<Scalar, Dynamic, Dynamic, ColMajor>& x) {
  typedef typename DecType::MatrixType FactorType;
  x = rhs;
  const auto& f = dec.matrixLLT();
  gb300_llt<Scalar>::potrs(f.data(), (int64_t)f.outerStride(), (FactorType::Flags & RowMajorBit) != 0,
                           DecType::UpLo == Lower ? 1 : 0, (int64_t)x.rows(), (int64_t)x.cols(), x.data());
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
      Matrix<EIGTYPE, Dynamic, Dynamic, ColMajor> x;                                                   \
      gb300_solve(src.dec(), src.rhs(), x);                                                            \
      dst = x;                                                                                         \
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
      Matrix<EIGTYPE, Dynamic, Dynamic, ColMajor> x;                                                   \
      gb300_solve(solve.dec(), solve.rhs(), x);                                                        \
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

}  // namespace internal
}  // namespace Eigen

#endif  // EIGEN_LLT_GB300_H
