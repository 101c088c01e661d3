/*
 * Minimal stand-in for the part of the Eigen API that the reference's
 * operate_dielectric.{h,cxx} and LinearOperator.h use, so that those files
 * compile unmodified into the oracle library (Eigen is not installed here).
 *
 * TEST INFRASTRUCTURE ONLY: this header is used to build oracle/_ref (the
 * reference's own sources compiled as a checker). It is never linked into
 * the product library.
 *
 * What it provides:
 *   - VectorXd (dense double column vector), Map/Triplet/SparseMatrix types
 *   - EigenBase / MatrixBase / Product / internal::traits /
 *     internal::generic_product_impl hooks so that the reference's
 *     MatrixReplacement specialisation (LinearOperator.h:61-85) is the code
 *     that applies the operator,
 *   - BiCGSTAB<MatrixType, Preconditioner> restating Eigen 3.3/3.4's published
 *     algorithm (van der Vorst 1992 with Eigen's restart and stopping rules):
 *       r = b - A x0; r0 = r; stop when |r|^2 <= tol^2 |b|^2 (recursively
 *       updated r) or iterations == maxit; if |rho| < eps^2 |r0|^2 the
 *       residual is recomputed, r0 := r and (on the first restart only) the
 *       iteration counter is reset; x = 0 is returned when |b| == 0.
 *       error() = |r|/|b| of the updated residual.
 *     solve(b) starts from a zero guess; solveWithGuess(b, x0) from x0.
 *   - IdentityPreconditioner and DiagonalPreconditioner (Jacobi; used only by
 *     the never-selected finite-difference variant in the reference).
 */
#ifndef ICEP_ORACLE_EIGEN_SHIM_H
#define ICEP_ORACLE_EIGEN_SHIM_H

#include <cmath>
#include <cstddef>
#include <vector>
#include <limits>
#include <algorithm>

#ifndef EIGEN_ONLY_USED_FOR_DEBUG
#define EIGEN_ONLY_USED_FOR_DEBUG(x) (void)(x)
#endif

namespace Eigen {

typedef std::ptrdiff_t Index;
const int Dynamic = -1;

enum {
  DefaultProduct = 0,
  LazyProduct,
  AliasFreeProduct,
  CoeffBasedProductMode,
  LazyCoeffBasedProductMode,
  OuterProduct,
  InnerProduct,
  GemvProduct,
  GemmProduct
};

template <typename Derived>
struct EigenBase {
  typedef Eigen::Index Index;
  Derived &derived() { return *static_cast<Derived *>(this); }
  const Derived &derived() const { return *static_cast<const Derived *>(this); }
};

template <typename Derived>
struct MatrixBase : public EigenBase<Derived> {};

template <typename Scalar_, int Rows_, int Cols_>
class Matrix : public MatrixBase<Matrix<Scalar_, Rows_, Cols_> > {
 public:
  typedef Scalar_ Scalar;
  typedef Scalar_ RealScalar;
  Matrix() {}
  explicit Matrix(Index n) : v_(static_cast<size_t>(n)) {}
  static Matrix Zero(Index n) {
    Matrix m(n);
    std::fill(m.v_.begin(), m.v_.end(), Scalar(0));
    return m;
  }
  Index size() const { return static_cast<Index>(v_.size()); }
  Index rows() const { return size(); }
  Index cols() const { return 1; }
  Scalar &operator[](Index i) { return v_[static_cast<size_t>(i)]; }
  const Scalar &operator[](Index i) const { return v_[static_cast<size_t>(i)]; }
  Scalar &operator()(Index i) { return v_[static_cast<size_t>(i)]; }
  const Scalar &operator()(Index i) const { return v_[static_cast<size_t>(i)]; }
  Scalar *data() { return v_.data(); }
  const Scalar *data() const { return v_.data(); }
  void setZero() { std::fill(v_.begin(), v_.end(), Scalar(0)); }
  void resize(Index n) { v_.resize(static_cast<size_t>(n)); }

 private:
  std::vector<Scalar> v_;
};

typedef Matrix<double, Dynamic, 1> VectorXd;

template <typename PlainObjectType, int MapOptions = 0, typename StrideType = void>
class Map;

template <typename Scalar_>
class Triplet {
 public:
  Triplet(Index r, Index c, Scalar_ v) : r_(r), c_(c), v_(v) {}
  Index row() const { return r_; }
  Index col() const { return c_; }
  Scalar_ value() const { return v_; }

 private:
  Index r_, c_;
  Scalar_ v_;
};

template <typename Scalar_, int Options_ = 0, typename StorageIndex_ = int>
class SparseMatrix : public EigenBase<SparseMatrix<Scalar_, Options_, StorageIndex_> > {
 public:
  typedef Scalar_ Scalar;
  SparseMatrix() : n_(0), m_(0) {}
  SparseMatrix(Index rows, Index cols) : n_(rows), m_(cols) {}
  Index rows() const { return n_; }
  Index cols() const { return m_; }
  template <typename It>
  void setFromTriplets(It begin, It end) {
    r_.clear(); c_.clear(); v_.clear();
    for (It it = begin; it != end; ++it) {
      r_.push_back(it->row()); c_.push_back(it->col()); v_.push_back(it->value());
    }
  }
  /* y = A x (duplicate triplets are summed, as Eigen's setFromTriplets does). */
  void apply(const Scalar *x, Scalar *y) const {
    for (Index i = 0; i < n_; i++) y[i] = 0;
    for (size_t t = 0; t < v_.size(); t++) y[r_[t]] += v_[t] * x[c_[t]];
  }
  Scalar diag(Index i) const {
    Scalar d = 0;
    for (size_t t = 0; t < v_.size(); t++)
      if (r_[t] == i && c_[t] == i) d += v_[t];
    return d;
  }
  Matrix<Scalar, Dynamic, 1> operator*(const Matrix<Scalar, Dynamic, 1> &x) const {
    Matrix<Scalar, Dynamic, 1> y(n_);
    apply(x.data(), y.data());
    return y;
  }

 private:
  Index n_, m_;
  std::vector<Index> r_, c_;
  std::vector<Scalar> v_;
};

template <typename Lhs, typename Rhs, int Option = DefaultProduct>
class Product {
 public:
  typedef double Scalar;
  Product(const Lhs &l, const Rhs &r) : lhs_(l), rhs_(r) {}
  const Lhs &lhs() const { return lhs_; }
  const Rhs &rhs() const { return rhs_; }

 private:
  const Lhs &lhs_;
  const Rhs &rhs_;
};

namespace internal {
template <typename T>
struct traits;
template <typename Scalar_, int O_, typename I_>
struct traits<SparseMatrix<Scalar_, O_, I_> > {
  typedef Scalar_ Scalar;
};
struct SparseShape {};
struct DenseShape {};
template <typename Lhs, typename Rhs, typename LhsShape = SparseShape,
          typename RhsShape = DenseShape, int ProductType = GemvProduct>
struct generic_product_impl;
template <typename Lhs, typename Rhs, typename Derived>
struct generic_product_impl_base {};

/* y = A x for a matrix-free operator: routed through the user's
 * generic_product_impl<...,GemvProduct>::scaleAndAddTo, the hook Eigen uses. */
template <typename MatrixType>
struct apply_op {
  static void run(const MatrixType &A, const VectorXd &x, VectorXd &y) {
    y.setZero();
    generic_product_impl<MatrixType, VectorXd, SparseShape, DenseShape, GemvProduct>::scaleAndAddTo(
        y, A, x, 1.0);
  }
};
template <typename S, int O, typename I>
struct apply_op<SparseMatrix<S, O, I> > {
  static void run(const SparseMatrix<S, O, I> &A, const VectorXd &x, VectorXd &y) {
    A.apply(x.data(), y.data());
  }
};

inline double dot(const VectorXd &a, const VectorXd &b) {
  double s = 0.0;
  for (Index i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}
}  // namespace internal

/* Statistics of the most recent solve (read by the oracle harness). */
namespace shim_stats {
inline long &iterations() { static long v = 0; return v; }
inline double &error() { static double v = 0; return v; }
inline long &matvecs() { static long v = 0; return v; }
}  // namespace shim_stats

class IdentityPreconditioner {
 public:
  template <typename M>
  void compute(const M &) {}
  void solve(const VectorXd &in, VectorXd &out) const { out = in; }
};

template <typename Scalar_>
class DiagonalPreconditioner {
 public:
  template <typename M>
  void compute(const M &A) {
    inv_.resize(A.rows());
    for (Index i = 0; i < A.rows(); i++) {
      Scalar_ d = A.diag(i);
      inv_[i] = (d == Scalar_(0)) ? Scalar_(1) : Scalar_(1) / d;
    }
  }
  void solve(const VectorXd &in, VectorXd &out) const {
    out.resize(in.size());
    for (Index i = 0; i < in.size(); i++) out[i] = inv_[i] * in[i];
  }

 private:
  VectorXd inv_;
};

template <typename MatrixType_, typename Preconditioner_ = DiagonalPreconditioner<double> >
class BiCGSTAB {
 public:
  BiCGSTAB() : A_(nullptr), tol_(std::numeric_limits<double>::epsilon()), maxit_(-1), iters_(0), err_(0) {}
  explicit BiCGSTAB(const MatrixType_ &A) : BiCGSTAB() { compute(A); }
  BiCGSTAB &compute(const MatrixType_ &A) {
    A_ = &A;
    pre_.compute(A);
    return *this;
  }
  BiCGSTAB &setTolerance(double t) { tol_ = t; return *this; }
  BiCGSTAB &setMaxIterations(Index m) { maxit_ = m; return *this; }
  Index iterations() const { return iters_; }
  double error() const { return err_; }
  Index maxIterations() const { return (maxit_ < 0) ? 2 * A_->cols() : maxit_; }

  VectorXd solveWithGuess(const VectorXd &b, const VectorXd &x0) {
    VectorXd x = x0;
    run(b, x);
    return x;
  }
  VectorXd solve(const VectorXd &b) {
    VectorXd x = VectorXd::Zero(b.size());
    run(b, x);
    return x;
  }

 private:
  void matvec(const VectorXd &x, VectorXd &y) const {
    ++shim_stats::matvecs();
    internal::apply_op<MatrixType_>::run(*A_, x, y);
  }

  void run(const VectorXd &b, VectorXd &x) {
    using internal::dot;
    const Index n = b.size();
    const double tol = tol_;
    const Index maxIters = maxIterations();
    VectorXd r(n), tmp(n);
    matvec(x, tmp);
    for (Index i = 0; i < n; i++) r[i] = b[i] - tmp[i];
    VectorXd r0 = r;
    double r0_sqnorm = dot(r0, r0);
    double rhs_sqnorm = dot(b, b);
    if (rhs_sqnorm == 0) {
      x.setZero();
      iters_ = 0;
      err_ = 0;
      shim_stats::iterations() = 0;
      shim_stats::error() = 0;
      return;
    }
    double rho = 1, alpha = 1, w = 1;
    VectorXd v = VectorXd::Zero(n), p = VectorXd::Zero(n);
    VectorXd y(n), z(n), s(n), t(n);
    const double tol2 = tol * tol * rhs_sqnorm;
    const double eps = std::numeric_limits<double>::epsilon();
    const double eps2 = eps * eps;
    Index i = 0, restarts = 0;
    while (dot(r, r) > tol2 && i < maxIters) {
      double rho_old = rho;
      rho = dot(r0, r);
      if (std::fabs(rho) < eps2 * r0_sqnorm) {
        matvec(x, tmp);
        for (Index k = 0; k < n; k++) r[k] = b[k] - tmp[k];
        r0 = r;
        rho = r0_sqnorm = dot(r, r);
        if (restarts++ == 0) i = 0;
      }
      double beta = (rho / rho_old) * (alpha / w);
      for (Index k = 0; k < n; k++) p[k] = r[k] + beta * (p[k] - w * v[k]);
      pre_.solve(p, y);
      matvec(y, v);
      alpha = rho / dot(r0, v);
      for (Index k = 0; k < n; k++) s[k] = r[k] - alpha * v[k];
      pre_.solve(s, z);
      matvec(z, t);
      double tt = dot(t, t);
      if (tt > 0.0)
        w = dot(t, s) / tt;
      else
        w = 0.0;
      for (Index k = 0; k < n; k++) x[k] += alpha * y[k] + w * z[k];
      for (Index k = 0; k < n; k++) r[k] = s[k] - w * t[k];
      ++i;
    }
    err_ = std::sqrt(dot(r, r) / rhs_sqnorm);
    iters_ = i;
    shim_stats::iterations() = i;
    shim_stats::error() = err_;
  }

  const MatrixType_ *A_;
  Preconditioner_ pre_;
  double tol_;
  Index maxit_;
  Index iters_;
  double err_;
};

}  // namespace Eigen

#endif
