// Minimal stand-in for the part of Eigen 3.4 that the LPM reference headers use.
//
// TEST INFRASTRUCTURE ONLY: this header exists so that the reference's own
// header-only C++ sources compile unmodified in an image without Eigen.  It is
// written from Eigen's documented behaviour, not from Eigen's sources, and it
// implements only what the reference calls:
//
//   MatrixXd / VectorXd / VectorXi::Constant / Map<const MatrixXd>
//     (unit_cell.h:49, particle_elastic.h:76-93, utilities.h:8-303,
//      solver.h:25-26,62-63,125-127)
//   SparseMatrix<double>: resize, reserve, insert, makeCompressed, setZero,
//     diagonal, coeffRef, outerSize (stiffness.h:24-25,234-262,269-293)
//   ConjugateGradient<SparseMatrix<double>, Lower|Upper> with the default
//     DiagonalPreconditioner: compute, solve, info, iterations, error
//     (solver.h:195-216)
//
// Documented semantics that the numbers depend on:
//   * storage is column-major; Map<const MatrixXd>(data, r, c) reads data
//     column by column;
//   * ConjugateGradient: zero initial guess for solve(); stop when
//     |r|^2 < max(tol^2 |b|^2, DBL_MIN); default tol = machine epsilon,
//     default max iterations = 2 * cols; info() = Success iff the final
//     relative residual <= tol; the Jacobi preconditioner is 1/A(j,j) where the
//     diagonal entry is stored and non-zero, else 1;
//   * with UpLo = Lower|Upper on a column-major matrix, Eigen applies the
//     stored matrix through its transposed (row-major) view, i.e. the operator
//     is A^T; the shim does the same.
//
// Knob (no reference patch needed): the environment variable
// LPM_ORACLE_CG_TOL, when set, replaces the default CG tolerance, and
// LPM_ORACLE_CG_MAXIT the default iteration cap.  Every solve is appended to a
// log (iterations, error) that the oracle driver dumps.
#pragma once

#include <algorithm>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <iostream>
#include <limits>
#include <utility>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;

enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };
enum UpLoType { Lower = 0x1, Upper = 0x2 };

class VectorXd;
class MatrixXd;

class VectorXd {
 public:
  std::vector<double> v;

  VectorXd() {}
  explicit VectorXd(Index n) : v((size_t)n, 0.0) {}
  // Eigen's VectorXd(int) constructor is explicit in spirit; int sizes go here.
  explicit VectorXd(int n) : v((size_t)n, 0.0) {}
  explicit VectorXd(size_t n) : v(n, 0.0) {}

  Index size() const { return (Index)v.size(); }
  Index rows() const { return (Index)v.size(); }
  Index cols() const { return 1; }
  void resize(Index n) {
    if ((Index)v.size() != n) v.assign((size_t)n, 0.0);
  }
  void setZero() { std::fill(v.begin(), v.end(), 0.0); }
  double& operator()(Index i) { return v[(size_t)i]; }
  double operator()(Index i) const { return v[(size_t)i]; }
  double& operator[](Index i) { return v[(size_t)i]; }
  double operator[](Index i) const { return v[(size_t)i]; }
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }

  double squaredNorm() const {
    double s = 0.0;
    for (double x : v) s += x * x;
    return s;
  }
  double norm() const { return std::sqrt(squaredNorm()); }
  double dot(const VectorXd& o) const {
    double s = 0.0;
    for (size_t i = 0; i < v.size(); ++i) s += v[i] * o.v[i];
    return s;
  }

  // comma initialiser: Ce << a, b, c;
  struct CommaInit {
    VectorXd* target;
    Index pos;
    CommaInit& operator,(double x) {
      (*target)(pos++) = x;
      return *this;
    }
  };
  CommaInit operator<<(double x) {
    (*this)(0) = x;
    return CommaInit{this, 1};
  }
};

inline std::ostream& operator<<(std::ostream& os, const VectorXd& x) {
  for (Index i = 0; i < x.size(); ++i) os << x(i) << "\n";
  return os;
}

class VectorXi {
 public:
  std::vector<int> v;
  VectorXi() {}
  explicit VectorXi(Index n) : v((size_t)n, 0) {}
  static VectorXi Constant(Index n, int value) {
    VectorXi r(n);
    std::fill(r.v.begin(), r.v.end(), value);
    return r;
  }
  Index size() const { return (Index)v.size(); }
  int operator()(Index i) const { return v[(size_t)i]; }
};

template <typename T>
class Map;

// Dense column-major matrix of doubles.
class MatrixXd {
 public:
  Index nr{0}, nc{0};
  std::vector<double> a;  // a[j * nr + i] = M(i, j)

  MatrixXd() {}
  MatrixXd(Index r, Index c) : nr(r), nc(c), a((size_t)(r * c), 0.0) {}
  MatrixXd(const Map<const MatrixXd>& m);
  MatrixXd& operator=(const Map<const MatrixXd>& m);

  Index rows() const { return nr; }
  Index cols() const { return nc; }
  double& operator()(Index i, Index j) { return a[(size_t)(j * nr + i)]; }
  double operator()(Index i, Index j) const { return a[(size_t)(j * nr + i)]; }
};

template <>
class Map<const MatrixXd> {
 public:
  const double* p;
  Index nr, nc;
  Map(const double* data, Index r, Index c) : p(data), nr(r), nc(c) {}
};

inline MatrixXd::MatrixXd(const Map<const MatrixXd>& m) : nr(m.nr), nc(m.nc), a(m.p, m.p + m.nr * m.nc) {}
inline MatrixXd& MatrixXd::operator=(const Map<const MatrixXd>& m) {
  nr = m.nr;
  nc = m.nc;
  a.assign(m.p, m.p + m.nr * m.nc);
  return *this;
}

// (s * M) kept unevaluated so that (s * M) * x applies s after the product,
// as a scaled matrix-vector product does.
struct ScaledMatrixXd {
  double s;
  const MatrixXd* m;
};
inline ScaledMatrixXd operator*(double s, const MatrixXd& m) { return ScaledMatrixXd{s, &m}; }

inline VectorXd operator*(const MatrixXd& m, const VectorXd& x) {
  VectorXd y(m.nr);
  for (Index i = 0; i < m.nr; ++i) {
    double acc = 0.0;
    for (Index j = 0; j < m.nc; ++j) acc += m(i, j) * x(j);
    y(i) = acc;
  }
  return y;
}
inline VectorXd operator*(const ScaledMatrixXd& sm, const VectorXd& x) {
  VectorXd y = (*sm.m) * x;
  for (Index i = 0; i < y.size(); ++i) y(i) *= sm.s;
  return y;
}

// Sparse matrix, column-major.  Insertion keeps each column sorted by row;
// makeCompressed() packs the columns into CSC arrays.
template <typename Scalar>
class SparseMatrix {
 public:
  Index nr{0}, nc{0};
  std::vector<std::vector<int>> col_rows;
  std::vector<std::vector<Scalar>> col_vals;
  // compressed form (valid after makeCompressed, until the next insertion)
  std::vector<Index> outer;
  std::vector<int> inner;
  std::vector<Scalar> values;
  bool compressed{false};

  SparseMatrix() {}
  SparseMatrix(Index r, Index c) { resize(r, c); }

  void resize(Index r, Index c) {
    nr = r;
    nc = c;
    col_rows.assign((size_t)c, std::vector<int>());
    col_vals.assign((size_t)c, std::vector<Scalar>());
    compressed = false;
  }
  Index rows() const { return nr; }
  Index cols() const { return nc; }
  Index outerSize() const { return nc; }
  Index innerSize() const { return nr; }

  // A per-column capacity hint; capped so that an over-generous estimate
  // cannot exhaust memory.
  void reserve(const VectorXi& per_col) {
    for (Index j = 0; j < nc && j < per_col.size(); ++j) {
      size_t want = (size_t)std::max(0, std::min(per_col(j), 256));
      col_rows[(size_t)j].reserve(want);
      col_vals[(size_t)j].reserve(want);
    }
  }

  void setZero() {
    for (auto& c : col_rows) c.clear();
    for (auto& c : col_vals) c.clear();
    compressed = false;
  }

  // New element (must not exist yet), value zero.
  Scalar& insert(Index r, Index c) {
    auto& rows_ = col_rows[(size_t)c];
    auto& vals_ = col_vals[(size_t)c];
    compressed = false;
    if (rows_.empty() || rows_.back() < r) {
      rows_.push_back((int)r);
      vals_.push_back(Scalar(0));
      return vals_.back();
    }
    auto it = std::lower_bound(rows_.begin(), rows_.end(), (int)r);
    assert(it == rows_.end() || *it != r);
    size_t k = (size_t)(it - rows_.begin());
    rows_.insert(it, (int)r);
    vals_.insert(vals_.begin() + (std::ptrdiff_t)k, Scalar(0));
    return vals_[k];
  }

  // Existing element, or a newly inserted zero.
  Scalar& coeffRef(Index r, Index c) {
    auto& rows_ = col_rows[(size_t)c];
    auto it = std::lower_bound(rows_.begin(), rows_.end(), (int)r);
    if (it != rows_.end() && *it == r) return col_vals[(size_t)c][(size_t)(it - rows_.begin())];
    return insert(r, c);
  }

  Scalar coeff(Index r, Index c) const {
    const auto& rows_ = col_rows[(size_t)c];
    auto it = std::lower_bound(rows_.begin(), rows_.end(), (int)r);
    if (it != rows_.end() && *it == r) return col_vals[(size_t)c][(size_t)(it - rows_.begin())];
    return Scalar(0);
  }

  void makeCompressed() {
    outer.assign((size_t)nc + 1, 0);
    size_t nnz = 0;
    for (Index j = 0; j < nc; ++j) nnz += col_rows[(size_t)j].size();
    inner.resize(nnz);
    values.resize(nnz);
    size_t k = 0;
    for (Index j = 0; j < nc; ++j) {
      outer[(size_t)j] = (Index)k;
      const auto& rows_ = col_rows[(size_t)j];
      const auto& vals_ = col_vals[(size_t)j];
      for (size_t t = 0; t < rows_.size(); ++t, ++k) {
        inner[k] = rows_[t];
        values[k] = vals_[t];
      }
    }
    outer[(size_t)nc] = (Index)k;
    compressed = true;
  }

  Index nonZeros() const {
    Index s = 0;
    for (const auto& c : col_rows) s += (Index)c.size();
    return s;
  }

  VectorXd diagonal() const {
    Index n = std::min(nr, nc);
    VectorXd d(n);
    for (Index j = 0; j < n; ++j) d(j) = coeff(j, j);
    return d;
  }
};

// Per-solve log kept by the shim (read by the oracle driver).
struct ShimCgRecord {
  long iterations;
  double error;
  int info;
};
inline std::vector<ShimCgRecord>& shim_cg_log() {
  static std::vector<ShimCgRecord> log;
  return log;
}

inline double shim_env_double(const char* name, double dflt) {
  const char* s = std::getenv(name);
  if (!s || !*s) return dflt;
  return std::strtod(s, nullptr);
}

template <typename MatrixType, int UpLo>
class ConjugateGradient {
 public:
  ConjugateGradient()
      : tol_(shim_env_double("LPM_ORACLE_CG_TOL", std::numeric_limits<double>::epsilon())),
        maxit_((long)shim_env_double("LPM_ORACLE_CG_MAXIT", -1.0)) {}

  void setTolerance(double t) { tol_ = t; }
  void setMaxIterations(long m) { maxit_ = m; }
  double tolerance() const { return tol_; }

  ConjugateGradient& compute(const MatrixType& A) {
    mat_ = &A;
    if (!A.compressed) const_cast<MatrixType&>(A).makeCompressed();
    Index n = A.cols();
    invdiag_.assign((size_t)n, 1.0);
    for (Index j = 0; j < n; ++j) {
      for (Index k = A.outer[(size_t)j]; k < A.outer[(size_t)j + 1]; ++k) {
        if (A.inner[(size_t)k] == j) {
          if (A.values[(size_t)k] != 0.0) invdiag_[(size_t)j] = 1.0 / A.values[(size_t)k];
          break;
        }
      }
    }
    info_ = Success;
    return *this;
  }

  ComputationInfo info() const { return info_; }
  long iterations() const { return iters_; }
  double error() const { return err_; }

  VectorXd solve(const VectorXd& b) {
    const MatrixType& A = *mat_;
    const Index n = A.cols();
    const long maxIters = maxit_ < 0 ? 2 * (long)n : maxit_;
    VectorXd x(n);
    // operator: y = A^T p  (column j of A gives entry j of y)
    auto apply = [&](const std::vector<double>& p, std::vector<double>& y) {
      for (Index j = 0; j < n; ++j) {
        double acc = 0.0;
        for (Index k = A.outer[(size_t)j]; k < A.outer[(size_t)j + 1]; ++k)
          acc += A.values[(size_t)k] * p[(size_t)A.inner[(size_t)k]];
        y[(size_t)j] = acc;
      }
    };
    std::vector<double> r(b.v), p((size_t)n), z((size_t)n), tmp((size_t)n);
    double rhsNorm2 = 0.0;
    for (double t : b.v) rhsNorm2 += t * t;
    if (rhsNorm2 == 0.0) {
      iters_ = 0;
      err_ = 0.0;
      info_ = Success;
      shim_cg_log().push_back({iters_, err_, (int)info_});
      return x;
    }
    const double considerAsZero = std::numeric_limits<double>::min();
    const double threshold = std::max(tol_ * tol_ * rhsNorm2, considerAsZero);
    double residualNorm2 = rhsNorm2;
    if (residualNorm2 < threshold) {
      iters_ = 0;
      err_ = std::sqrt(residualNorm2 / rhsNorm2);
      info_ = err_ <= tol_ ? Success : NoConvergence;
      shim_cg_log().push_back({iters_, err_, (int)info_});
      return x;
    }
    for (Index i = 0; i < n; ++i) p[(size_t)i] = invdiag_[(size_t)i] * r[(size_t)i];
    double absNew = 0.0;
    for (Index i = 0; i < n; ++i) absNew += r[(size_t)i] * p[(size_t)i];
    long it = 0;
    while (it < maxIters) {
      apply(p, tmp);
      double pAp = 0.0;
      for (Index i = 0; i < n; ++i) pAp += p[(size_t)i] * tmp[(size_t)i];
      double alpha = absNew / pAp;
      for (Index i = 0; i < n; ++i) {
        x.v[(size_t)i] += alpha * p[(size_t)i];
        r[(size_t)i] -= alpha * tmp[(size_t)i];
      }
      residualNorm2 = 0.0;
      for (Index i = 0; i < n; ++i) residualNorm2 += r[(size_t)i] * r[(size_t)i];
      if (residualNorm2 < threshold) break;
      for (Index i = 0; i < n; ++i) z[(size_t)i] = invdiag_[(size_t)i] * r[(size_t)i];
      double absOld = absNew;
      absNew = 0.0;
      for (Index i = 0; i < n; ++i) absNew += r[(size_t)i] * z[(size_t)i];
      double beta = absNew / absOld;
      for (Index i = 0; i < n; ++i) p[(size_t)i] = z[(size_t)i] + beta * p[(size_t)i];
      ++it;
    }
    iters_ = it;
    err_ = std::sqrt(residualNorm2 / rhsNorm2);
    info_ = err_ <= tol_ ? Success : NoConvergence;
    shim_cg_log().push_back({iters_, err_, (int)info_});
    return x;
  }

 private:
  const MatrixType* mat_{nullptr};
  std::vector<double> invdiag_;
  double tol_;
  long maxit_;
  long iters_{0};
  double err_{0.0};
  ComputationInfo info_{Success};
};

}  // namespace Eigen
