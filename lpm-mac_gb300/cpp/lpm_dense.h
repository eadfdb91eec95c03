// Dense 3x3-sized matrices and vectors for the set-up API of the LPM class
// mirror (UnitCell::el_mapping, createRMatrix, the lattice generators).
// When Eigen is on the include path it is used; otherwise this header
// provides the small subset of Eigen's interface those call sites need, in
// namespace Eigen so that example code written against the reference
// compiles unchanged.
#pragma once

#if __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
#else
#include <cmath>
#include <cstddef>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;

class VectorXd {
 public:
  std::vector<double> v;
  VectorXd() {}
  explicit VectorXd(Index n) : v((size_t)n, 0.0) {}
  explicit VectorXd(int n) : v((size_t)n, 0.0) {}
  Index size() const { return (Index)v.size(); }
  void resize(Index n) {
    if ((Index)v.size() != n) v.assign((size_t)n, 0.0);
  }
  double& operator()(Index i) { return v[(size_t)i]; }
  double operator()(Index i) const { return v[(size_t)i]; }
  double& operator[](Index i) { return v[(size_t)i]; }
  double operator[](Index i) const { return v[(size_t)i]; }
  double* data() { return v.data(); }
  double squaredNorm() const {
    double s = 0;
    for (double x : v) s += x * x;
    return s;
  }
  double norm() const { return std::sqrt(squaredNorm()); }
  struct Comma {
    VectorXd* t;
    Index k;
    Comma& operator,(double x) {
      (*t)(k++) = x;
      return *this;
    }
  };
  Comma operator<<(double x) {
    (*this)(0) = x;
    return Comma{this, 1};
  }
};

class MatrixXd;
template <typename T>
class Map;
template <>
class Map<const MatrixXd> {
 public:
  const double* p;
  Index r, c;
  Map(const double* d, Index rows, Index cols) : p(d), r(rows), c(cols) {}
};

// column-major, as Eigen's default storage
class MatrixXd {
 public:
  Index nr{0}, nc{0};
  std::vector<double> a;
  MatrixXd() {}
  MatrixXd(Index r, Index c) : nr(r), nc(c), a((size_t)(r * c), 0.0) {}
  MatrixXd(const Map<const MatrixXd>& m) : nr(m.r), nc(m.c), a(m.p, m.p + m.r * m.c) {}
  MatrixXd& operator=(const Map<const MatrixXd>& m) {
    nr = m.r;
    nc = m.c;
    a.assign(m.p, m.p + m.r * m.c);
    return *this;
  }
  Index rows() const { return nr; }
  Index cols() const { return nc; }
  double& operator()(Index i, Index j) { return a[(size_t)(j * nr + i)]; }
  double operator()(Index i, Index j) const { return a[(size_t)(j * nr + i)]; }
};

struct ScaledMatrixXd {
  double s;
  const MatrixXd* m;
};
inline ScaledMatrixXd operator*(double s, const MatrixXd& m) { return ScaledMatrixXd{s, &m}; }
inline VectorXd operator*(const MatrixXd& m, const VectorXd& x) {
  VectorXd y(m.nr);
  for (Index i = 0; i < m.nr; ++i) {
    double acc = 0;
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

}  // namespace Eigen
#endif
