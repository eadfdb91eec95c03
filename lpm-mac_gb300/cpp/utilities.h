// Lattice generators and the rotation matrix (utilities.h:8-300 of the
// reference).  Each generator lays out an oversized lattice around the
// origin (half-width = the box diagonal), rotates every point by R and keeps
// the points inside the box, in generation order.  The start points and
// pitches of each lattice are the reference's, including its quirks (the
// square plate is offset by one radius; the simple cubic rows start at
// box[0] rather than at the oversized box's edge), so that the same boxes
// give the same particles.
#pragma once

#include "unit_cell.h"

// Euler-angle rotation, row major: 0 = X1-Y2-Z3, 1 = Z1-Y2-Z3 (Kocks),
// 2 = Z1-X2-Z3 (Bunge)
inline Eigen::MatrixXd createRMatrix(int eulerflag, double angles[]) {
  const double c1 = cos(angles[0]), s1 = sin(angles[0]), c2 = cos(angles[1]), s2 = sin(angles[1]),
               c3 = cos(angles[2]), s3 = sin(angles[2]);
  double r[9] = {0};
  if (eulerflag == 0) {
    const double m[9] = {c2 * c3, -c2 * s3, s2, c1 * s3 + s1 * s2 * c3, c1 * c3 - s1 * s2 * s3, -s1 * c2,
                         s1 * s3 - c1 * s2 * c3, s1 * c3 + c1 * s2 * s3, c1 * c2};
    std::copy(m, m + 9, r);
  } else if (eulerflag == 1) {
    const double m[9] = {-c1 * c2 * c3 - s1 * s3, c3 * s1 - s3 * c2 * c1, s2 * c1, s3 * c1 - c3 * c2 * s1,
                         -c1 * c3 - s1 * c2 * s3, s2 * s1, c3 * s2, s3 * s2, c2};
    std::copy(m, m + 9, r);
  } else if (eulerflag == 2) {
    const double m[9] = {-s1 * c2 * s3 + c1 * c3, -s3 * c1 - c3 * c2 * s1, s1 * s2, c3 * s1 + s3 * c2 * c1,
                         -s1 * s3 + c1 * c2 * c3, -c1 * s2, s2 * s3, s2 * c3, c2};
    std::copy(m, m + 9, r);
  }
  Eigen::MatrixXd R(NDIM, NDIM);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R(i, j) = r[3 * i + j];
  return R;
}

namespace lpm_detail {
// rotate each candidate and keep those inside the box (2D tests x, y only)
inline std::vector<std::array<double, NDIM>> rotateAndClip(const std::vector<std::array<double, NDIM>>& pts,
                                                          const std::array<double, 2 * NDIM>& box,
                                                          const Eigen::MatrixXd& R, int dim, bool zero_z) {
  std::vector<std::array<double, NDIM>> out;
  Eigen::VectorXd p(NDIM), q(NDIM);
  for (const std::array<double, NDIM>& x : pts) {
    p(0) = x[0], p(1) = x[1], p(2) = x[2];
    q = R * p;
    bool in = q(0) >= box[0] && q(0) <= box[1] && q(1) >= box[2] && q(1) <= box[3];
    if (dim == 3) in = in && q(2) >= box[4] && q(2) <= box[5];
    if (in) out.push_back({q(0), q(1), zero_z ? 0.0 : q(2)});
  }
  return out;
}
inline double halfWidth(const std::array<double, 2 * NDIM>& box, int dim) {
  double s = pow(box[1] - box[0], 2) + pow(box[3] - box[2], 2);
  if (dim == 3) s += pow(box[5] - box[4], 2);
  return sqrt(s);
}
}  // namespace lpm_detail

inline std::vector<std::array<double, NDIM>> createPlateSQ2D(std::array<double, 2 * NDIM> box, UnitCell cell,
                                                              Eigen::MatrixXd R_matrix) {
  const double a = lpm_detail::halfWidth(box, 2), h = 2 * cell.radius;
  const int ncol = (int)floor(2 * a / h), nrow = ncol;
  std::vector<std::array<double, NDIM>> pts;
  for (int j = 0; j < nrow; ++j)
    for (int i = 0; i < ncol; ++i) pts.push_back({-a + h * i + cell.radius, -a + h * j + cell.radius, 0.0});
  return lpm_detail::rotateAndClip(pts, box, R_matrix, 2, true);
}

inline std::vector<std::array<double, NDIM>> createPlateHEX2D(std::array<double, 2 * NDIM> box, UnitCell cell,
                                                               Eigen::MatrixXd R_matrix) {
  const double a = lpm_detail::halfWidth(box, 2), hx = 2 * cell.radius, hy = hx * sqrt(3.0) / 2.0;
  const int ncol = 1 + (int)floor(2 * a / hx), nrow = 1 + (int)floor(2 * a / hy);
  std::vector<std::array<double, NDIM>> pts;
  for (int j = 0; j < nrow; ++j) {
    const double y = -a + hy * j;
    if (j % 2 == 0)
      for (int i = 0; i < ncol; ++i) pts.push_back({-a + hx * i, y, 0.0});
    else
      for (int i = 1; i < ncol; ++i) pts.push_back({-a + hx * (2 * i - 1) / 2.0, y, 0.0});
  }
  return lpm_detail::rotateAndClip(pts, box, R_matrix, 2, false);
}

inline std::vector<std::array<double, NDIM>> createCuboidSC3D(std::array<double, 2 * NDIM> box, UnitCell cell,
                                                               Eigen::MatrixXd R_matrix) {
  const double a = lpm_detail::halfWidth(box, 3), h = 2 * cell.radius;
  const int n = 1 + (int)floor(2 * a / h);
  std::vector<std::array<double, NDIM>> pts;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) pts.push_back({box[0] + h * i, -a + h * j, -a + h * k});
  return lpm_detail::rotateAndClip(pts, box, R_matrix, 3, false);
}

inline std::vector<std::array<double, NDIM>> createCuboidFCC3D(std::array<double, 2 * NDIM> box, UnitCell cell,
                                                                Eigen::MatrixXd R_matrix) {
  const double a = lpm_detail::halfWidth(box, 3), h = 4 * cell.radius / sqrt(2.0);
  const int ncol = 1 + (int)floor(2 * a / h), nrow = 1 + (int)floor(2 * a / (h / 2.0)), nlay = nrow;
  std::vector<std::array<double, NDIM>> pts;
  for (int k = 0; k < nlay; ++k)
    for (int j = 0; j < nrow; ++j) {
      // full rows where the row and layer parities agree, shifted rows otherwise
      const bool full = (j % 2) == (k % 2);
      const double y = -a + h / 2.0 * j, z = -a + h / 2.0 * k;
      for (int i = 0; i < (full ? ncol : ncol - 1); ++i) pts.push_back({-a + h * i + (full ? 0.0 : h / 2.0), y, z});
    }
  return lpm_detail::rotateAndClip(pts, box, R_matrix, 3, false);
}
