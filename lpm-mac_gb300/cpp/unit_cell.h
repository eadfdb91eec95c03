// UnitCell: per-lattice constants (unit_cell.h:27-127 of the reference).
#pragma once

#include "lpm.h"

class UnitCell {
 public:
  LatticeType lattice;
  int dim;
  int nneighbors, nneighbors1, nneighbors2;
  int nneighbors_AFEM, nneighbors_AFEM1, nneighbors_AFEM2;
  double radius;
  double particle_volume;
  Eigen::MatrixXd el_mapping;  // built from the written data read column by column, as Eigen::Map does
  std::vector<double> neighbor_cutoff;

  UnitCell(LatticeType p_lattice, double p_radius) : lattice(p_lattice), radius(p_radius) {
    switch (lattice) {
      case LatticeType::Square2D: {
        const double d[] = {1. / 2., -1. / 2., 0., 0., 0., 1. / 2., 0., 1. / 12., -1. / 12.};
        set(d, 2, 8, 4, 4, 16, 12, 12, 2.0, 2.0 * sqrt(2.0), 4 * pow(radius, 2));
        break;
      }
      case LatticeType::Hexagon2D: {
        const double d[] = {sqrt(3.0) / 12.0, -sqrt(3.0) / 12.0, 0., -sqrt(3.0) / 144.0, sqrt(3.0) / 48.0, 0.0,
                            0.0, 0.0, 1.0};
        set(d, 2, 12, 6, 6, 30, 18, 18, 2.0, 2.0 * sqrt(3.0), 2 * sqrt(3) * pow(radius, 2));
        break;
      }
      case LatticeType::SimpleCubic3D: {
        const double d[] = {1, -1, -1.0, 0.0, 0.0, 1., 0.0, 1 / 18.0, -1 / 18.0};
        set(d, 3, 18, 6, 12, 60, 24, 54, 2.0, 2.0 * sqrt(2.0), pow(2 * radius, 3));
        break;
      }
      case LatticeType::FCC3D: {
        const double d[] = {0.0, 0.0, sqrt(2.0), sqrt(2.0) / 4, -sqrt(2.0) / 4, -sqrt(2.0) / 4, 0.0,
                            sqrt(2.0) / 24, -sqrt(2.0) / 24};
        set(d, 3, 18, 12, 6, 60, 54, 24, 2.0, 2.0 * sqrt(2.0), 4.0 * sqrt(2.0) * pow(radius, 3));
        break;
      }
      default: {  // the three BCC variants share one cell
        const double d[] = {0.0, 0.0, sqrt(3.0), 1 / sqrt(3.0), -1 / sqrt(3.0), 0., 0.0, sqrt(3.0) / 14,
                            sqrt(3.0) / 14};
        set(d, 3, 14, 8, 6, 40, 34, 24, 2.0, 4.0 / sqrt(3.0), 32.0 * sqrt(3.0) / 9.0 * pow(radius, 3));
      }
    }
  }

 private:
  void set(const double* data, int d, int nn, int nn1, int nn2, int af, int af1, int af2, double c0, double c1,
           double vol) {
    el_mapping = Eigen::Map<const Eigen::MatrixXd>(data, NDIM, NDIM);
    dim = d;
    nneighbors = nn;
    nneighbors1 = nn1;
    nneighbors2 = nn2;
    nneighbors_AFEM = af;
    nneighbors_AFEM1 = af1;
    nneighbors_AFEM2 = af2;
    neighbor_cutoff = {c0 * radius, c1 * radius};
    particle_volume = vol;
  }
};
