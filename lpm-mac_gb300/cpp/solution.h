// Solution (solution.h:12-63 of the reference): closed-form cantilever
// displacement and the relative L2 error of the LPM displacement field.
#pragma once

#include "assembly.h"

template <int nlayer>
class Solution {
 public:
  ExactSolution exact_sol_mode;
  Assembly<nlayer> ass;
  std::vector<std::array<double, NDIM>> position;
  std::vector<double> exact_u, approx_u, error;

  Solution(Assembly<nlayer>& p_ass, const ExactSolution& p_exact_sol) : exact_sol_mode{p_exact_sol}, ass{p_ass} {}

  // Timoshenko cantilever of length L, depth D, tip load P (plane stress)
  void computeSolBeam001(const double& L, const double& D, const double& P, const double& E, const double& mu) {
    const double G = E / 2 / (1 + mu), I = D * D * D / 12;
    for (Particle<nlayer>* pt : ass.pt_sys) {
      const double x = pt->xyz_initial[0], y = pt->xyz_initial[1];
      approx_u.push_back(pt->xyz[0] - x);
      approx_u.push_back(pt->xyz[1] - y);
      // 1 / 6 / G / I is integer division in the reference's expression and so zero
      const double u1 = -P * x * x * y / 2 / E / I + P * y * y * y * (0.0 - mu / 6 / E / I) +
                        y * (P * L * L / 2 / E / I - P * D * D / 8 / G / I);
      const double u2 = mu * P * x * y * y / 2 / E / I + P * x * x * x / 6 / E / I - P * L * L * x / 2 / E / I +
                        P * L * L * L / 3 / E / I;
      exact_u.push_back(u1);
      exact_u.push_back(u2);
    }
  }
  double computeL2Error() {
    double e2 = 0, x2 = 0;
    for (size_t i = 0; i < exact_u.size(); ++i) {
      e2 += pow(exact_u[i] - approx_u[i], 2);
      x2 += pow(exact_u[i], 2);
    }
    if (x2 < EPS) return -1;
    return sqrt(e2 / x2);
  }
};
