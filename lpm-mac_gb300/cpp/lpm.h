// LPM class API on the GB300 path: base definitions.
//
// Same names and values as the reference's lpm.h (lpm.h:36-96): macros,
// func_phi, and the mode enums, so that an example's run() compiles against
// these headers unchanged.  The hot methods of the classes forward to
// liblpmgpu (include/lpm_gpu.h).
#pragma once

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdio>
#include <deque>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <map>
#include <queue>
#include <string>
#include <vector>

#if __has_include(<omp.h>)
#include <omp.h>
#else
#include <chrono>
inline double omp_get_wtime() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
inline int omp_get_max_threads() { return 1; }
#endif

#include "lpm_dense.h"
#include "lpm_gpu.h"

#define PI 3.14159265358979323846
#define EPS 1e-6
#define NDIM 3

// nonlocal weight (lpm.h:45-49)
inline double func_phi(const double x, const double L) {
  double p = 8, q = 2;
  return pow(1 / (1 + pow(x / L, p)), q);
}

enum class ExactSolution : char { Beam001 };
enum class LoadMode : char { Relative, Absolute };
enum class SolverMode : char { CG };
enum class StiffnessMode : char { Analytical, FiniteDifference };
enum class TimeMapMode : char { Linear, Exponential };
enum class ParticleType : char { Elastic, ElasticDamage, J2Plasticity, FatigueHCF };
enum class LatticeType : char { Square2D, Hexagon2D, SimpleCubic3D, FCC3D, BCC3D_1Slip, BCC3D_2Slip, BCC3D_3Slip };

// Run-time choices of the GPU path that have no counterpart in the
// reference's interface.  Defaults reproduce the reference; environment
// variables override them (LPM_TANGENT=symmetric, LPM_PRECISION=mixed,
// LPM_CG_TOL=1e-10, LPM_STATIC_BC=eliminate; LPM_PRECOND=coarse or
// coarse:<box edge> for the coarse-space preconditioner of the mixed solve).
struct LpmGpuOptions {
  int tangent = LPM_TANGENT_AS_WRITTEN;
  int precision = LPM_PREC_FP64;
  double cg_tol = 2.220446049250313e-16;  // Eigen's default: machine epsilon
  int static_bc = LPM_BC_NONE;            // SolverStatic leaves the BC elimination out
  bool verbose = true;                    // the reference's printf lines
  int precond = LPM_PRECOND_JACOBI;       // Eigen's DiagonalPreconditioner
  double precond_box = 0.0;               // coarse box edge (0: automatic)
};
inline LpmGpuOptions& lpm_gpu_options() {
  static LpmGpuOptions o = [] {
    LpmGpuOptions v;
    if (const char* s = getenv("LPM_TANGENT")) v.tangent = strcmp(s, "symmetric") == 0 ? LPM_TANGENT_SYMMETRIC
                                                                                      : LPM_TANGENT_AS_WRITTEN;
    if (const char* s = getenv("LPM_PRECISION")) v.precision = strcmp(s, "mixed") == 0 ? LPM_PREC_MIXED : LPM_PREC_FP64;
    if (const char* s = getenv("LPM_CG_TOL")) v.cg_tol = atof(s);
    if (const char* s = getenv("LPM_STATIC_BC")) v.static_bc = strcmp(s, "eliminate") == 0 ? LPM_BC_ELIMINATE
                                                                                          : LPM_BC_NONE;
    if (const char* s = getenv("LPM_QUIET")) v.verbose = atoi(s) == 0;
    if (const char* s = getenv("LPM_PRECOND")) {
      if (strncmp(s, "coarse", 6) == 0) {
        v.precond = LPM_PRECOND_COARSE;
        if (s[6] == ':') v.precond_box = atof(s + 7);
      }
    }
    return v;
  }();
  return o;
}

inline void lpm_check(int st, const char* what) {
  if (st < 0) {
    fprintf(stderr, "liblpmgpu: %s failed (%d): %s\n", what, st, lpm_last_error(nullptr));
    exit(1);
  }
}
