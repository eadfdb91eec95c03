// Rigid-body modes of an aggregate of particles, the columns of the
// coarse-space preconditioner's prolongation P (lpm_coarse.cu builds the
// coarse operator, k_mx_persistent applies it).
#pragma once

namespace lpm {

template <int DIM>
constexpr int kModes = DIM == 3 ? 6 : 3;

// Row k (DOF direction) of P for a particle at offset d from its aggregate's
// centroid: translations, then rotations (about z in 2-D; about x, y, z in
// 3-D, omega x d).
template <int DIM, typename T>
__device__ __forceinline__ void mode_row(int k, T dx, T dy, T dz, T (&w)[kModes<DIM>]) {
#pragma unroll
  for (int m = 0; m < kModes<DIM>; ++m) w[m] = T(0);
  w[k] = T(1);
  if (DIM == 2) {
    w[2] = k == 0 ? -dy : dx;
  } else {
    if (k == 0) {
      w[4] = dz;
      w[5] = -dy;
    } else if (k == 1) {
      w[3] = -dz;
      w[5] = dx;
    } else {
      w[3] = dy;
      w[4] = -dx;
    }
  }
}

}  // namespace lpm
