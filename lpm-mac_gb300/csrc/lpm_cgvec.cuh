// Vector kernels of the Jacobi-PCG iteration shared by the solvers on the
// assembled operator (lpm_cg.cu) and on the exact Jacobian (lpm_adjoint.cu):
//   k_cg_init     x = 0, r = b, p = M^-1 r, |b|^2, r.z, convergence set-up
//   k_cg_update   x += alpha p, r -= alpha q, |r|^2, r.z; convergence, beta
//   k_cg_pupdate  p = M^-1 r + beta p
// The iteration is Eigen's ConjugateGradient recurrence (zero start, stop
// when |r|^2 < max(tol^2 |b|^2, DBL_MIN)); alpha comes from the product
// kernel of the caller.
#pragma once

#include <cfloat>
#include <cmath>

#include "lpm_device.cuh"

namespace lpm {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_cg_update(int64_t ndof, T* __restrict__ x, T* __restrict__ r,
                                                   const T* __restrict__ p, const T* __restrict__ q,
                                                   const T* __restrict__ invd, CgScalars* cg, double* partials,
                                                   unsigned int* ticket) {
  if (cg->done) return;
  const T alpha = (T)cg->alpha;
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = r[i] - alpha * q[i];
    x[i] = x[i] + alpha * p[i];
    r[i] = ri;
    const T zi = invd[i] * ri;
    v[0] += (double)ri * (double)ri;
    v[1] += (double)ri * (double)zi;
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rr = tot[0];
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      cg->done = 3;
    } else if (tot[0] < cg->threshold) {
      cg->done = 1;
    } else {
      const double old = cg->abs_new;
      cg->abs_new = tot[1];
      cg->beta = tot[1] / old;
      cg->it += 1;
      if (cg->it >= cg->maxit) cg->done = 2;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_cg_pupdate(int64_t ndof, const T* __restrict__ r, const T* __restrict__ invd,
                                                    T* __restrict__ p, CgScalars* cg,
                                                    cudaGraphConditionalHandle loop_cond) {
  // inside a solve graph, the last kernel of an iteration: block 0 sets the
  // loop condition and counts the pass
  if (loop_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    cudaGraphSetConditional(loop_cond, cg->done ? 0u : 1u);
    cg->graph_passes += 1;
  }
  if (cg->done) return;
  const T beta = (T)cg->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = invd[i] * r[i] + beta * p[i];
}

template <typename T>
__global__ void k_cg_init(int64_t ndof, const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                          T* __restrict__ p, const T* __restrict__ invd, CgScalars* cg, double tol, long long maxit,
                          double* partials, unsigned int* ticket) {
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const T bi = b[i];
    const T pi = invd[i] * bi;
    x[i] = T(0);
    r[i] = bi;
    p[i] = pi;
    v[0] += (double)bi * (double)bi;
    v[1] += (double)bi * (double)pi;
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rhs_norm2 = tot[0];
    cg->rr = tot[0];
    cg->threshold = fmax(tol * tol * tot[0], DBL_MIN);
    cg->abs_new = tot[1];
    cg->alpha = 0.0;
    cg->beta = 0.0;
    cg->it = 0;
    cg->maxit = maxit;
    cg->graph_passes = 0;
    cg->pfault = 0;
    if (!isfinite(tot[0]) || !isfinite(tot[1]))
      cg->done = 3;
    else if (tot[0] == 0.0 || tot[0] < cg->threshold)
      cg->done = 1;
    else if (maxit <= 0)
      cg->done = 2;
    else
      cg->done = 0;
  }
}

}  // namespace
}  // namespace lpm
