// Device helpers: deterministic block and grid reductions.
//
// Every sum the solvers use is folded in a fixed order (warp shuffles in a
// fixed tree, then block partials in block order), so a run gives the same
// bits every time for a given grid size.  The grid fold uses the
// last-block-done pattern: blocks publish their partials, take an atomic
// ticket, and the block that draws the last ticket folds all partials.  No
// block ever waits on another.
#pragma once

#include "lpm_internal.cuh"

namespace lpm {

template <int K>
__device__ __forceinline__ void warp_sum(double (&v)[K]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
}

// Sum over the block; the result is valid in thread 0.  blockDim.x must be a
// multiple of 32 and at most 1024.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K]) {
  __shared__ double sm[K][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  warp_sum<K>(v);
  __syncthreads();  // sm may still be read by a previous call
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sm[k][warp] = v[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = lane < nw ? sm[k][lane] : 0.0;
    warp_sum<K>(v);
  }
}

// Grid-wide sum.  Returns true in the one block that finishes last; there,
// after the call, tot[k] holds the totals in every thread.  partials needs
// K * gridDim.x doubles, ticket one zeroed counter (reset here for the next
// launch).  gridDim.x <= kMaxRedBlocks.
template <int K>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double* partials, unsigned int* ticket, double (&tot)[K]) {
  __shared__ bool last;
  __shared__ double res[K];
  block_sum<K>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] += __ldcg(&partials[k * gridDim.x + b]);
  block_sum<K>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) res[k] = acc[k];
    *ticket = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) tot[k] = res[k];
  return true;
}

// Grid-wide sum of values already reduced per block (valid in thread 0 of
// each block): the last-block fold of grid_sum without its block reduction.
template <int K>
__device__ __forceinline__ bool grid_fold(const double (&v)[K], double* partials, unsigned int* ticket,
                                          double (&tot)[K]) {
  __shared__ bool last;
  __shared__ double res[K];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] += __ldcg(&partials[k * gridDim.x + b]);
  block_sum<K>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) res[k] = acc[k];
    *ticket = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) tot[k] = res[k];
  return true;
}

__device__ __forceinline__ bool is_broken(double bdamage) { return fabs(bdamage - 1.0) < EPS; }

// Particle::distanceTo (particle.h:277-280): sqrt(dx^2 + dy^2 + dz^2) with each
// square rounded and the sum taken left to right, no fused multiply-add, so
// the length is the reference's bit for bit (sqrt and the products are
// correctly rounded on both sides).
__device__ __forceinline__ double bond_length(double dx, double dy, double dz) {
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

}  // namespace lpm
