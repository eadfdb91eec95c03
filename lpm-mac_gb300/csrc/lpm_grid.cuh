// Grid barriers for kernels whose blocks are all resident (cooperative
// launches): the persistent CG solves (lpm_cg.cu) and the coarse inverse
// (lpm_coarse.cu).
#pragma once

#include "lpm_device.cuh"

namespace lpm {

// Polls before a grid-barrier wait gives up: at least 32 ns apart, so more
// than half a second, against microseconds for a barrier that completes.
constexpr long long kPcgSpinLimit = 1LL << 24;

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* a) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
  return v;
}

// Grid barrier on a monotone arrival count: the k-th barrier of a launch
// waits until k * gridDim.x arrivals.  The fence before the arrival and the
// acquire loads and fence after the wait order every block's writes before
// the barrier ahead of every read after it.  The wait is bounded; returns
// false in every thread of the block if it gave up.
__device__ __forceinline__ bool grid_barrier(unsigned long long* gbar, unsigned long long target, long long limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(gbar, 1ULL);
    int good = 1;
    long long polls = 0;
    while (ld_acquire_u64(gbar) < target) {
      if (++polls > limit) {
        good = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Grid totals of K values per block (valid in thread 0): published in slots
// slot..slot+K-1 of the partials, then, after the barrier, folded by warp 0
// of every block in block order and returned in every thread.
template <int K>
__device__ __forceinline__ bool grid_allreduce(const double (&v)[K], double* partials, int slot,
                                               unsigned long long* gbar, unsigned long long& target, long long limit,
                                               double (&tot)[K]) {
  __shared__ double res[K];
  const int G = gridDim.x;
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) partials[(int64_t)(slot + k) * G + blockIdx.x] = v[k];
  target += (unsigned long long)G;
  if (!grid_barrier(gbar, target, limit)) return false;
  if (threadIdx.x < 32) {
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < G; b += 32)
#pragma unroll
      for (int k = 0; k < K; ++k) acc[k] += __ldcg(&partials[(int64_t)(slot + k) * G + b]);
    warp_sum<K>(acc);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < K; ++k) res[k] = acc[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) tot[k] = res[k];
  return true;
}

}  // namespace lpm
