// Double-float (FP32 pair) arithmetic shared by the FP32 kernels of the
// mixed-precision solve: compensated dot products (TwoProduct by FMA plus
// TwoSum), pair additions and block reductions of pairs.
#pragma once

#include <cuda_runtime.h>

namespace lpm {
namespace {

// s + c += a*b with the rounding errors of the product and of the sum kept
// in c (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26 (2005): TwoProduct by FMA, TwoSum).  The _rn intrinsics keep the
// compiler from contracting the steps into other FMAs.
__device__ __forceinline__ void dot2_acc(float& s, float& c, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float pe = fmaf(a, b, -p);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  const float se = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c = __fadd_rn(c, __fadd_rn(pe, se));
}

// (s, c) += (x, xc) for double-float pairs: TwoSum of the leading parts,
// the rounding error and the trailing parts kept in c.
__device__ __forceinline__ void df_add(float& s, float& c, float x, float xc) {
  const float t = __fadd_rn(s, x);
  const float z = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z));
  s = t;
  c = __fadd_rn(c, __fadd_rn(xc, e));
}

// Double-float vector arithmetic: a value held as an FP32 pair (hi, lo) with
// |lo| at most half an ulp of hi (Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18 (1971)), built from
// TwoSum and TwoProduct by FMA as in dot2_acc.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float z = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}

// (xh, xl) += (ah, al) * (bh, bl), normalised; the product's low-order cross
// terms are kept, the (al, bl) term (below the pair's precision) is not.
__device__ __forceinline__ void df_madd(float& xh, float& xl, float ah, float al, float bh, float bl) {
  const float ph = __fmul_rn(ah, bh);
  const float pl = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -ph)));
  float sh, se;
  two_sum(xh, ph, sh, se);
  two_sum(sh, __fadd_rn(se, __fadd_rn(xl, pl)), xh, xl);
}

// A double rounded to a normalised FP32 pair.
__device__ __forceinline__ void df_split(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// Block sum of per-thread double-float partials, result in thread 0 as
// FP64.  Both the warp and the cross-warp stage stay in FP32 pairs: GB300's
// FP64 pipe takes a whole warp slot even for a one-lane instruction, so an
// FP64 step per warp over a grid of thousands of warps costs microseconds.
// One conversion per block remains.
template <int K>
__device__ __forceinline__ void block_df_sum(float (&s)[K], float (&c)[K], double (&out)[K]) {
  __shared__ float sm[K][2][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const float so = __shfl_xor_sync(0xffffffffu, s[k], o), co = __shfl_xor_sync(0xffffffffu, c[k], o);
      df_add(s[k], c[k], so, co);
    }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      sm[k][0][warp] = s[k];
      sm[k][1][warp] = c[k];
    }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      s[k] = lane < nw ? sm[k][0][lane] : 0.f;
      c[k] = lane < nw ? sm[k][1][lane] : 0.f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const float so = __shfl_xor_sync(0xffffffffu, s[k], o), co = __shfl_xor_sync(0xffffffffu, c[k], o);
        df_add(s[k], c[k], so, co);
      }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < K; ++k) out[k] = (double)s[k] + (double)c[k];
  }
}

}  // namespace
}  // namespace lpm
