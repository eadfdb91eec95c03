// Matrix-free application of the analytical tangent (lpm_set_operator with
// LPM_OPERATOR_MATRIX_FREE): the CG runs on A = K^T, the operator that
// Eigen's ConjugateGradient applies to the column-major K of
// Stiffness::calcStiffness (stiffness.h:228-263, derivative.h), without
// assembling it.
//
// Block K_ij of the tangent (i != j, per layer l, bond b = i->j, n = cs_b,
// w = 1 - bdamage, t = w Tv, a = w (2 Kn + Tv), S_i = sum of i's layer-l
// cosines, T_i = sum t n over i's layer-l bonds) is
//   own:   w[(-Kn n[s] + Tv S_j[s]) n[r] - (Kn + Tv) n[r] n[s]] - o[r] n[s],
//          o = (t (S_i - n) + T_i - t n) / 2,
//   paths: -1/2 (t_kj + t_ik) n_ik[r] n_kj[s] over layer-l paths i->k->j.
// Row i of A holds the blocks K_ji^T.  Gathered over i's bonds b = i->j,
// with b' = opp(b) the bond j->i (n' = cs_b', t', a'), and taken in
// difference form, y_i = R_i p_i + sum_{j != i} K_ji^T (p_j - p_i) with R_i
// the block row sum of A, the product is
//   y_i = R_i p_i + sum_b n' [ -(a' - t') s' - (t' U_j.d + V_j.d + t' H_j + F_j) / 2 ]
//                 + sum_l (sum_{b in l} t' s') S_i,
//   d = p_j - p_i, s' = n'.d,  U_j = S_j + sum n'_c, V_j = T_j + sum t'_c n'_c
// (sums over j's layer-l bonds c, with their opposite bonds' values), and
// the first pass's sums  H_j = sum_c n'_c.(p_m - p_j),  F_j = sum_c t'_c n'_c.(p_m - p_j)
// over j's bonds c = j->m.  The paths that return to i and the diagonal
// block enter only R_i (their difference terms vanish).  For intact bonds
// n' = -n and t' = t, so U and V vanish.  This is exact algebra: the
// product equals the assembled A p up to rounding, for both tangent
// variants (they differ only in K_ii, which is inside R_i).
//
// Two passes per product: pass 1 (thread per particle over its slots)
// forms H and F per particle and layer; pass 2 (the same walk) forms y,
// then the epilogue of the CG product (q, p.q, alpha) or of the mixed
// solve's FP64 true residual.  The FP32 passes take the differences in
// FP32 and accumulate with compensated sums (as the assembled FP32
// product), and write q as a double-float pair.  BC elimination
// (stiffness.h:265-294) is A' = P A P + nd (I - P): the input is masked,
// the fixed rows return nd p.
//
// Bytes per FP32 product: pass 1 reads per slot the partner and one 16-byte
// word {n', t'} (20 B), pass 2 the same and a' - t' (24 B); per particle the
// row sums (36 B), S, U, V of both layers (72 B), H and F (16 B), p and
// the pair q (36 B).  At 101^3 that is about 1.0 GB against 2.4 GB for the
// assembled FP32 product.
#include <algorithm>
#include <cmath>
#include <vector>

#include "lpm_device.cuh"
#include "lpm_df.cuh"
#include "lpm_graph.cuh"

namespace lpm {
namespace {

constexpr unsigned kLayerBit = 1u << 31;  // slot word: the bond's layer
constexpr unsigned kUVBit = 1u << 30;     // slot word: the partner's U, V (this layer) are not zero
constexpr unsigned kIdMask = kUVBit - 1;  // slot word: the partner
constexpr int kMfFields = 5;  // per slot: n'x, n'y, n'z, a' - t', t'

// Slot partners: bond k of particle i at mbase[i/32] + 32 k + i%32 in
// stored (layer 0, then layer 1) order; the slice's padding slots point at
// the particle itself and keep zero coefficients.
__global__ void k_mf_slots(int n, const int64_t* __restrict__ bptr, const int* __restrict__ bp2,
                           const int* __restrict__ blayer, const int64_t* __restrict__ mbase,
                           unsigned* __restrict__ mp2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sl = i / 32;
  const int64_t s0 = mbase[sl] + (i % 32);
  const int width = (int)((mbase[sl + 1] - mbase[sl]) / 32);
  int k = 0;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b, ++k)
    mp2[s0 + 32 * k] = (unsigned)bp2[b] | (blayer[b] ? kLayerBit : 0u);
  for (; k < width; ++k) mp2[s0 + 32 * k] = (unsigned)i;
}

// Per assembly: the opposite bond's values in each slot, and S, U, V per
// particle and layer, in FP64 and FP32.
__global__ void k_mf_prep(int n, const int64_t* __restrict__ bptr, const int64_t* __restrict__ mbase,
                          const int* __restrict__ blayer, const int* __restrict__ opp, const double* __restrict__ cs,
                          const double* __restrict__ bdamage, const double* __restrict__ Kn,
                          const double* __restrict__ Tv, const double* __restrict__ cs_sum,
                          const double* __restrict__ tsum, int64_t ns, double* __restrict__ m64,
                          float* __restrict__ m32, double* __restrict__ S64, double* __restrict__ U64,
                          double* __restrict__ V64, float* __restrict__ S32, float* __restrict__ U32,
                          float* __restrict__ V32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s0 = mbase[i / 32] + (i % 32);
  double so[NL][3] = {{0, 0, 0}, {0, 0, 0}}, to[NL][3] = {{0, 0, 0}, {0, 0, 0}};
  int k = 0;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b, ++k) {
    const int bo = opp[b];
    const double w = 1.0 - bdamage[bo], tv = Tv[bo];
    const double tp = w * tv, c1 = w * (2.0 * Kn[bo] + tv) - tp;
    const double v[kMfFields] = {cs[3 * (int64_t)bo], cs[3 * (int64_t)bo + 1], cs[3 * (int64_t)bo + 2], c1, tp};
    const int64_t slot = s0 + 32 * k;
#pragma unroll
    for (int e = 0; e < kMfFields; ++e) m64[e * ns + slot] = v[e];
    // FP32: one 16-byte word {n'x, n'y, n'z, t'} per slot, then a' - t'
    reinterpret_cast<float4*>(m32)[slot] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)tp);
    m32[4 * ns + slot] = (float)c1;
    const int l = blayer[b] != 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      so[l][c] += v[c];
      to[l][c] += tp * v[c];
    }
  }
#pragma unroll
  for (int l = 0; l < NL; ++l)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t q = ((int64_t)i * NL + l) * 3 + c;
      const double S = cs_sum[q], U = S + so[l][c], V = tsum[q] + to[l][c];
      S64[q] = S;
      U64[q] = U;
      V64[q] = V;
      S32[q] = (float)S;
      U32[q] = (float)U;
      V32[q] = (float)V;
    }
}

// Per assembly: the block row sums R_i of A (FP64, and rounded to FP32),
// the diagonal of K per DOF, the eliminated DOFs and nd = |diag(K)|_2
// (stiffness.h:269-277).  R_i = K_ii^T + sum over i's bonds b = i->j of
//   n' [ -a' n'^T - (t' (U_j - n' - n)^T + V_j^T - t' n'^T - t n^T) / 2 ] + t' S_i n'^T
// (n, t of b itself), the non-difference form of the product applied to the
// three translations.  K_ii = sum_l M_i + T_i S_i^T taken from its upper
// triangle (derivative.h:8-45; [1][0] = 0 in the as-written variant).
template <int DIM>
__global__ void k_mf_rowsum(int n, const int64_t* __restrict__ bptr, const int64_t* __restrict__ mbase,
                            const unsigned* __restrict__ mp2, const double* __restrict__ m64, int64_t ns,
                            const double* __restrict__ cs, const double* __restrict__ bdamage,
                            const double* __restrict__ Tv, const double* __restrict__ S64,
                            const double* __restrict__ U64, const double* __restrict__ V64,
                            const double* __restrict__ tsum, const double* __restrict__ msum, int sym, int elim,
                            const int* __restrict__ mask, const double* __restrict__ dvis,
                            unsigned char* __restrict__ fixed, double* __restrict__ R64, float* __restrict__ R32,
                            double* __restrict__ diag, double* partials, unsigned int* ticket, double* norms) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double K[3][3];
    {
      double k00 = 0, k01 = 0, k02 = 0, k11 = 0, k12 = 0, k22 = 0;
#pragma unroll
      for (int l = 0; l < NL; ++l) {
        const double* M = msum + ((int64_t)NL * i + l) * 6;
        const double* T = tsum + ((int64_t)NL * i + l) * 3;
        const double* S = S64 + ((int64_t)NL * i + l) * 3;
        k00 += M[0] + T[0] * S[0];
        k01 += M[1] + T[0] * S[1];
        k02 += M[2] + T[0] * S[2];
        k11 += M[3] + T[1] * S[1];
        k12 += M[4] + T[1] * S[2];
        k22 += M[5] + T[2] * S[2];
      }
      K[0][0] = k00;
      K[0][1] = k01;
      K[0][2] = k02;
      K[1][0] = sym ? k01 : 0.0;
      K[1][1] = k11;
      K[1][2] = k12;
      K[2][0] = k02;
      K[2][1] = k12;
      K[2][2] = k22;
    }
    double R[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) R[r][c] = K[c][r];
    const int64_t s0 = mbase[i / 32] + (i % 32);
    int k = 0;
    for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b, ++k) {
      const int64_t slot = s0 + 32 * k;
      const unsigned w = mp2[slot];
      const int j = (int)(w & kIdMask), l = (w & kLayerBit) ? 1 : 0;
      const double np[3] = {m64[slot], m64[ns + slot], m64[2 * ns + slot]};
      const double c1 = m64[3 * ns + slot], tp = m64[4 * ns + slot];
      const double nb[3] = {cs[3 * b], cs[3 * b + 1], cs[3 * b + 2]};
      const double tb = (1.0 - bdamage[b]) * Tv[b];
      const double* Uj = U64 + ((int64_t)NL * j + l) * 3;
      const double* Vj = V64 + ((int64_t)NL * j + l) * 3;
      const double* Si = S64 + ((int64_t)NL * i + l) * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double e = np[c];
        const double base = -(c1 + tp) * e - 0.5 * (tp * (Uj[c] - e - nb[c]) + Vj[c] - tp * e - tb * nb[c]);
#pragma unroll
        for (int r = 0; r < 3; ++r) R[r][c] += np[r] * base + tp * e * Si[r];
      }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        R64[(int64_t)i * 9 + r * 3 + c] = R[r][c];
        R32[(int64_t)i * 9 + r * 3 + c] = (float)R[r][c];
      }
    const bool dead = fabs(dvis[i] - 1.0) < EPS;
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
      diag[(int64_t)DIM * i + r] = K[r][r];
      acc[0] += K[r][r] * K[r][r];
      fixed[(int64_t)DIM * i + r] = elim && (mask[3 * i + r] == 1 || dead) ? 1 : 0;
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, partials, ticket, tot) && threadIdx.x == 0) norms[2] = sqrt(tot[0]);
}

// Jacobi preconditioner of A': 1/K_ii[r][r] (1 where it is zero), 1/nd on
// eliminated DOFs.
__global__ void k_mf_invd(int64_t ndof, const double* __restrict__ diag, const unsigned char* __restrict__ fixed,
                          const double* norms, double* __restrict__ invd64, float* __restrict__ invd32) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ndof) return;
  const double a = fixed[q] ? norms[2] : diag[q];
  const double v = a != 0.0 ? 1.0 / a : 1.0;
  invd64[q] = v;
  if (invd32) invd32[q] = (float)v;
}

// Per-precision view of the matrix-free data for the two passes.
template <typename T>
struct MfView {
  const int64_t* __restrict__ mbase;
  const unsigned* __restrict__ mp2;
  // slot coefficients: FP64 [5][ns] (n'x, n'y, n'z, a' - t', t'); FP32 a
  // float4 {n'x, n'y, n'z, t'} per slot, then [ns] a' - t'
  const T* __restrict__ m;
  const T* __restrict__ S;  // [n][2][3]
  const T* __restrict__ U;
  const T* __restrict__ V;
  const T* __restrict__ R;  // [n][9]
  const unsigned char* __restrict__ fixed;
  const double* norms;
  T* __restrict__ HF;  // [2][n][2]: H, F per layer and particle (pass 1 out, pass 2 in)
  int64_t ns;
  int n;
};

// The product's input: p (MODE 0), or the mixed solve's FP64 solution plus
// its double-float increment x64 + (x32 + x32lo) (MODE 1).  With MASK the
// eliminated DOFs read as zero (A' = P A P + nd (I - P)); inside the solves
// the input is already zero there (the right-hand side, and so every
// residual, direction and increment, vanishes on eliminated DOFs), so the
// CG products skip the mask.
template <typename T, int MODE>
__device__ __forceinline__ T mf_in(const T* __restrict__ p, const float* __restrict__ a, const float* __restrict__ b,
                                   int64_t q) {
  if constexpr (MODE == 1) return p[q] + ((T)a[q] + (T)b[q]);
  return p[q];
}

template <typename T, int DIM, int MODE, bool MASK>
__device__ __forceinline__ void mf_load(const MfView<T>& v, const T* __restrict__ p, const float* __restrict__ a,
                                        const float* __restrict__ b, int i, T (&o)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (c < DIM) {
      const int64_t q = (int64_t)DIM * i + c;
      o[c] = (MASK && v.fixed[q]) ? T(0) : mf_in<T, MODE>(p, a, b, q);
    } else {
      o[c] = T(0);
    }
  }
}

// One slot's coefficients.
template <typename T, int DIM>
struct MfSlot {
  T n[3], c1, tp;
};

template <typename T, int DIM>
__device__ __forceinline__ void mf_slot(const MfView<T>& v, int64_t slot, MfSlot<T, DIM>& o) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(v.m) + slot);
    o.n[0] = a.x;
    o.n[1] = a.y;
    o.n[2] = DIM == 3 ? a.z : 0.f;
    o.tp = a.w;
    o.c1 = v.m[4 * v.ns + slot];
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) o.n[c] = c < DIM ? v.m[c * v.ns + slot] : T(0);
    o.c1 = v.m[3 * v.ns + slot];
    o.tp = v.m[4 * v.ns + slot];
  }
}

// The first pass's sums (H, F) of particle j, layer l: one 8- or 16-byte
// load (stored per layer, so a warp's partners read adjacent pairs).
template <typename T>
__device__ __forceinline__ void mf_hf(const MfView<T>& v, int j, int l, T (&o)[2]) {
  const int64_t q = ((int64_t)l * v.n + j) * 2;
  if constexpr (sizeof(T) == 4) {
    const float2 a = *reinterpret_cast<const float2*>(v.HF + q);
    o[0] = a.x;
    o[1] = a.y;
  } else {
    const double2 a = *reinterpret_cast<const double2*>(v.HF + q);
    o[0] = a.x;
    o[1] = a.y;
  }
}

// Pass 1: H_j = sum n'.(p_m - p_j), F_j = sum t' n'.(p_m - p_j) per layer
// over j's bonds.  FP32 sums are compensated and rounded once.  The loop is
// software-pipelined: the next slot's coefficients and partner values, and
// the partner word of the slot after it, are loaded while the current slot
// is used.
template <typename T, int DIM, int MODE, bool MASK>
__global__ void __launch_bounds__(256) k_mf_pass1(MfView<T> v, const T* __restrict__ p, const float* __restrict__ xa,
                                                  const float* __restrict__ xb, const CgScalars* cg) {
  if (cg->done || (MODE == 1 && !cg->ru)) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < v.n; j += gridDim.x * blockDim.x) {
    T pj[3];
    mf_load<T, DIM, MODE, MASK>(v, p, xa, xb, j, pj);
    const int sl = j / 32;
    const int64_t s0 = v.mbase[sl] + (j % 32);
    const int len = (int)((v.mbase[sl + 1] - v.mbase[sl]) / 32);
    T hs[NL] = {T(0), T(0)}, hc[NL] = {T(0), T(0)}, fs[NL] = {T(0), T(0)}, fc[NL] = {T(0), T(0)};
    MfSlot<T, DIM> cur{}, nxt{};
    T pc[3] = {T(0), T(0), T(0)}, pn[3] = {T(0), T(0), T(0)};
    unsigned wc = 0, wn = 0, w2 = 0;
    if (len > 0) {
      wc = v.mp2[s0];
      mf_slot<T, DIM>(v, s0, cur);
      mf_load<T, DIM, MODE, MASK>(v, p, xa, xb, (int)(wc & kIdMask), pc);
      if (len > 1) wn = v.mp2[s0 + 32];
    }
    for (int k = 0; k < len; ++k) {
      if (k + 1 < len) {
        mf_slot<T, DIM>(v, s0 + 32 * (int64_t)(k + 1), nxt);
        mf_load<T, DIM, MODE, MASK>(v, p, xa, xb, (int)(wn & kIdMask), pn);
        if (k + 2 < len) w2 = v.mp2[s0 + 32 * (int64_t)(k + 2)];
      }
      const int l = (wc & kLayerBit) ? 1 : 0;
      T s = cur.n[0] * (pc[0] - pj[0]);
#pragma unroll
      for (int c = 1; c < DIM; ++c) s = fma(cur.n[c], pc[c] - pj[c], s);
      if constexpr (sizeof(T) == 4) {
        df_add(hs[l], hc[l], s, 0.f);
        dot2_acc(fs[l], fc[l], cur.tp, s);
      } else {
        hs[l] += s;
        fs[l] = fma(cur.tp, s, fs[l]);
      }
      cur = nxt;
      wc = wn;
      wn = w2;
#pragma unroll
      for (int c = 0; c < 3; ++c) pc[c] = pn[c];
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      v.HF[((int64_t)l * v.n + j) * 2] = hs[l] + hc[l];
      v.HF[((int64_t)l * v.n + j) * 2 + 1] = fs[l] + fc[l];
    }
  }
}

// Pass 2: y = A' v (see the header), then
//   MODE 0: q = y (FP32: the pair q, qlo), p.q, and alpha in the last block;
//   MODE 1: r = s b - y, |r|^2, and the reliable update's convergence test
//           in the last block (as k_mx_residual).
// Pipelined as pass 1; U and V of the partner are read only for the slots
// flagged by kUVBit (a bond of the partner is damaged or broken on one side).
template <typename T, int DIM, int MODE, bool MASK>
__global__ void __launch_bounds__(256) k_mf_pass2(MfView<T> v, const T* __restrict__ p, const float* __restrict__ xa,
                                                  const float* __restrict__ xb, T* __restrict__ q,
                                                  float* __restrict__ qlo, const double* __restrict__ rhs,
                                                  CgScalars* cg, double* partials, unsigned int* ticket) {
  if (cg->done || (MODE == 1 && !cg->ru)) return;
  double acc = 0.0;
  float ps = 0.f, pcs = 0.f;
  const double nd = v.norms[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += gridDim.x * blockDim.x) {
    T pi[3];
    mf_load<T, DIM, MODE, MASK>(v, p, xa, xb, i, pi);
    T ys[3] = {T(0), T(0), T(0)}, yc[3] = {T(0), T(0), T(0)};
    const T* Ri = v.R + (int64_t)i * 9;
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int c = 0; c < DIM; ++c) {
        if constexpr (sizeof(T) == 4)
          dot2_acc(ys[r], yc[r], Ri[r * 3 + c], pi[c]);
        else
          ys[r] = fma(Ri[r * 3 + c], pi[c], ys[r]);
      }
    const int sl = i / 32;
    const int64_t s0 = v.mbase[sl] + (i % 32);
    const int len = (int)((v.mbase[sl + 1] - v.mbase[sl]) / 32);
    T as[NL] = {T(0), T(0)}, ac[NL] = {T(0), T(0)};
    MfSlot<T, DIM> cur{}, nxt{};
    T pc[3] = {T(0), T(0), T(0)}, pn[3] = {T(0), T(0), T(0)}, hc2[2] = {T(0), T(0)}, hn2[2] = {T(0), T(0)};
    unsigned wc = 0, wn = 0, w2 = 0;
    if (len > 0) {
      wc = v.mp2[s0];
      mf_slot<T, DIM>(v, s0, cur);
      const int j0 = (int)(wc & kIdMask), l0 = (wc & kLayerBit) ? 1 : 0;
      mf_load<T, DIM, MODE, MASK>(v, p, xa, xb, j0, pc);
      mf_hf<T>(v, j0, l0, hc2);
      if (len > 1) wn = v.mp2[s0 + 32];
    }
    for (int k = 0; k < len; ++k) {
      if (k + 1 < len) {
        mf_slot<T, DIM>(v, s0 + 32 * (int64_t)(k + 1), nxt);
        const int j1 = (int)(wn & kIdMask), l1 = (wn & kLayerBit) ? 1 : 0;
        mf_load<T, DIM, MODE, MASK>(v, p, xa, xb, j1, pn);
        mf_hf<T>(v, j1, l1, hn2);
        if (k + 2 < len) w2 = v.mp2[s0 + 32 * (int64_t)(k + 2)];
      }
      const int j = (int)(wc & kIdMask);
      const int l = (wc & kLayerBit) ? 1 : 0;
      T d[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) d[c] = c < DIM ? pc[c] - pi[c] : T(0);
      T s = cur.n[0] * d[0];
#pragma unroll
      for (int c = 1; c < DIM; ++c) s = fma(cur.n[c], d[c], s);
      T ud = T(0), vd = T(0);
      if (wc & kUVBit) {
        const T* Uj = v.U + ((int64_t)j * NL + l) * 3;
        const T* Vj = v.V + ((int64_t)j * NL + l) * 3;
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          ud = fma(Uj[c], d[c], ud);
          vd = fma(Vj[c], d[c], vd);
        }
      }
      const T coef = fma(-cur.c1, s, T(-0.5) * fma(cur.tp, ud + hc2[0], vd + hc2[1]));
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        if constexpr (sizeof(T) == 4)
          dot2_acc(ys[r], yc[r], cur.n[r], coef);
        else
          ys[r] = fma(cur.n[r], coef, ys[r]);
      }
      if constexpr (sizeof(T) == 4)
        dot2_acc(as[l], ac[l], cur.tp, s);
      else
        as[l] = fma(cur.tp, s, as[l]);
      cur = nxt;
      wc = wn;
      wn = w2;
#pragma unroll
      for (int c = 0; c < 3; ++c) pc[c] = pn[c];
      hc2[0] = hn2[0];
      hc2[1] = hn2[1];
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const T* Si = v.S + ((int64_t)i * NL + l) * 3;
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        if constexpr (sizeof(T) == 4) {
          dot2_acc(ys[r], yc[r], as[l], Si[r]);
          yc[r] = fmaf(ac[l], Si[r], yc[r]);
        } else {
          ys[r] = fma(as[l], Si[r], ys[r]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
      const int64_t qi = (int64_t)DIM * i + r;
      T yh, yl;
      if (v.fixed[qi]) {  // eliminated DOF: nd times the unmasked input
        yh = (T)(nd * (double)mf_in<T, MODE>(p, xa, xb, qi));
        yl = T(0);
      } else if constexpr (sizeof(T) == 4) {
        two_sum(ys[r], yc[r], yh, yl);
      } else {
        yh = ys[r];
        yl = T(0);
      }
      if constexpr (MODE == 0) {
        const T pr = p[qi];
        q[qi] = yh;
        if constexpr (sizeof(T) == 4) {
          qlo[qi] = yl;
          dot2_acc(ps, pcs, pr, yh);
          pcs = fmaf(pr, yl, pcs);
        } else {
          acc += (double)pr * (double)yh;
        }
      } else {
        const double ri = rhs[qi] * cg->bscale - (double)yh;
        q[qi] = (T)ri;
        acc += ri * ri;
      }
    }
  }
  double w[1], tot[1];
  bool last;
  if constexpr (sizeof(T) == 4) {
    float s1[1] = {ps}, c1[1] = {pcs};
    block_df_sum<1>(s1, c1, w);
    last = grid_fold<1>(w, partials, ticket, tot);
  } else {
    w[0] = acc;
    last = grid_sum<1>(w, partials, ticket, tot);
  }
  if (last && threadIdx.x == 0) {
    if constexpr (MODE == 0) {
      cg->alpha = cg->abs_new / tot[0];
      df_split(cg->alpha, cg->alpha32, cg->alpha32lo);
    } else {
      cg->rr = tot[0];
      cg->ru_count += 1;
      if (!isfinite(tot[0]))
        cg->done = 3;
      else if (tot[0] < cg->threshold)
        cg->done = 1;
    }
  }
}

// Per assembly: each slot's kUVBit from its partner's U and V (zero for
// intact bonds, whose opposite bonds mirror them exactly).
__global__ void k_mf_flags(int n, const int64_t* __restrict__ mbase, const double* __restrict__ U64,
                           const double* __restrict__ V64, unsigned* __restrict__ mp2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sl = i / 32;
  const int64_t s0 = mbase[sl] + (i % 32);
  const int len = (int)((mbase[sl + 1] - mbase[sl]) / 32);
  for (int k = 0; k < len; ++k) {
    const int64_t slot = s0 + 32 * (int64_t)k;
    const unsigned w = mp2[slot];
    const int j = (int)(w & kIdMask), l = (w & kLayerBit) ? 1 : 0;
    bool nz = false;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      nz = nz || U64[((int64_t)j * NL + l) * 3 + c] != 0.0 || V64[((int64_t)j * NL + l) * 3 + c] != 0.0;
    mp2[slot] = nz ? (w | kUVBit) : (w & ~kUVBit);
  }
}

}  // namespace

namespace {

// Slices of 32 particles as wide as their particle with the most bonds;
// slot partners written once (the bond topology is fixed for the handle).
int mf_setup(lpm_handle* h) {
  Dev& d = h->d;
  const int n = h->n;
  if (n >= (1 << 30)) {
    h->err = "matrix-free operator: 2^30 or more particles";
    return LPM_ERR_ARG;
  }
  std::vector<int64_t> bptr((size_t)n + 1);
  LPM_CUDA(h, cudaMemcpy(bptr.data(), d.bptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
  const int nsl = (n + 31) / 32;
  std::vector<int64_t> mb((size_t)nsl + 1, 0);
  for (int sl = 0; sl < nsl; ++sl) {
    int64_t w = 0;
    for (int i = sl * 32; i < std::min(n, sl * 32 + 32); ++i) w = std::max(w, bptr[(size_t)i + 1] - bptr[(size_t)i]);
    mb[(size_t)sl + 1] = mb[(size_t)sl] + 32 * w;
  }
  const int64_t ns = std::max<int64_t>(mb[(size_t)nsl], 1);
  const size_t N = (size_t)n, P = N * NL * 3;
  d.mbase = (int64_t*)dev_alloc(h, sizeof(int64_t) * mb.size());
  d.mp2 = (unsigned*)zeros_dev(h, sizeof(unsigned) * (size_t)ns);
  d.m64 = (double*)zeros_dev(h, sizeof(double) * kMfFields * (size_t)ns);
  d.m32 = (float*)zeros_dev(h, sizeof(float) * kMfFields * (size_t)ns);
  d.mS64 = (double*)dev_alloc(h, sizeof(double) * P);
  d.mU64 = (double*)dev_alloc(h, sizeof(double) * P);
  d.mV64 = (double*)dev_alloc(h, sizeof(double) * P);
  d.mS32 = (float*)dev_alloc(h, sizeof(float) * P);
  d.mU32 = (float*)dev_alloc(h, sizeof(float) * P);
  d.mV32 = (float*)dev_alloc(h, sizeof(float) * P);
  d.mR64 = (double*)dev_alloc(h, sizeof(double) * N * 9);
  d.mR32 = (float*)dev_alloc(h, sizeof(float) * N * 9);
  d.mdiag = (double*)dev_alloc(h, sizeof(double) * N * h->dim);
  d.mHF64 = (double*)dev_alloc(h, sizeof(double) * N * NL * 2);
  d.mHF32 = (float*)dev_alloc(h, sizeof(float) * N * NL * 2);
  if (!d.mbase || !d.mp2 || !d.m64 || !d.m32 || !d.mS64 || !d.mU64 || !d.mV64 || !d.mS32 || !d.mU32 || !d.mV32 ||
      !d.mR64 || !d.mR32 || !d.mdiag || !d.mHF64 || !d.mHF32)
    return LPM_ERR_NOMEM;
  LPM_CUDA(h, cudaMemcpy(d.mbase, mb.data(), sizeof(int64_t) * mb.size(), cudaMemcpyHostToDevice));
  k_mf_slots<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.bp2, d.blayer, d.mbase, d.mp2);
  LPM_LAUNCHED(h, "k_mf_slots");
  h->mslots = ns;
  h->mnsl = nsl;
  return LPM_OK;
}

template <typename T>
MfView<T> mf_view(lpm_handle* h) {
  Dev& d = h->d;
  if constexpr (sizeof(T) == 4)
    return MfView<T>{d.mbase, d.mp2, d.m32, d.mS32, d.mU32, d.mV32, d.mR32, d.fixed, d.norms, d.mHF32, h->mslots,
                     h->n};
  else
    return MfView<T>{d.mbase, d.mp2, d.m64, d.mS64, d.mU64, d.mV64, d.mR64, d.fixed, d.norms, d.mHF64, h->mslots,
                     h->n};
}

// Grid of the two passes: one thread per particle, grid-stride, at most as
// many blocks as the reduction partials hold.
int mf_grid(const lpm_handle* h) { return grid_for(h->n, 256, kMaxRedBlocks); }

template <typename T, int DIM, bool MASK>
int mf_product_dim(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, const T* p, T* q, float* qlo,
                   cudaGraphNode_t* last) {
  Dev& d = h->d;
  const MfView<T> v = mf_view<T>(h);
  const int G = mf_grid(h);
  const float* nf = nullptr;
  const double* nb = nullptr;
  if (!g) {
    k_mf_pass1<T, DIM, 0, MASK><<<G, 256, 0, h->stream>>>(v, p, nf, nf, d.cg);
    LPM_LAUNCHED(h, "k_mf_pass1");
    k_mf_pass2<T, DIM, 0, MASK><<<G, 256, 0, h->stream>>>(v, p, nf, nf, q, qlo, nb, d.cg, d.red.partials,
                                                            d.red.ticket + 3);
    LPM_LAUNCHED(h, "k_mf_pass2");
    return LPM_OK;
  }
  cudaGraphNode_t n1;
  LPM_CUDA(h, add_kernel(&n1, g, dep, k_mf_pass1<T, DIM, 0, MASK>, G, 256, v, p, nf, nf, (const CgScalars*)d.cg));
  LPM_CUDA(h, add_kernel(last, g, &n1, k_mf_pass2<T, DIM, 0, MASK>, G, 256, v, p, nf, nf, q, qlo, nb, d.cg,
                         d.red.partials, d.red.ticket + 3));
  return LPM_OK;
}

template <int DIM>
int mf_residual_dim(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphNode_t* last) {
  Dev& d = h->d;
  const MfView<double> v = mf_view<double>(h);
  const int G = mf_grid(h);
  float* nf = nullptr;
  if (!g) {
    k_mf_pass1<double, DIM, 1, false><<<G, 256, 0, h->stream>>>(v, d.x64, d.x32, d.x32lo, d.cg);
    LPM_LAUNCHED(h, "k_mf_pass1");
    k_mf_pass2<double, DIM, 1, false><<<G, 256, 0, h->stream>>>(v, d.x64, d.x32, d.x32lo, d.r64, nf, d.rhs, d.cg,
                                                                  d.red.partials, d.red.ticket + 6);
    LPM_LAUNCHED(h, "k_mf_pass2");
    return LPM_OK;
  }
  cudaGraphNode_t n1;
  LPM_CUDA(h, add_kernel(&n1, g, dep, k_mf_pass1<double, DIM, 1, false>, G, 256, v, (const double*)d.x64,
                         (const float*)d.x32, (const float*)d.x32lo, (const CgScalars*)d.cg));
  LPM_CUDA(h, add_kernel(last, g, &n1, k_mf_pass2<double, DIM, 1, false>, G, 256, v, (const double*)d.x64,
                         (const float*)d.x32, (const float*)d.x32lo, d.r64, nf, (const double*)d.rhs, d.cg,
                         d.red.partials, d.red.ticket + 6));
  return LPM_OK;
}

template <bool MASK>
int mf_product_any(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, bool fp32, const void* p, void* q,
                   float* qlo, cudaGraphNode_t* last) {
  if (fp32)
    return h->dim == 3 ? mf_product_dim<float, 3, MASK>(h, g, dep, (const float*)p, (float*)q, qlo, last)
                       : mf_product_dim<float, 2, MASK>(h, g, dep, (const float*)p, (float*)q, qlo, last);
  return h->dim == 3 ? mf_product_dim<double, 3, MASK>(h, g, dep, (const double*)p, (double*)q, nullptr, last)
                     : mf_product_dim<double, 2, MASK>(h, g, dep, (const double*)p, (double*)q, nullptr, last);
}

}  // namespace

int mf_assemble(lpm_handle* h, int tangent, int bc) {
  Dev& d = h->d;
  if (!d.mbase) {
    const int st = mf_setup(h);
    if (st) return st;
  }
  const int n = h->n;
  k_mf_prep<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.mbase, d.blayer, d.opp, d.cs, d.bdamage, d.Kn,
                                                      d.Tv, d.cs_sum, d.tsum, h->mslots, d.m64, d.m32, d.mS64, d.mU64,
                                                      d.mV64, d.mS32, d.mU32, d.mV32);
  LPM_LAUNCHED(h, "k_mf_prep");
  k_mf_flags<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.mbase, d.mU64, d.mV64, d.mp2);
  LPM_LAUNCHED(h, "k_mf_flags");
  const int G = grid_for(n, kRedThreads, kMaxRedBlocks);
  const int sym = tangent == LPM_TANGENT_SYMMETRIC ? 1 : 0, elim = bc == LPM_BC_ELIMINATE ? 1 : 0;
  if (h->dim == 3)
    k_mf_rowsum<3><<<G, kRedThreads, 0, h->stream>>>(n, d.bptr, d.mbase, d.mp2, d.m64, h->mslots, d.cs, d.bdamage,
                                                     d.Tv, d.mS64, d.mU64, d.mV64, d.tsum, d.msum, sym, elim, d.mask,
                                                     d.dvis, d.fixed, d.mR64, d.mR32, d.mdiag, d.red.partials,
                                                     d.red.ticket + 1, d.norms);
  else
    k_mf_rowsum<2><<<G, kRedThreads, 0, h->stream>>>(n, d.bptr, d.mbase, d.mp2, d.m64, h->mslots, d.cs, d.bdamage,
                                                     d.Tv, d.mS64, d.mU64, d.mV64, d.tsum, d.msum, sym, elim, d.mask,
                                                     d.dvis, d.fixed, d.mR64, d.mR32, d.mdiag, d.red.partials,
                                                     d.red.ticket + 1, d.norms);
  LPM_LAUNCHED(h, "k_mf_rowsum");
  h->have_K = true;
  h->tangent = tangent;
  return LPM_OK;
}

int mf_prepare_invd(lpm_handle* h, bool want32) {
  Dev& d = h->d;
  const int64_t ndof = (int64_t)h->n * h->dim;
  k_mf_invd<<<grid_for(ndof, 256), 256, 0, h->stream>>>(ndof, d.mdiag, d.fixed, d.norms, d.invd64,
                                                         want32 ? d.invd32 : nullptr);
  LPM_LAUNCHED(h, "k_mf_invd");
  return LPM_OK;
}

int mf_launch_product(lpm_handle* h, bool fp32, const void* p, void* q, float* qlo, bool mask) {
  return mask ? mf_product_any<true>(h, nullptr, nullptr, fp32, p, q, qlo, nullptr)
              : mf_product_any<false>(h, nullptr, nullptr, fp32, p, q, qlo, nullptr);
}

int mf_graph_product(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, bool fp32, const void* p, void* q,
                     float* qlo, cudaGraphNode_t* last) {
  return mf_product_any<false>(h, g, dep, fp32, p, q, qlo, last);
}

int mf_launch_residual(lpm_handle* h) {
  return h->dim == 3 ? mf_residual_dim<3>(h, nullptr, nullptr, nullptr) : mf_residual_dim<2>(h, nullptr, nullptr, nullptr);
}

int mf_graph_residual(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphNode_t* last) {
  return h->dim == 3 ? mf_residual_dim<3>(h, g, dep, last) : mf_residual_dim<2>(h, g, dep, last);
}

}  // namespace lpm
