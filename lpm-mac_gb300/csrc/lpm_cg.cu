// Jacobi-preconditioned conjugate gradients on A = K^T.
//
// The iteration is the one Eigen's ConjugateGradient runs for
// Solver::LPM_CG (solver.h:192-217): zero start, p = M^-1 r,
//   q = A p; alpha = (r.z)/(p.q); x += alpha p; r -= alpha q;
//   stop if |r|^2 < max(tol^2 |b|^2, DBL_MIN); z = M^-1 r; beta = (r.z)_new/(r.z)_old;
//   p = z + beta p; it++   (at most maxit iterations)
// with M the diagonal of the matrix (1 where it is zero or missing).
//
// Each iteration is three kernels on the handle's stream:
//   k_cg_spmv    q = A p and p.q; the last block sets alpha
//   k_cg_update  x, r, |r|^2, r.z; the last block tests convergence, sets beta
//   k_cg_pupdate p = z + beta p
// Kernels return at once when the device flag `done` is set.  Each solve
// runs its whole loop as one CUDA graph whose loop condition (and, for the
// mixed solve, reliable-update condition) is set on the device
// (build_fp64_graph, build_mixed_graph); under kernel timing the host
// enqueues the iterations in batches instead and reads the flag once per
// batch.
//
// Mixed precision: the same recurrence on an FP32 copy of A with FP32
// vectors; the dots accumulate as compensated FP32 pairs, converted to FP64
// once per block, and the scalars are FP64.  The FP32 product is taken in
// difference form, (A p)_i = S_i p_i + sum_j A_ij (p_j - p_i) with S_i the
// block row sum of A (exact algebra).  The stiffness rows nearly sum to zero
// (rigid translations cost no force), so for the smooth directions that CG
// resolves last the plain sum cancels to a small fraction of its terms and
// FP32 rounding swamps it; the differences keep those terms small, and a
// compensated accumulation (dot2_acc) removes the rounding of the sum.
// Without both, the FP32 iterate carries errors along the smooth directions
// that its residual barely shows, and the next Newton solve pays for them
// (about 50% more iterations at 101^3).  With both, the first solve of a
// load step takes the FP64 iteration count and later ones 10-30% more.  (An
// operator kept as two FP32 words per value did not remove that excess on a
// 2-D compact-tension plate; an emulation of this recurrence places it in the
// FP32 residual, product output and solution increment, and in alpha and
// beta rounded to FP32.)
// The recurrence runs with reliable updates (residual replacement): when the
// iterated residual has fallen by kDelta since the last update, the FP32
// solution increment is folded into the FP64 solution, the residual is
// recomputed in FP64 as b - A64 x and replaces the iterated one, and the
// iteration continues with its search direction.  The solve stops on the
// FP64 residual.  Every update is one FP64 sparse product.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <tuple>
#include <vector>

#include "lpm_cgvec.cuh"
#include "lpm_coarse.cuh"
#include "lpm_device.cuh"
#include "lpm_df.cuh"
#include "lpm_graph.cuh"
#include "lpm_grid.cuh"

namespace lpm {
namespace {

// One thread per row of A over the sliced layout: the 32 rows of a warp read
// their k-th blocks from consecutive slots, and every FMA is useful work
// (no cross-lane reduction of the row sums).
struct SellView {
  const int64_t* __restrict__ sell_ptr;
  const int* __restrict__ scol;
  const int* __restrict__ rowlen;
  const float* __restrict__ S;     // block row sums (FP32 difference-form product only)
  const short* __restrict__ soff;  // column - row per slot when every offset fits 16 bits (FP32 product)
  int64_t nslots;
  int n;
};

// Four column indices of a group of slots: 16-bit offsets from the row
// (8 bytes a group) when they fit, else the 32-bit columns (16 bytes).
template <bool OFF16>
__device__ __forceinline__ int4 group_cols(const SellView& v, int row, int64_t s) {
  if (OFF16) {
    const short4 o = __ldg(reinterpret_cast<const short4*>(v.soff + s));
    return make_int4(row + o.x, row + o.y, row + o.z, row + o.w);
  }
  return __ldg(reinterpret_cast<const int4*>(v.scol + s));
}

__device__ __forceinline__ int comp(const int4& v, int t) { return t == 0 ? v.x : t == 1 ? v.y : t == 2 ? v.z : v.w; }
__device__ __forceinline__ float comp(const float4& v, int t) {
  return t == 0 ? v.x : t == 1 ? v.y : t == 2 ? v.z : v.w;
}

// Four values of the FP32 operator.  An operator that fits in L2 with room
// to spare is read with the default policy and stays there from one
// iteration to the next (KEEP); a larger one streams through with
// evict-first loads, which leaves L2 to the vectors.
template <bool KEEP>
__device__ __forceinline__ float4 op_load(const float* a) {
  if (KEEP) return __ldg(reinterpret_cast<const float4*>(a));
  return __ldcs(reinterpret_cast<const float4*>(a));
}
template <bool KEEP>
__device__ __forceinline__ float op_load1(const float* a) {
  if (KEEP) return __ldg(a);
  return __ldcs(a);
}

// A vector entry.  Kernels that never write the vector read it through the
// read-only cache; the persistent solve (COH), whose blocks write the
// vectors between grid barriers, reads them from L2 (ld.global.cg), which
// the barrier's fences order after the writes.
template <bool COH>
__device__ __forceinline__ float ldv(const float* a) {
  if (COH) return __ldcg(a);
  return __ldg(a);
}
template <bool COH>
__device__ __forceinline__ double ldv(const double* a) {
  if (COH) return __ldcg(a);
  return __ldg(a);
}

// y = row `row` of A times p (FP32), in difference form with compensated
// accumulation: the sum comes out as if accumulated in twice the precision
// and then rounded, so the only FP32 errors left are in the differences
// (exact for neighbouring values within a factor of two) and the operator's
// own rounding.  The row is walked in groups of four blocks: one 16-byte load
// brings a block element for four blocks.  Padding blocks are zero and point
// at the row itself.  The blocks past the slice's groups (at most three) are
// read one at a time, in the same order, so the sum is that of the blocks in
// slot order either way.
template <int DIM, bool OFF16, bool KEEP, bool COH = false>
__device__ __forceinline__ void row_product32(const SellView& v, const float* __restrict__ A,
                                              const float* __restrict__ p, int row, float (&y)[DIM],
                                              float (&ylo)[DIM]) {
  float sc[DIM], cc[DIM];
#pragma unroll
  for (int r = 0; r < DIM; ++r) sc[r] = cc[r] = 0.f;
  float pi[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) pi[k] = ldv<COH>(&p[(int64_t)row * DIM + k]);
  const int len = v.rowlen[row];
  const SellRow sr = sell_row(v.sell_ptr, row);
  const int ng = (min(len, sr.g4) + kVec - 1) / kVec;
  const int64_t base = sr.base;
  // software pipeline: the next group's values and partner values, and the
  // columns of the group after it, are in flight while the current group is
  // multiplied
  int4 c4n = make_int4(row, row, row, row);
  float4 an[DIM * DIM];
  float pn[kVec][DIM];
  if (ng > 0) {
    const int4 c40 = group_cols<OFF16>(v, row, base);
#pragma unroll
    for (int e = 0; e < DIM * DIM; ++e) an[e] = op_load<KEEP>(A + e * v.nslots + base);
#pragma unroll
    for (int t = 0; t < kVec; ++t)
#pragma unroll
      for (int k = 0; k < DIM; ++k) pn[t][k] = ldv<COH>(&p[(int64_t)comp(c40, t) * DIM + k]);
    if (ng > 1) c4n = group_cols<OFF16>(v, row, base + kSlice * kVec);
  }
  for (int g = 0; g < ng; ++g) {
    float4 a[DIM * DIM];
    float pg[kVec][DIM];
#pragma unroll
    for (int e = 0; e < DIM * DIM; ++e) a[e] = an[e];
#pragma unroll
    for (int t = 0; t < kVec; ++t)
#pragma unroll
      for (int k = 0; k < DIM; ++k) pg[t][k] = pn[t][k];
    if (g + 1 < ng) {
      const int64_t s1 = base + (int64_t)(g + 1) * (kSlice * kVec);
#pragma unroll
      for (int e = 0; e < DIM * DIM; ++e) an[e] = op_load<KEEP>(A + e * v.nslots + s1);
#pragma unroll
      for (int t = 0; t < kVec; ++t)
#pragma unroll
        for (int k = 0; k < DIM; ++k) pn[t][k] = ldv<COH>(&p[(int64_t)comp(c4n, t) * DIM + k]);
      if (g + 2 < ng) c4n = group_cols<OFF16>(v, row, s1 + kSlice * kVec);
    }
#pragma unroll
    for (int t = 0; t < kVec; ++t) {
      float pc[DIM];
#pragma unroll
      for (int k = 0; k < DIM; ++k) pc[k] = pg[t][k] - pi[k];
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int k = 0; k < DIM; ++k) dot2_acc(sc[r], cc[r], comp(a[r * DIM + k], t), pc[k]);
    }
  }
  for (int k = sr.g4; k < len; ++k) {
    const int64_t st = sr.tail + (int64_t)(k - sr.g4) * kSlice;
    const int c = OFF16 ? row + __ldg(&v.soff[st]) : __ldg(&v.scol[st]);
    float pc[DIM];
#pragma unroll
    for (int q = 0; q < DIM; ++q) pc[q] = ldv<COH>(&p[(int64_t)c * DIM + q]) - pi[q];
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int q = 0; q < DIM; ++q) dot2_acc(sc[r], cc[r], op_load1<KEEP>(A + (r * DIM + q) * v.nslots + st), pc[q]);
  }
  const float* Si = v.S + (int64_t)row * DIM * DIM;
#pragma unroll
  for (int r = 0; r < DIM; ++r) {
#pragma unroll
    for (int k = 0; k < DIM; ++k) dot2_acc(sc[r], cc[r], __ldg(&Si[r * DIM + k]), pi[k]);
    two_sum(sc[r], cc[r], y[r], ylo[r]);  // the compensated sum as a double-float pair
  }
}

// FP64: the partner values of the four blocks are gathered first; then each
// element's 32-byte run (four blocks) is read as two back-to-back 16-byte
// loads, so both halves of a sector are used by the same instruction pair.
// The blocks past the slice's groups follow one at a time.
// With ADD32 the product is taken of p + (p32 + p32lo) (an FP64 vector plus
// a double-float increment not yet folded into it).
template <int DIM, bool ADD32 = false, bool COH = false>
__device__ __forceinline__ double add_increment(const double* __restrict__ p, const float* __restrict__ p32,
                                                const float* __restrict__ p32lo, int64_t i) {
  if (ADD32) return ldv<COH>(&p[i]) + ((double)ldv<COH>(&p32[i]) + (double)ldv<COH>(&p32lo[i]));
  return ldv<COH>(&p[i]);
}

template <int DIM, bool ADD32 = false, bool COH = false>
__device__ __forceinline__ void row_product(const SellView& v, const double* __restrict__ A,
                                            const double* __restrict__ p, int row, double (&y)[DIM],
                                            const float* __restrict__ p32 = nullptr,
                                            const float* __restrict__ p32lo = nullptr) {
#pragma unroll
  for (int r = 0; r < DIM; ++r) y[r] = 0.0;
  const int len = v.rowlen[row];
  const SellRow sr = sell_row(v.sell_ptr, row);
  const int ng = (min(len, sr.g4) + kVec - 1) / kVec;
  const int64_t base = sr.base;
  for (int g = 0; g < ng; ++g) {
    const int64_t s0 = base + (int64_t)g * (kSlice * kVec);
    const int4 c4 = __ldg(reinterpret_cast<const int4*>(v.scol + s0));
    double pc[kVec][DIM];
#pragma unroll
    for (int t = 0; t < kVec; ++t) {
      const int64_t c = (int64_t)comp(c4, t) * DIM;
#pragma unroll
      for (int k = 0; k < DIM; ++k) pc[t][k] = add_increment<DIM, ADD32, COH>(p, p32, p32lo, c + k);
    }
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const double* a = A + (r * DIM + k) * v.nslots + s0;
        const double2 lo = __ldcs(reinterpret_cast<const double2*>(a));
        const double2 hi = __ldcs(reinterpret_cast<const double2*>(a + 2));
        y[r] = fma(lo.x, pc[0][k], y[r]);
        y[r] = fma(lo.y, pc[1][k], y[r]);
        y[r] = fma(hi.x, pc[2][k], y[r]);
        y[r] = fma(hi.y, pc[3][k], y[r]);
      }
  }
  for (int k = sr.g4; k < len; ++k) {
    const int64_t st = sr.tail + (int64_t)(k - sr.g4) * kSlice;
    const int64_t c = (int64_t)__ldg(&v.scol[st]) * DIM;
    double pc[DIM];
#pragma unroll
    for (int q = 0; q < DIM; ++q) pc[q] = add_increment<DIM, ADD32, COH>(p, p32, p32lo, c + q);
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int q = 0; q < DIM; ++q) y[r] = fma(__ldcs(A + (r * DIM + q) * v.nslots + st), pc[q], y[r]);
  }
}

// Launch bounds: the 3-D FP32 product is held to two blocks per SM (128
// registers), which measured level with the product before the partner
// values were prefetched; the 2-D one takes 80 registers (three blocks per SM)
// and measured 2 % faster on the CT plate's load step than at 64 registers.
// The FP64 product, bound by the FP64 pipe, is held to four blocks per SM (64
// registers): at 70 registers and three blocks it measured 2 % slower.
template <typename T, int DIM>
constexpr int kSpmvMinBlocks = sizeof(T) == 8 ? 4 : DIM == 3 ? 2 : 0;

// q = A p and the p.q sum for alpha.  The FP32 product (mixed solve) writes
// q as a double-float pair: its high words to q, its low words to qlo.
template <typename T, int DIM, bool OFF16 = false, bool KEEP = false>
__global__ void __launch_bounds__(256, (kSpmvMinBlocks<T, DIM>)) k_cg_spmv(SellView v, const T* __restrict__ A,
                                                                         const T* __restrict__ p, T* __restrict__ q,
                                                                         CgScalars* cg, double* partials,
                                                                         unsigned int* ticket,
                                                                         float* __restrict__ qlo) {
  if (cg->done) return;
  double acc = 0.0;
  float ps = 0.f, pc = 0.f;  // FP32: p.q as a compensated double-float sum
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < v.n; row += gridDim.x * blockDim.x) {
    T y[DIM];
    if constexpr (sizeof(T) == 4) {
      float yl[DIM];
      row_product32<DIM, OFF16, KEEP>(v, A, p, row, y, yl);
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        const float pr = p[(int64_t)row * DIM + r];
        q[(int64_t)row * DIM + r] = y[r];
        qlo[(int64_t)row * DIM + r] = yl[r];
        dot2_acc(ps, pc, pr, y[r]);
        pc = fmaf(pr, yl[r], pc);
      }
    } else {
      row_product<DIM>(v, A, p, row, y);
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        q[(int64_t)row * DIM + r] = y[r];
        acc += (double)p[(int64_t)row * DIM + r] * (double)y[r];
      }
    }
  }
  double w[1], tot[1];
  bool last;
  if constexpr (sizeof(T) == 4) {
    float s1[1] = {ps}, c1[1] = {pc};
    block_df_sum<1>(s1, c1, w);
    last = grid_fold<1>(w, partials, ticket, tot);
  } else {
    w[0] = acc;
    last = grid_sum<1>(w, partials, ticket, tot);
  }
  if (last && threadIdx.x == 0) {
    cg->alpha = cg->abs_new / tot[0];
    df_split(cg->alpha, cg->alpha32, cg->alpha32lo);
  }
}

// Jacobi preconditioner from the diagonal blocks of A (= diagonal of K).
template <int DIM>
__global__ void k_invd(int n, const int* __restrict__ diag_slot, const double* __restrict__ A, int64_t nslots,
                       double* __restrict__ invd64, float* __restrict__ invd32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = diag_slot[i];
#pragma unroll
  for (int r = 0; r < DIM; ++r) {
    const double a = s >= 0 ? A[(r * DIM + r) * nslots + s] : 0.0;
    const double v = a != 0.0 ? 1.0 / a : 1.0;
    invd64[DIM * i + r] = v;
    if (invd32) invd32[DIM * i + r] = (float)v;
  }
}

constexpr double kDelta = 0.1;  // reliable-update trigger: |r| < kDelta * max |r| since the last update

// max |b| for the scaling of the mixed solve
__global__ void k_absmax(int64_t m, const double* __restrict__ b, CgScalars* cg) {
  unsigned long long mx = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const double a = fabs(b[i]);
    if (isfinite(a)) mx = max(mx, (unsigned long long)__double_as_longlong(a));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(&cg->bmax_bits, mx);
}

// Power of two s with s max|b| in [1, 2): the FP32 recurrence then works on
// values of order one whatever the load magnitude (no FP32 underflow or
// overflow), and the scaling is exact in FP64.
__device__ __forceinline__ double rhs_scale(const CgScalars* cg) {
  const double m = __longlong_as_double((long long)cg->bmax_bits);
  return m > 0.0 ? ldexp(1.0, -ilogb(m)) : 1.0;
}

// Mixed solve set-up: (r32, r32lo) = s b, x = 0, p32 = M r32, |s b|^2, r.z.
__global__ void k_mx_init(int64_t ndof, const double* __restrict__ b, float* __restrict__ x32,
                          float* __restrict__ x32lo, float* __restrict__ r32, float* __restrict__ r32lo,
                          float* __restrict__ p32, const float* __restrict__ invd, CgScalars* cg, double tol,
                          long long maxit, double* partials, unsigned int* ticket) {
  double v[2] = {0.0, 0.0};
  const double sc = rhs_scale(cg);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const double bi = b[i] * sc;
    float r, rl;
    df_split(bi, r, rl);
    const float z = invd[i] * r;
    x32[i] = 0.f;
    x32lo[i] = 0.f;
    r32[i] = r;
    r32lo[i] = rl;
    p32[i] = z;
    v[0] += bi * bi;
    v[1] += bi * (double)z;
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rhs_norm2 = tot[0];
    cg->rr = tot[0];
    cg->threshold = fmax(tol * tol * tot[0], DBL_MIN);
    cg->abs_new = tot[1];
    cg->alpha = cg->beta = 0.0;
    cg->it = 0;
    cg->maxit = maxit;
    cg->ru = 0;
    cg->pfault = 0;
    cg->ru_count = 0;
    cg->graph_passes = 0;
    cg->zcoef = 1.0;
    cg->alpha32 = cg->beta32 = cg->alpha32lo = cg->beta32lo = 0.f;
    cg->zcoef32 = 1.f;
    cg->bscale = sc;
    cg->rmax = sqrt(tot[0]);
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

// Double-float update of the solution increment x and the residual r:
// x += alpha p, r -= alpha q, with alpha a double-float pair, then FP64
// |r|^2 and r.z (z = M r rounded to FP32).  The last block either asks for a
// reliable update (residual fell by kDelta, or below the tolerance: the true
// residual decides) or forms beta.
__global__ void __launch_bounds__(256) k_mx_update(int64_t ndof, float* __restrict__ x, float* __restrict__ xlo,
                                                   float* __restrict__ r, float* __restrict__ rlo,
                                                   const float* __restrict__ p, const float* __restrict__ q,
                                                   const float* __restrict__ qlo, const float* __restrict__ invd,
                                                   CgScalars* cg, double* partials, unsigned int* ticket,
                                                   cudaGraphConditionalHandle ru_cond) {
  if (cg->done) return;
  const float ah = cg->alpha32, al = cg->alpha32lo;
  // |r|^2 and r.z as compensated double-float sums, FP64 only per warp
  float s[2] = {0.f, 0.f}, c[2] = {0.f, 0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    float rh = r[i], rl = rlo[i], xh = x[i], xl = xlo[i];
    df_madd(rh, rl, -ah, -al, q[i], qlo[i]);
    df_madd(xh, xl, ah, al, p[i], 0.f);
    x[i] = xh;
    xlo[i] = xl;
    r[i] = rh;
    rlo[i] = rl;
    const float zi = invd[i] * rh;
    dot2_acc(s[0], c[0], rh, rh);
    c[0] = fmaf(2.f * rh, rl, c[0]);
    dot2_acc(s[1], c[1], rh, zi);
    c[1] = fmaf(rl, zi, c[1]);
  }
  double v[2];
  block_df_sum<2>(s, c, v);
  double tot[2];
  if (grid_fold<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rr = tot[0];
    cg->it += 1;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      cg->done = 3;
      if (ru_cond) cudaGraphSetConditional(ru_cond, 0u);
      return;
    }
    const double rn = sqrt(tot[0]);
    if (tot[0] < cg->threshold || rn < kDelta * cg->rmax) {
      cg->ru = 1;
    } else {
      cg->rmax = fmax(cg->rmax, rn);
      const double old = cg->abs_new;
      cg->abs_new = tot[1];
      cg->beta = tot[1] / old;
      cg->zcoef = 1.0;
      df_split(cg->beta, cg->beta32, cg->beta32lo);
      cg->zcoef32 = 1.f;
    }
    if (cg->it >= cg->maxit) cg->done = 2;
    if (ru_cond) cudaGraphSetConditional(ru_cond, cg->ru ? 1u : 0u);
  }
}

// End of the solve: x64 += x (what the last iterations added, a double-float
// pair), x = 0, and the right-hand-side scaling undone.
__global__ void k_mx_fold(int64_t ndof, float* __restrict__ x32, float* __restrict__ x32lo, double* __restrict__ x64,
                          const CgScalars* cg) {
  const double unscale = 1.0 / cg->bscale;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    x64[i] = (x64[i] + ((double)x32[i] + (double)x32lo[i])) * unscale;
    x32[i] = 0.f;
    x32lo[i] = 0.f;
  }
}

// Reliable update, part 1: r64 = s b - A64 (x64 + x) with the increment x a
// double-float pair, and |r64|^2; converged when it is below the threshold.
template <int DIM>
__global__ void __launch_bounds__(256) k_mx_residual(SellView v, const double* __restrict__ A,
                                                     const double* __restrict__ x, const float* __restrict__ x32,
                                                     const float* __restrict__ x32lo, const double* __restrict__ b,
                                                     double* __restrict__ r, CgScalars* cg, double* partials,
                                                     unsigned int* ticket) {
  if (cg->done || !cg->ru) return;
  double acc = 0.0;
  const double sc = cg->bscale;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < v.n; row += gridDim.x * blockDim.x) {
    double y[DIM];
    row_product<DIM, true>(v, A, x, row, y, x32, x32lo);
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const double ri = b[(int64_t)row * DIM + c] * sc - y[c];
      r[(int64_t)row * DIM + c] = ri;
      acc += ri * ri;
    }
  }
  double w[1] = {acc}, tot[1];
  if (grid_sum<1>(w, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rr = tot[0];
    cg->ru_count += 1;
    if (!isfinite(tot[0]))
      cg->done = 3;
    else if (tot[0] < cg->threshold)
      cg->done = 1;
  }
}

// Reliable update, part 2: x64 += x, x = 0, r = r64 (as a double-float
// pair), new r.z and beta, reset the maximum.  The replaced residual is no
// longer orthogonal to the last search direction; the next direction is
// formed from p - (r.p / r.z) z, which restores r.p = 0, i.e.
// p_new = (1 - beta gamma) z + beta p.
__global__ void k_mx_replace(int64_t ndof, const double* __restrict__ r64, float* __restrict__ r32,
                             float* __restrict__ r32lo, float* __restrict__ x32, float* __restrict__ x32lo,
                             double* __restrict__ x64, const float* __restrict__ p32, const float* __restrict__ invd,
                             CgScalars* cg, double* partials, unsigned int* ticket) {
  if (cg->done || !cg->ru) return;
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    x64[i] += (double)x32[i] + (double)x32lo[i];
    x32[i] = 0.f;
    x32lo[i] = 0.f;
    const double ri = r64[i];
    float rh, rl;
    df_split(ri, rh, rl);
    r32[i] = rh;
    r32lo[i] = rl;
    v[0] += ri * (double)(invd[i] * rh);
    v[1] += ri * (double)p32[i];
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    const double old = cg->abs_new;
    cg->abs_new = tot[0];
    cg->beta = tot[0] / old;
    const double gamma = tot[0] != 0.0 ? tot[1] / tot[0] : 0.0;
    cg->zcoef = 1.0 - cg->beta * gamma;
    df_split(cg->beta, cg->beta32, cg->beta32lo);
    cg->zcoef32 = (float)cg->zcoef;
    cg->rmax = sqrt(cg->rr);
    cg->ru = 0;
  }
}

// p = zcoef z + beta p with z = M^-1 r (r's high words), beta a
// double-float pair, p in FP32.
// Inside the solve graph it is the last kernel of an iteration: block 0
// sets the loop condition (continue while nothing has ended the solve) and
// counts the iteration's kernel launches.
__global__ void __launch_bounds__(256) k_mx_pupdate(int64_t ndof, const float* __restrict__ r,
                                                    const float* __restrict__ invd, float* __restrict__ p,
                                                    CgScalars* cg, cudaGraphConditionalHandle loop_cond) {
  if (loop_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    cudaGraphSetConditional(loop_cond, cg->done ? 0u : 1u);
    cg->graph_passes += 1;
  }
  if (cg->done) return;
  const float bh = cg->beta32, bl = cg->beta32lo, zc = cg->zcoef32;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const float pi = p[i];
    p[i] = fmaf(bh, pi, fmaf(bl, pi, __fmul_rn(zc, __fmul_rn(invd[i], r[i]))));
  }
}

// ---- the mixed solve as one persistent kernel ----------------------------
// For systems that do not fill the GPU, the graph's three kernels per
// iteration each cost a launch, a partly idle tail and a last-block fold,
// together as much as the product itself on a 100k-particle plate.  Here the
// blocks stay resident for the whole solve.  Every phase gives a thread the
// same rows (the update and direction of a row's DOFs run on the thread that
// took its product), so only p (read at the neighbours by the product) and
// the solution (read at the neighbours by the FP64 residual) cross blocks,
// and those reads go to L2.  Sums meet at grid barriers: each block
// publishes its partial, waits, and folds all partials in block order, so
// every block holds the same totals and takes the same branches.  The
// recurrence, the reliable updates and the stopping rule are those of
// k_mx_update, k_mx_residual, k_mx_replace and k_mx_pupdate.

// Everything the persistent solve reads and writes.
struct PcgMixed {
  SellView v;
  const float* A32;
  const double* A64;
  const double* b;     // right-hand side (unscaled)
  const float* invd;
  float *x, *xlo, *r, *rlo, *p, *q, *qlo;
  double *x64, *r64;
  CgScalars* cg;
  double* partials;          // 7 x gridDim.x
  unsigned long long* gbar;  // barrier arrivals, zero at launch
  long long spin_limit;      // polls before a barrier wait gives up
  // coarse correction (COARSE): z = D^-1 r + P A_c^-1 P^T r (lpm_coarse.cu)
  const int *cagg, *cmem_ptr, *cmem;
  const float* coff;
  const unsigned char* cfixed;  // eliminated DOFs, or null
  const double* cAinv;  // inverse of A_c (symmetric)
  double *cyc, *cec;
  float* cz;
  int cnagg;
};

// z = D^-1 r + P A_c^-1 P^T r for this thread's rows, into a.cz, from r's
// high words (written before the caller's last barrier).  The restriction
// y = P^T r and the coarse solve e = A_c^-1 y each take one block per
// aggregate (the members, or the columns of A_c^-1, spread over the block's
// threads, summed in FP32 pairs reduced over the block in a fixed order:
// GB300's FP64 pipe would make FP64 sums cost more than the product; the
// coarse product keeps one FP64 product per term, since A_c^-1 of small
// boxes can be too ill-conditioned for FP32 entries) and end at a grid
// barrier; then each row adds P_i e to its Jacobi term.  False if a barrier
// wait gave up.
template <int DIM>
__device__ bool coarse_z(const PcgMixed& a, unsigned long long& target) {
  constexpr int NM = kModes<DIM>;
  const int nc = a.cnagg * NM;
  for (int ag = blockIdx.x; ag < a.cnagg; ag += gridDim.x) {
    float sm[NM], cm[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) sm[m] = cm[m] = 0.f;
    for (int t = a.cmem_ptr[ag] + threadIdx.x; t < a.cmem_ptr[ag + 1]; t += blockDim.x) {
      const int i = a.cmem[t];
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const int64_t q = (int64_t)DIM * i + k;
        if (a.cfixed && a.cfixed[q]) continue;
        float w[NM];
        mode_row<DIM, float>(k, a.coff[3 * i], a.coff[3 * i + 1], a.coff[3 * i + 2], w);
        const float rk = __ldcg(&a.r[q]);
#pragma unroll
        for (int m = 0; m < NM; ++m) dot2_acc(sm[m], cm[m], w[m], rk);
      }
    }
    double y[NM];
    block_df_sum<NM>(sm, cm, y);
    if (threadIdx.x == 0)
#pragma unroll
      for (int m = 0; m < NM; ++m) a.cyc[ag * NM + m] = y[m];
  }
  target += (unsigned long long)gridDim.x;
  if (!grid_barrier(a.gbar, target, a.spin_limit)) return false;
  for (int ag = blockIdx.x; ag < a.cnagg; ag += gridDim.x) {
    float sm[NM], cm[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) sm[m] = cm[m] = 0.f;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
      const double yc = __ldcg(&a.cyc[c]);
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        // one FP64 product per term, summed as a compensated FP32 pair
        float ph, pl;
        df_split(__ldg(&a.cAinv[(int64_t)(ag * NM + m) * nc + c]) * yc, ph, pl);
        df_add(sm[m], cm[m], ph, pl);
      }
    }
    double e[NM];
    block_df_sum<NM>(sm, cm, e);
    if (threadIdx.x == 0)
#pragma unroll
      for (int m = 0; m < NM; ++m) a.cec[ag * NM + m] = e[m];
  }
  target += (unsigned long long)gridDim.x;
  if (!grid_barrier(a.gbar, target, a.spin_limit)) return false;
  const int stride = gridDim.x * blockDim.x;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.v.n; row += stride) {
    const int ag = a.cagg[row];
    float e[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) e[m] = (float)__ldcg(&a.cec[ag * NM + m]);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const int64_t q = (int64_t)row * DIM + k;
      float zi = a.invd[q] * a.r[q];
      if (!(a.cfixed && a.cfixed[q])) {
        float w[NM];
        mode_row<DIM, float>(k, a.coff[3 * row], a.coff[3 * row + 1], a.coff[3 * row + 2], w);
#pragma unroll
        for (int m = 0; m < NM; ++m) zi = fmaf(w[m], e[m], zi);
      }
      a.cz[q] = zi;
    }
  }
  return true;
}

// The block's copy of the solve's scalars: thread 0 updates it between
// barriers, every thread reads it.
struct PcgState {
  double abs_new, rmax, threshold, bscale, rr;
  long long it, maxit, ru_count, passes;
  int done, ru;
  float ah, al, bh, bl, zc;
};

// Most threads per block of the persistent kernel: one block per SM with
// the register budget of the FP32 product (2-D: 80 registers, 3-D: 128), as
// many threads per SM as the product's 256-thread blocks.  Few large blocks
// keep the barriers short: a barrier with its fold measured 2.6 us over 152
// blocks against 4.4 us over 456.
template <int DIM>
constexpr int kPcgThreads = DIM == 3 ? 512 : 768;

template <int DIM, bool OFF16, bool COARSE>
__global__ void __launch_bounds__(kPcgThreads<DIM>, 1) k_mx_persistent(PcgMixed a) {
  __shared__ PcgState s;
  if (threadIdx.x == 0) {
    const CgScalars* c = a.cg;
    s.abs_new = c->abs_new;
    s.rmax = c->rmax;
    s.threshold = c->threshold;
    s.bscale = c->bscale;
    s.rr = c->rr;
    s.it = c->it;
    s.maxit = c->maxit;
    s.ru_count = c->ru_count;
    s.passes = 0;
    s.done = c->done;
    s.ru = 0;
    s.ah = s.al = s.bh = s.bl = 0.f;
    s.zc = 1.f;
  }
  __syncthreads();
  const int n = a.v.n;
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long target = 0;
  bool fault = false;
  if (COARSE && !s.done) {
    // the first direction is the coarse-corrected z of the initial residual
    if (!coarse_z<DIM>(a, target)) fault = true;
    if (!fault) {
      float sz[1] = {0.f}, cz[1] = {0.f};
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          const float zi = a.cz[i];
          a.p[i] = zi;
          dot2_acc(sz[0], cz[0], a.r[i], zi);
          cz[0] = fmaf(a.rlo[i], zi, cz[0]);
        }
      double w[1] = {0.0}, tot[1];
      block_df_sum<1>(sz, cz, w);
      if (!grid_allreduce<1>(w, a.partials, 6, a.gbar, target, a.spin_limit, tot)) fault = true;
      if (threadIdx.x == 0 && !fault) s.abs_new = tot[0];
      __syncthreads();
    }
  }
  while (!s.done && !fault) {
    // q = A p (FP32, double-float output) and p.q; alpha
    {
      float ps = 0.f, pc = 0.f;
      for (int row = t0; row < n; row += stride) {
        float y[DIM], yl[DIM];
        row_product32<DIM, OFF16, true, true>(a.v, a.A32, a.p, row, y, yl);
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
          const int64_t i = (int64_t)row * DIM + r;
          const float pr = a.p[i];
          a.q[i] = y[r];
          a.qlo[i] = yl[r];
          dot2_acc(ps, pc, pr, y[r]);
          pc = fmaf(pr, yl[r], pc);
        }
      }
      float s1[1] = {ps}, c1[1] = {pc};
      double w[1] = {0.0}, tot[1];
      block_df_sum<1>(s1, c1, w);
      if (!grid_allreduce<1>(w, a.partials, 0, a.gbar, target, a.spin_limit, tot)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) df_split(s.abs_new / tot[0], s.ah, s.al);
      __syncthreads();
    }
    // x += alpha p, r -= alpha q (double-float pairs), |r|^2 and r.z; then
    // a reliable update is due, or beta
    {
      const float ah = s.ah, al = s.al;
      float sb[2] = {0.f, 0.f}, cb[2] = {0.f, 0.f};
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          float rh = a.r[i], rl = a.rlo[i], xh = a.x[i], xl = a.xlo[i];
          df_madd(rh, rl, -ah, -al, a.q[i], a.qlo[i]);
          df_madd(xh, xl, ah, al, a.p[i], 0.f);
          a.x[i] = xh;
          a.xlo[i] = xl;
          a.r[i] = rh;
          a.rlo[i] = rl;
          const float zi = a.invd[i] * rh;
          dot2_acc(sb[0], cb[0], rh, rh);
          cb[0] = fmaf(2.f * rh, rl, cb[0]);
          dot2_acc(sb[1], cb[1], rh, zi);
          cb[1] = fmaf(rl, zi, cb[1]);
        }
      double w[2] = {0.0, 0.0}, tot[2];
      block_df_sum<2>(sb, cb, w);
      if (!grid_allreduce<2>(w, a.partials, 1, a.gbar, target, a.spin_limit, tot)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) {
        s.rr = tot[0];
        s.it += 1;
        if (!isfinite(tot[0]) || !isfinite(tot[1])) {
          s.done = 3;
        } else {
          const double rn = sqrt(tot[0]);
          if (tot[0] < s.threshold || rn < kDelta * s.rmax) {
            s.ru = 1;
          } else {
            s.rmax = fmax(s.rmax, rn);
            if (!COARSE) {
              const double beta = tot[1] / s.abs_new;
              s.abs_new = tot[1];
              df_split(beta, s.bh, s.bl);
              s.zc = 1.f;
            }
          }
          if (s.it >= s.maxit) s.done = 2;
        }
      }
      __syncthreads();
    }
    if (s.done) break;
    if (COARSE && !s.ru) {
      // z with the coarse correction, r.z and beta
      if (!coarse_z<DIM>(a, target)) {
        fault = true;
        break;
      }
      float sz[1] = {0.f}, cz[1] = {0.f};
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          const float zi = a.cz[i];
          dot2_acc(sz[0], cz[0], a.r[i], zi);
          cz[0] = fmaf(a.rlo[i], zi, cz[0]);
        }
      double w[1] = {0.0}, tot[1];
      block_df_sum<1>(sz, cz, w);
      if (!grid_allreduce<1>(w, a.partials, 6, a.gbar, target, a.spin_limit, tot)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) {
        if (!isfinite(tot[0])) {
          s.done = 3;
        } else {
          const double beta = tot[0] / s.abs_new;
          s.abs_new = tot[0];
          df_split(beta, s.bh, s.bl);
          s.zc = 1.f;
        }
      }
      __syncthreads();
      if (s.done) break;
    }
    if (s.ru) {
      // reliable update: r64 = s b - A64 (x64 + x) and |r64|^2
      double acc[1] = {0.0}, tot[1];
      const double sc = s.bscale;
      for (int row = t0; row < n; row += stride) {
        double y[DIM];
        row_product<DIM, true, true>(a.v, a.A64, a.x64, row, y, a.x, a.xlo);
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          const double ri = a.b[i] * sc - y[c];
          a.r64[i] = ri;
          acc[0] += ri * ri;
        }
      }
      block_sum<1>(acc);
      if (!grid_allreduce<1>(acc, a.partials, 3, a.gbar, target, a.spin_limit, tot)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) {
        s.rr = tot[0];
        s.ru_count += 1;
        if (!isfinite(tot[0]))
          s.done = 3;
        else if (tot[0] < s.threshold)
          s.done = 1;
      }
      __syncthreads();
      if (s.done) break;
      // x64 += x, x = 0, r = r64 as a pair; r.z and r.p give beta and the
      // direction coefficient that restores r.p = 0 (as k_mx_replace)
      double v[2] = {0.0, 0.0}, t2[2];
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          a.x64[i] += (double)a.x[i] + (double)a.xlo[i];
          a.x[i] = 0.f;
          a.xlo[i] = 0.f;
          const double ri = a.r64[i];
          float rh, rl;
          df_split(ri, rh, rl);
          a.r[i] = rh;
          a.rlo[i] = rl;
          if (!COARSE) v[0] += ri * (double)(a.invd[i] * rh);
          v[1] += ri * (double)a.p[i];
        }
      if (COARSE) {
        // the replaced residual's coarse-corrected z (its restriction reads
        // the other rows' new residual: a barrier first)
        target += (unsigned long long)gridDim.x;
        if (!grid_barrier(a.gbar, target, a.spin_limit) || !coarse_z<DIM>(a, target)) {
          fault = true;
          break;
        }
        for (int row = t0; row < n; row += stride)
#pragma unroll
          for (int c = 0; c < DIM; ++c) {
            const int64_t i = (int64_t)row * DIM + c;
            v[0] += a.r64[i] * (double)a.cz[i];
          }
      }
      block_sum<2>(v);
      if (!grid_allreduce<2>(v, a.partials, 4, a.gbar, target, a.spin_limit, t2)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) {
        const double old = s.abs_new;
        s.abs_new = t2[0];
        const double beta = t2[0] / old;
        const double gamma = t2[0] != 0.0 ? t2[1] / t2[0] : 0.0;
        df_split(beta, s.bh, s.bl);
        s.zc = (float)(1.0 - beta * gamma);
        s.rmax = sqrt(s.rr);
        s.ru = 0;
      }
      __syncthreads();
    }
    // p = zc z + beta p with z = M^-1 r
    {
      const float bh = s.bh, bl = s.bl, zc = s.zc;
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          const float pi = a.p[i];
          const float zi = COARSE ? a.cz[i] : __fmul_rn(a.invd[i], a.r[i]);
          a.p[i] = fmaf(bh, pi, fmaf(bl, pi, __fmul_rn(zc, zi)));
        }
      target += (unsigned long long)gridDim.x;
      if (!grid_barrier(a.gbar, target, a.spin_limit)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) s.passes += 1;
    }
  }
  if (fault) {
    if (threadIdx.x == 0) atomicExch(&a.cg->pfault, 1);
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    CgScalars* c = a.cg;
    c->done = s.done;
    c->rr = s.rr;
    c->it = s.it;
    c->abs_new = s.abs_new;
    c->rmax = s.rmax;
    c->ru = s.ru;
    c->ru_count = s.ru_count;
    c->graph_passes = s.passes;
  }
}

// The FP64 solve as one persistent kernel: the recurrence of k_cg_spmv,
// k_cg_update and k_cg_pupdate (Eigen's), with the same row ownership and
// barriers as k_mx_persistent and no reliable updates.
struct PcgFp64 {
  SellView v;
  const double* A;
  const double* invd;
  double *x, *r, *p, *q;
  CgScalars* cg;
  double* partials;          // 3 x gridDim.x
  unsigned long long* gbar;  // barrier arrivals, zero at launch
  long long spin_limit;
};

// Most threads per block: the FP64 product's 64 registers, one block per SM.
constexpr int kPcg64Threads = 1024;

template <int DIM>
__global__ void __launch_bounds__(kPcg64Threads, 1) k_cg_persistent(PcgFp64 a) {
  __shared__ double s_abs_new, s_threshold, s_alpha, s_beta, s_rr;
  __shared__ long long s_it, s_maxit, s_passes;
  __shared__ int s_done;
  if (threadIdx.x == 0) {
    const CgScalars* c = a.cg;
    s_abs_new = c->abs_new;
    s_threshold = c->threshold;
    s_alpha = c->alpha;
    s_beta = c->beta;
    s_rr = c->rr;
    s_it = c->it;
    s_maxit = c->maxit;
    s_passes = 0;
    s_done = c->done;
  }
  __syncthreads();
  const int n = a.v.n;
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long target = 0;
  bool fault = false;
  while (!s_done) {
    // q = A p and p.q; alpha
    {
      double acc[1] = {0.0}, tot[1];
      for (int row = t0; row < n; row += stride) {
        double y[DIM];
        row_product<DIM, false, true>(a.v, a.A, a.p, row, y);
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
          const int64_t i = (int64_t)row * DIM + r;
          a.q[i] = y[r];
          acc[0] += a.p[i] * y[r];
        }
      }
      block_sum<1>(acc);
      if (!grid_allreduce<1>(acc, a.partials, 0, a.gbar, target, a.spin_limit, tot)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) s_alpha = s_abs_new / tot[0];
      __syncthreads();
    }
    // x += alpha p, r -= alpha q, |r|^2 and r.z; convergence, beta
    {
      const double alpha = s_alpha;
      double v[2] = {0.0, 0.0}, tot[2];
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          const double ri = a.r[i] - alpha * a.q[i];
          a.x[i] = a.x[i] + alpha * a.p[i];
          a.r[i] = ri;
          const double zi = a.invd[i] * ri;
          v[0] += ri * ri;
          v[1] += ri * zi;
        }
      block_sum<2>(v);
      if (!grid_allreduce<2>(v, a.partials, 1, a.gbar, target, a.spin_limit, tot)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) {
        s_rr = tot[0];
        if (!isfinite(tot[0]) || !isfinite(tot[1])) {
          s_done = 3;
        } else if (tot[0] < s_threshold) {
          s_done = 1;
        } else {
          s_beta = tot[1] / s_abs_new;
          s_abs_new = tot[1];
          s_it += 1;
          if (s_it >= s_maxit) s_done = 2;
        }
      }
      __syncthreads();
    }
    if (s_done) break;
    // p = M^-1 r + beta p
    {
      const double beta = s_beta;
      for (int row = t0; row < n; row += stride)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const int64_t i = (int64_t)row * DIM + c;
          a.p[i] = a.invd[i] * a.r[i] + beta * a.p[i];
        }
      target += (unsigned long long)gridDim.x;
      if (!grid_barrier(a.gbar, target, a.spin_limit)) {
        fault = true;
        break;
      }
      if (threadIdx.x == 0) s_passes += 1;
    }
  }
  if (fault) {
    if (threadIdx.x == 0) atomicExch(&a.cg->pfault, 1);
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    CgScalars* c = a.cg;
    c->done = s_done;
    c->rr = s_rr;
    c->it = s_it;
    c->abs_new = s_abs_new;
    c->alpha = s_alpha;
    c->beta = s_beta;
    c->graph_passes = s_passes;
  }
}

// Grid of the FP64 row kernels (product, true residual): these are bound by
// the FP64 pipe, and measured faster with several waves of blocks than with
// one resident wave (0.99 against 1.06 ms per product at 101^3).
int fp64_row_grid(lpm_handle* h) { return grid_for((long long)h->n, 256, kMaxRedBlocks); }
SellView sell_view(lpm_handle* h) {
  return SellView{h->d.sell_ptr, h->d.scol, h->d.rowlen, h->d.S32, h->soff16_ok ? h->d.soff16 : nullptr, h->nslots,
                  h->n};
}
int vec_grid(long long m) { return grid_for(m, 256, kMaxRedBlocks); }

// Grid of a CG loop kernel of 256 threads: as many blocks as the device
// holds at once (SMs x resident blocks per SM), so that a launch is one wave
// with no partly filled last wave; never more blocks than `work` items need,
// and at most kMaxRedBlocks (the reduction partials).  The grid-stride loops
// cover any size.
template <typename K>
int resident_grid(lpm_handle* h, K kernel, long long work) {
  if (!h->sms && cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess)
    h->sms = 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  const long long resident = h->sms > 0 ? (long long)h->sms * per_sm : kMaxRedBlocks;
  const long long g = std::min<long long>(resident, (work + 255) / 256);
  return (int)std::max<long long>(1, std::min<long long>(g, kMaxRedBlocks));
}

// Launch shape of a persistent solve, grid 0 where the graph runs instead.
// The rows are spread over every SM: about rows / SMs threads per block (a
// multiple of 32, at least 128, at most `cap`), so a lattice of 80k rows
// takes 148 blocks of 544 threads rather than 105 full ones.  At most one
// resident wave (a cooperative launch refuses more) and no more blocks than
// `slots` partials per block fit in the reduction buffer.  LPM_CG_LOOP_AUTO
// takes it when every row has a thread (and `auto_ok`).
template <typename K>
int persistent_shape(lpm_handle* h, K kernel, int cap, bool auto_ok, int slots, int* threads_out) {
  if (h->mf || h->cg_loop == LPM_CG_LOOP_GRAPH) return 0;
  int coop = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device) != cudaSuccess || !coop) return 0;
  if (!h->sms && cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) return 0;
  const long long per_sm_rows = ((long long)h->n + h->sms - 1) / h->sms;
  const int threads = (int)std::min<long long>(cap, std::max<long long>(128, (per_sm_rows + 31) / 32 * 32));
  *threads_out = threads;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
    return 0;
  const long long resident = (long long)h->sms * per_sm;
  const long long need = ((long long)h->n + threads - 1) / threads;
  if (h->cg_loop == LPM_CG_LOOP_AUTO && (!auto_ok || need > resident)) return 0;
  const long long g = std::min<long long>(std::min(resident, need), (long long)kMaxRedBlocks * 4 / slots);
  return (int)std::max<long long>(1, g);
}

// The FP64 solve's loop as one persistent kernel, when persistent_shape
// allows.  Returns 1 if it ran (its scalars then in h->h_cg), 0 if the graph
// should run, or an error.
int run_persistent_fp64(lpm_handle* h, const SellView& sv, const double* A, double* x, double* r, double* p,
                        double* q, const double* invd) {
  using Fn = void (*)(PcgFp64);
  const Fn fn = h->dim == 3 ? k_cg_persistent<3> : k_cg_persistent<2>;
  int threads = 0;
  const int grid = persistent_shape(h, fn, kPcg64Threads, true, 3, &threads);
  if (grid <= 0) return 0;
  Dev& d = h->d;
  LPM_CUDA(h, cudaMemsetAsync(d.gbar, 0, sizeof(unsigned long long), h->stream));
  PcgFp64 a{sv, A, invd, x, r, p, q, d.cg, d.red.partials, d.gbar, kPcgSpinLimit};
  void* args[] = {&a};
  LPM_CUDA(h, cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(threads), args, 0, h->stream));
  LPM_LAUNCHED(h, "k_cg_persistent");
  LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stats.persistent_solves += 1;
  if (h->h_cg->pfault) {
    h->err = "persistent solve: a grid-barrier wait gave up";
    return LPM_ERR_STATE;
  }
  return 1;
}

cudaEvent_t next_event(lpm_handle* h) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_used++];
}

int build_fp64_graph(lpm_handle* h, const double* A, const double* b, double* x, double* r, double* p, double* q,
                     const double* invd, int GV, int GR, const SellView& sv);

// Runs the CG iteration on the given operator/vectors.  Returns the device
// `done` code through h->h_cg.
template <typename T>
int run_cg(lpm_handle* h, const T* A, const T* b, T* x, T* r, T* p, T* q, const T* invd, double tol, long long maxit) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t ndof = (int64_t)h->n * dim;
  const int GV = vec_grid(ndof), GR = fp64_row_grid(h);
  const SellView sv = sell_view(h);
  k_cg_init<T><<<GV, 256, 0, h->stream>>>(ndof, b, x, r, p, invd, d.cg, tol, maxit, d.red.partials,
                                          d.red.ticket + 2);
  LPM_LAUNCHED(h, "k_cg_init");
  const bool timing = h->timing;
  if constexpr (sizeof(T) == 8) {
    if (!timing) {  // the whole iteration loop as one persistent kernel, or as one graph launch
      const int pst = run_persistent_fp64(h, sv, A, x, r, p, q, invd);
      if (pst < 0) return pst;
      if (pst == 1) return LPM_OK;
      if (!h->fp_exec || h->fp_graph_x != (const void*)x || h->fp_graph_mf != h->mf) {
        const int st = build_fp64_graph(h, A, b, x, r, p, q, invd, GV, GR, sv);
        if (st) return st;
      }
      LPM_CUDA(h, cudaGraphLaunch(h->fp_exec, h->stream));
      LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
      LPM_CUDA(h, cudaStreamSynchronize(h->stream));
      h->stats.kernel_launches += 3 * h->h_cg->graph_passes;
      return LPM_OK;
    }
  }
  // host-launched loop (kernel timing on): events around each product; the
  // host reads the device flag once per batch of iterations
  const size_t ev0 = h->ev_used;
  long long batch = 8;
  for (;;) {
    for (long long k = 0; k < batch; ++k) {
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (timing) {
        e0 = next_event(h);
        e1 = next_event(h);
        if (e0) cudaEventRecord(e0, h->stream);
      }
      if (h->mf) {
        const int st = mf_launch_product(h, sizeof(T) == 4, p, q, nullptr);
        if (st) return st;
      } else {
        if (dim == 3)
          k_cg_spmv<T, 3><<<GR, 256, 0, h->stream>>>(sv, A, p, q, d.cg, d.red.partials, d.red.ticket + 3, nullptr);
        else
          k_cg_spmv<T, 2><<<GR, 256, 0, h->stream>>>(sv, A, p, q, d.cg, d.red.partials, d.red.ticket + 3, nullptr);
        LPM_LAUNCHED(h, "k_cg_spmv");
      }
      if (timing && e1) cudaEventRecord(e1, h->stream);
      k_cg_update<T><<<GV, 256, 0, h->stream>>>(ndof, x, r, p, q, invd, d.cg, d.red.partials, d.red.ticket + 4);
      LPM_LAUNCHED(h, "k_cg_update");
      k_cg_pupdate<T><<<GV, 256, 0, h->stream>>>(ndof, r, invd, p, d.cg, 0);
      LPM_LAUNCHED(h, "k_cg_pupdate");
    }
    LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->h_cg->done) break;
    if (batch < 64) batch *= 2;
  }
  if (timing) {
    // sparse products that did work: one per completed iteration, plus the
    // one of the final iteration when it stopped on the tolerance
    long long real = h->h_cg->it + (h->h_cg->done == 1 && h->h_cg->rhs_norm2 > 0 && h->h_cg->maxit > 0 ? 1 : 0);
    double ms_sum = 0.0;
    long long used = 0;
    for (size_t k = ev0; k + 1 < h->ev_used && used < real; k += 2, ++used) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, h->ev_pool[k], h->ev_pool[k + 1]) == cudaSuccess) ms_sum += ms;
    }
    if (sizeof(T) == 8) {
      h->stats.spmv_launches += used;
      h->stats.spmv_ms += ms_sum;
    } else {
      h->stats.spmv32_launches += used;
      h->stats.spmv32_ms += ms_sum;
    }
    h->ev_used = ev0;
  }
  return LPM_OK;
}

}  // namespace

// Jacobi preconditioner of the assembled operator (FP64, and FP32 on request).
int prepare_invd(lpm_handle* h, bool want32) {
  if (h->mf) return mf_prepare_invd(h, want32);
  Dev& d = h->d;
  if (h->dim == 3)
    k_invd<3><<<grid_for(h->n, 256), 256, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nslots, d.invd64,
                                                          want32 ? d.invd32 : nullptr);
  else
    k_invd<2><<<grid_for(h->n, 256), 256, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nslots, d.invd64,
                                                          want32 ? d.invd32 : nullptr);
  LPM_LAUNCHED(h, "k_invd");
  return LPM_OK;
}


int solve_fp64(lpm_handle* h, double tol, long long maxit, long long* iters, double* relres) {
  Dev& d = h->d;
  if ((!h->mf && (!d.A64 || !d.diag_slot)) || !d.rhs || !d.disp || !d.r64 || !d.p64 || !d.q64 || !d.invd64) {
    h->err = "FP64 solve: work buffers missing";
    return LPM_ERR_STATE;
  }
  if (maxit < 0) maxit = 2LL * h->n * h->dim;  // Eigen's default: twice the number of columns
  int st = prepare_invd(h, false);
  if (st) return st;
  st = run_cg<double>(h, d.A64, d.rhs, d.disp, d.r64, d.p64, d.q64, d.invd64, tol, maxit);
  if (st) return st;
  const CgScalars& c = *h->h_cg;
  const double err = c.rhs_norm2 > 0 ? sqrt(c.rr / c.rhs_norm2) : 0.0;
  if (iters) *iters = c.it;
  if (relres) *relres = err;
  h->stats.cg_iters_total += c.it;
  if (c.done == 3) {
    h->err = "non-finite value in the CG iteration";
    return LPM_ERR_NONFINITE;
  }
  return err <= tol ? LPM_OK : LPM_NOT_CONVERGED;
}

namespace {

// Grids of the mixed solve's loop kernels: one resident wave for the FP32
// product and the vector kernels (resident_grid), several waves for the FP64
// residual (fp64_row_grid).
struct MixedGrids {
  int spmv, update, residual, replace, pupdate;
};

// The FP32 product of a mixed solve: 16-bit column offsets when they fit;
// the operator kept in L2 when its FP32 values take at most kKeepBytes.
using Spmv32Fn = void (*)(SellView, const float*, const float*, float*, CgScalars*, double*, unsigned int*, float*);
constexpr long long kKeepBytes = 64LL << 20;  // half of GB300's L2
template <int DIM>
Spmv32Fn spmv32_fn_dim(bool o16, bool keep) {
  if (keep) return o16 ? k_cg_spmv<float, DIM, true, true> : k_cg_spmv<float, DIM, false, true>;
  return o16 ? k_cg_spmv<float, DIM, true> : k_cg_spmv<float, DIM>;
}
Spmv32Fn spmv32_fn(const lpm_handle* h, const SellView& sv) {
  const bool keep = (long long)h->nslots * h->dim * h->dim * 4 <= kKeepBytes;
  return h->dim == 3 ? spmv32_fn_dim<3>(sv.soff != nullptr, keep) : spmv32_fn_dim<2>(sv.soff != nullptr, keep);
}

// Grid of a vector kernel: one resident wave, but for small systems no more
// than about one block per 1024 entries (at least two per SM), which shortens
// the per-block epilogues and the grid reduction that dominate a kernel of a
// few microseconds (a 112k-particle plate: 3.6 % off the step; at 101^3 the
// resident wave stands).
template <typename K>
int vector_grid(lpm_handle* h, K kernel, long long ndof) {
  const int g = resident_grid(h, kernel, ndof);
  const long long small = std::max<long long>(2LL * h->sms, (ndof + 1023) / 1024);
  return (int)std::max<long long>(1, std::min<long long>(g, small));
}

int mixed_grids(lpm_handle* h, const SellView& sv, MixedGrids* mg) {
  const long long n = h->n, ndof = n * h->dim;
  mg->spmv = h->mf ? 0 : resident_grid(h, spmv32_fn(h, sv), n);
  mg->residual = fp64_row_grid(h);
  mg->update = vector_grid(h, k_mx_update, ndof);
  mg->replace = vector_grid(h, k_mx_replace, ndof);
  mg->pupdate = vector_grid(h, k_mx_pupdate, ndof);
  return LPM_OK;
}

// The persistent solve's kernel for the dimension, column format and
// preconditioner.
using PcgFn = void (*)(PcgMixed);
template <int DIM>
PcgFn pcg_fn_dim(bool o16, bool coarse) {
  if (coarse) return o16 ? k_mx_persistent<DIM, true, true> : k_mx_persistent<DIM, false, true>;
  return o16 ? k_mx_persistent<DIM, true, false> : k_mx_persistent<DIM, false, false>;
}
PcgFn pcg_fn(const SellView& sv, int dim, bool coarse) {
  return dim == 3 ? pcg_fn_dim<3>(sv.soff != nullptr, coarse) : pcg_fn_dim<2>(sv.soff != nullptr, coarse);
}

// Launch shape of the persistent mixed solve (persistent_shape); AUTO takes
// it only when the FP32 operator stays in L2.  The coarse preconditioner
// runs only here, whatever the loop mode.
int pcg_grid(lpm_handle* h, const SellView& sv, int* threads_out, bool coarse) {
  const bool keep = (long long)h->nslots * h->dim * h->dim * 4 <= kKeepBytes;
  const int mode = h->cg_loop;
  if (coarse) h->cg_loop = LPM_CG_LOOP_PERSISTENT;
  const int g = persistent_shape(h, pcg_fn(sv, h->dim, coarse), h->dim == 3 ? kPcgThreads<3> : kPcgThreads<2>,
                                 keep, 7, threads_out);
  h->cg_loop = mode;
  return g;
}

int run_persistent_mixed(lpm_handle* h, const SellView& sv, int grid, int threads, bool coarse) {
  Dev& d = h->d;
  LPM_CUDA(h, cudaMemsetAsync(d.gbar, 0, sizeof(unsigned long long), h->stream));
  PcgMixed a{sv,    d.A32,  d.A64, d.rhs, d.invd32, d.x32, d.x32lo,        d.r32,         d.r32lo,
             d.p32, d.q32,  d.q32lo, d.x64, d.r64,  d.cg,  d.red.partials, d.gbar, kPcgSpinLimit};
  if (coarse) {
    a.cagg = d.cagg;
    a.cmem_ptr = d.cmem_ptr;
    a.cmem = d.cmem;
    a.coff = d.coff;
    a.cfixed = h->last_bc == LPM_BC_ELIMINATE ? d.fixed : nullptr;
    a.cAinv = d.cAinv;
    a.cyc = d.cyc;
    a.cec = d.cec;
    a.cz = d.cz;
    a.cnagg = h->cnagg;
  }
  void* args[] = {&a};
  LPM_CUDA(h, cudaLaunchCooperativeKernel((const void*)pcg_fn(sv, h->dim, coarse), dim3(grid), dim3(threads), args,
                                          0, h->stream));
  LPM_LAUNCHED(h, "k_mx_persistent");
  return LPM_OK;
}

// The mixed solve's iteration loop as one graph:
//   while (loop_cond) { spmv; update; if (ru_cond) { residual; replace } pupdate }
// update sets ru_cond (a reliable update is due) and pupdate sets
// loop_cond (the solve goes on), so a whole solve is one graph launch with
// no host round trip and no launch of an idle reliable-update kernel.
int build_mixed_graph(lpm_handle* h, const SellView& sv, const MixedGrids& mg) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t ndof = (int64_t)h->n * dim;
  if (h->mx_exec) cudaGraphExecDestroy(h->mx_exec);
  if (h->mx_graph) cudaGraphDestroy(h->mx_graph);
  h->mx_exec = nullptr;
  h->mx_graph = nullptr;
  cudaGraph_t g;
  LPM_CUDA(h, cudaGraphCreate(&g, 0));
  h->mx_graph = g;
  cudaGraphConditionalHandle loop_cond, ru_cond;
  LPM_CUDA(h, cudaGraphConditionalHandleCreate(&loop_cond, g, 1u, cudaGraphCondAssignDefault));
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = loop_cond;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t wnode;
  LPM_CUDA(h, cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  LPM_CUDA(h, cudaGraphConditionalHandleCreate(&ru_cond, body, 0u, cudaGraphCondAssignDefault));
  cudaGraphNode_t n_spmv, n_upd, n_if, n_res, n_rep, n_pup;
  cudaError_t e;
  const Spmv32Fn spmv = h->mf ? nullptr : spmv32_fn(h, sv);
  if (h->mf) {
    const int st = mf_graph_product(h, body, nullptr, true, d.p32, d.q32, d.q32lo, &n_spmv);
    if (st) return st;
  } else {
    LPM_CUDA(h, add_kernel(&n_spmv, body, nullptr, spmv, mg.spmv, 256, sv, (const float*)d.A32, (const float*)d.p32,
                           d.q32, d.cg, d.red.partials, d.red.ticket + 3, d.q32lo));
  }
  LPM_CUDA(h, add_kernel(&n_upd, body, &n_spmv, k_mx_update, mg.update, 256, ndof, d.x32, d.x32lo, d.r32, d.r32lo,
                         (const float*)d.p32, (const float*)d.q32, (const float*)d.q32lo, (const float*)d.invd32,
                         d.cg, d.red.partials, d.red.ticket + 4, ru_cond));
  cudaGraphNodeParams ip = {};
  ip.type = cudaGraphNodeTypeConditional;
  ip.conditional.handle = ru_cond;
  ip.conditional.type = cudaGraphCondTypeIf;
  ip.conditional.size = 1;
  LPM_CUDA(h, cudaGraphAddNode(&n_if, body, &n_upd, nullptr, 1, &ip));
  cudaGraph_t ifb = ip.conditional.phGraph_out[0];
  if (h->mf) {
    const int st = mf_graph_residual(h, ifb, nullptr, &n_res);
    if (st) return st;
    e = cudaSuccess;
  } else if (dim == 3)
    e = add_kernel(&n_res, ifb, nullptr, k_mx_residual<3>, mg.residual, 256, sv, (const double*)d.A64, (const double*)d.x64,
                   (const float*)d.x32, (const float*)d.x32lo, (const double*)d.rhs, d.r64, d.cg, d.red.partials,
                   d.red.ticket + 6);
  else
    e = add_kernel(&n_res, ifb, nullptr, k_mx_residual<2>, mg.residual, 256, sv, (const double*)d.A64, (const double*)d.x64,
                   (const float*)d.x32, (const float*)d.x32lo, (const double*)d.rhs, d.r64, d.cg, d.red.partials,
                   d.red.ticket + 6);
  LPM_CUDA(h, e);
  LPM_CUDA(h, add_kernel(&n_rep, ifb, &n_res, k_mx_replace, mg.replace, 256, ndof, (const double*)d.r64, d.r32, d.r32lo,
                         d.x32, d.x32lo, d.x64, (const float*)d.p32, (const float*)d.invd32, d.cg, d.red.partials,
                         d.red.ticket + 7));
  LPM_CUDA(h, add_kernel(&n_pup, body, &n_if, k_mx_pupdate, mg.pupdate, 256, ndof, (const float*)d.r32,
                         (const float*)d.invd32, d.p32, d.cg, loop_cond));
  LPM_CUDA(h, cudaGraphInstantiate(&h->mx_exec, g, 0));
  h->mx_graph_spmv = (const void*)spmv;
  h->mx_graph_mf = h->mf;
  return LPM_OK;
}

// The FP64 solve's iteration loop as one graph:
//   while (loop_cond) { spmv; update; pupdate }
// with pupdate setting loop_cond once update has decided (converged,
// iteration cap or non-finite).
int build_fp64_graph(lpm_handle* h, const double* A, const double* b, double* x, double* r, double* p, double* q,
                     const double* invd, int GV, int GR, const SellView& sv) {
  Dev& d = h->d;
  const int64_t ndof = (int64_t)h->n * h->dim;
  if (h->fp_exec) cudaGraphExecDestroy(h->fp_exec);
  if (h->fp_graph) cudaGraphDestroy(h->fp_graph);
  h->fp_exec = nullptr;
  h->fp_graph = nullptr;
  h->fp_graph_x = nullptr;
  cudaGraph_t g;
  LPM_CUDA(h, cudaGraphCreate(&g, 0));
  h->fp_graph = g;
  cudaGraphConditionalHandle loop_cond;
  LPM_CUDA(h, cudaGraphConditionalHandleCreate(&loop_cond, g, 1u, cudaGraphCondAssignDefault));
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = loop_cond;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t wnode, n_spmv, n_upd, n_pup;
  LPM_CUDA(h, cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  if (h->mf) {
    const int st = mf_graph_product(h, body, nullptr, false, p, q, nullptr, &n_spmv);
    if (st) return st;
  } else if (h->dim == 3) {
    LPM_CUDA(h, add_kernel(&n_spmv, body, nullptr, k_cg_spmv<double, 3>, GR, 256, sv, A, (const double*)p, q, d.cg,
                           d.red.partials, d.red.ticket + 3, (float*)nullptr));
  } else {
    LPM_CUDA(h, add_kernel(&n_spmv, body, nullptr, k_cg_spmv<double, 2>, GR, 256, sv, A, (const double*)p, q, d.cg,
                           d.red.partials, d.red.ticket + 3, (float*)nullptr));
  }
  LPM_CUDA(h, add_kernel(&n_upd, body, &n_spmv, k_cg_update<double>, GV, 256, ndof, x, r, (const double*)p,
                         (const double*)q, invd, d.cg, d.red.partials, d.red.ticket + 4));
  LPM_CUDA(h, add_kernel(&n_pup, body, &n_upd, k_cg_pupdate<double>, GV, 256, ndof, (const double*)r, invd, p, d.cg,
                         loop_cond));
  LPM_CUDA(h, cudaGraphInstantiate(&h->fp_exec, g, 0));
  h->fp_graph_x = x;
  h->fp_graph_mf = h->mf;
  return LPM_OK;
}

}  // namespace

namespace {

// FP32 work vectors, allocated on the first mixed solve (or product).
int mixed_buffers(lpm_handle* h) {
  Dev& d = h->d;
  const int64_t ndof = (int64_t)h->n * h->dim;
  if (!d.b32) {
    float** vecs[9] = {&d.b32, &d.x32, &d.r32, &d.p32, &d.q32, &d.invd32, &d.r32lo, &d.q32lo, &d.x32lo};
    for (float** v : vecs) {
      *v = (float*)dev_alloc(h, sizeof(float) * (size_t)ndof);
      if (!*v) return LPM_ERR_NOMEM;
    }
  }
  return LPM_OK;
}

}  // namespace

// y = A' v with the operator the solves use (assembled or matrix-free), in
// FP64 or as the FP32 product of the mixed solve (its double-float output
// summed in FP64).  v and y are host vectors of n*dim.
int apply_operator(lpm_handle* h, int precision, const double* v, double* y) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t ndof = (int64_t)h->n * dim;
  LPM_CUDA(h, cudaMemsetAsync(d.cg, 0, sizeof(CgScalars), h->stream));
  if (precision == LPM_PREC_FP64) {
    const SellView sv = sell_view(h);
    LPM_CUDA(h, cudaMemcpyAsync(d.p64, v, sizeof(double) * ndof, cudaMemcpyHostToDevice, h->stream));
    if (h->mf) {
      const int st = mf_launch_product(h, false, d.p64, d.q64, nullptr, true);
      if (st) return st;
    } else {
      const int GR = fp64_row_grid(h);
      if (dim == 3)
        k_cg_spmv<double, 3><<<GR, 256, 0, h->stream>>>(sv, d.A64, d.p64, d.q64, d.cg, d.red.partials,
                                                        d.red.ticket + 3, nullptr);
      else
        k_cg_spmv<double, 2><<<GR, 256, 0, h->stream>>>(sv, d.A64, d.p64, d.q64, d.cg, d.red.partials,
                                                        d.red.ticket + 3, nullptr);
      LPM_LAUNCHED(h, "k_cg_spmv");
    }
    LPM_CUDA(h, cudaMemcpyAsync(y, d.q64, sizeof(double) * ndof, cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    return LPM_OK;
  }
  int st = mixed_buffers(h);
  if (st) return st;
  if (!h->mf && !h->a32_valid) {
    st = convert_A32(h);
    if (st) return st;
  }
  // the view after the conversion: it carries the row sums and column
  // offsets that convert_A32 creates on the first FP32 use
  const SellView sv = sell_view(h);
  std::vector<float> v32((size_t)ndof), hi((size_t)ndof), lo((size_t)ndof);
  for (int64_t q = 0; q < ndof; ++q) v32[(size_t)q] = (float)v[q];
  LPM_CUDA(h, cudaMemcpyAsync(d.p32, v32.data(), sizeof(float) * ndof, cudaMemcpyHostToDevice, h->stream));
  if (h->mf) {
    st = mf_launch_product(h, true, d.p32, d.q32, d.q32lo, true);
    if (st) return st;
  } else {
    MixedGrids mg;
    st = mixed_grids(h, sv, &mg);
    if (st) return st;
    spmv32_fn(h, sv)<<<mg.spmv, 256, 0, h->stream>>>(sv, d.A32, d.p32, d.q32, d.cg, d.red.partials, d.red.ticket + 3,
                                                     d.q32lo);
    LPM_LAUNCHED(h, "k_cg_spmv");
  }
  LPM_CUDA(h, cudaMemcpyAsync(hi.data(), d.q32, sizeof(float) * ndof, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(lo.data(), d.q32lo, sizeof(float) * ndof, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int64_t q = 0; q < ndof; ++q) y[q] = (double)hi[(size_t)q] + (double)lo[(size_t)q];
  return LPM_OK;
}

int solve_mixed(lpm_handle* h, double tol, long long maxit, long long* iters, double* relres) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t ndof = (int64_t)h->n * dim;
  if (maxit < 0) maxit = 2LL * ndof;
  {
    const int st0 = mixed_buffers(h);
    if (st0) return st0;
  }
  if (!h->mf && !h->a32_valid) {
    const int st0 = convert_A32(h);
    if (st0) return st0;
  }
  if ((!h->mf && (!d.A32 || !d.S32)) || !d.x32 || !d.r32 || !d.p32 || !d.q32 || !d.invd32 || !d.r32lo || !d.q32lo ||
      !d.x32lo || !d.x64 || !d.r64 || !d.rhs || !d.disp) {
    h->err = "mixed solve: work buffers missing";
    return LPM_ERR_STATE;
  }
  const int GV = vec_grid(ndof);
  const SellView sv = sell_view(h);
  MixedGrids mg;
  int st = mixed_grids(h, sv, &mg);
  if (st) return st;
  st = prepare_invd(h, true);
  if (st) return st;
  LPM_CUDA(h, cudaMemsetAsync(d.x64, 0, sizeof(double) * ndof, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(&d.cg->bmax_bits, 0, sizeof(unsigned long long), h->stream));
  k_absmax<<<GV, 256, 0, h->stream>>>(ndof, d.rhs, d.cg);
  LPM_LAUNCHED(h, "k_absmax");
  k_mx_init<<<GV, 256, 0, h->stream>>>(ndof, d.rhs, d.x32, d.x32lo, d.r32, d.r32lo, d.p32, d.invd32, d.cg, tol, maxit,
                                       d.red.partials, d.red.ticket + 2);
  LPM_LAUNCHED(h, "k_mx_init");
  const bool timing = h->timing;
  const size_t ev0 = h->ev_used;
  const bool coarse = h->precond == LPM_PRECOND_COARSE;
  if (coarse) {
    if (h->mf || h->tangent != LPM_TANGENT_SYMMETRIC) {
      h->err = "coarse preconditioner: needs the assembled symmetric tangent";
      return LPM_ERR_STATE;
    }
    if (!h->coarse_valid) {
      st = coarse_assemble(h);
      if (st) return st;
    }
  }
  int pthreads = 0;
  const int pgrid = timing && !coarse ? 0 : pcg_grid(h, sv, &pthreads, coarse);
  if (coarse && pgrid <= 0) {
    h->err = "coarse preconditioner: the persistent solve cannot be launched on this device";
    return LPM_ERR_STATE;
  }
  if (pgrid > 0) {
    // the whole iteration loop as one persistent kernel
    st = run_persistent_mixed(h, sv, pgrid, pthreads, coarse);
    if (st) return st;
  } else if (!timing) {
    // the whole iteration loop as one graph launch
    if (!h->mx_exec || h->mx_graph_mf != h->mf || (!h->mf && h->mx_graph_spmv != (const void*)spmv32_fn(h, sv))) {
      st = build_mixed_graph(h, sv, mg);
      if (st) return st;
    }
    LPM_CUDA(h, cudaGraphLaunch(h->mx_exec, h->stream));
  }
  // with kernel timing on, the same kernels launched one by one from the
  // host, with events around each sparse product; the host reads the device
  // flag once per batch of iterations
  const Spmv32Fn spmv32 = spmv32_fn(h, sv);
  long long batch = 8;
  for (; timing && pgrid <= 0;) {
    for (long long k = 0; k < batch; ++k) {
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (timing) {
        e0 = next_event(h);
        e1 = next_event(h);
        if (e0) cudaEventRecord(e0, h->stream);
      }
      if (h->mf) {
        st = mf_launch_product(h, true, d.p32, d.q32, d.q32lo);
        if (st) return st;
      } else {
        spmv32<<<mg.spmv, 256, 0, h->stream>>>(sv, d.A32, d.p32, d.q32, d.cg, d.red.partials, d.red.ticket + 3,
                                               d.q32lo);
        LPM_LAUNCHED(h, "k_cg_spmv");
      }
      if (timing && e1) cudaEventRecord(e1, h->stream);
      k_mx_update<<<mg.update, 256, 0, h->stream>>>(ndof, d.x32, d.x32lo, d.r32, d.r32lo, d.p32, d.q32, d.q32lo, d.invd32,
                                                    d.cg, d.red.partials, d.red.ticket + 4, 0);
      LPM_LAUNCHED(h, "k_mx_update");
      if (h->mf) {
        st = mf_launch_residual(h);
        if (st) return st;
      } else {
        if (dim == 3)
          k_mx_residual<3><<<mg.residual, 256, 0, h->stream>>>(sv, d.A64, d.x64, d.x32, d.x32lo, d.rhs, d.r64, d.cg,
                                                               d.red.partials, d.red.ticket + 6);
        else
          k_mx_residual<2><<<mg.residual, 256, 0, h->stream>>>(sv, d.A64, d.x64, d.x32, d.x32lo, d.rhs, d.r64, d.cg,
                                                               d.red.partials, d.red.ticket + 6);
        LPM_LAUNCHED(h, "k_mx_residual");
      }
      k_mx_replace<<<mg.replace, 256, 0, h->stream>>>(ndof, d.r64, d.r32, d.r32lo, d.x32, d.x32lo, d.x64, d.p32, d.invd32,
                                                      d.cg, d.red.partials, d.red.ticket + 7);
      LPM_LAUNCHED(h, "k_mx_replace");
      k_mx_pupdate<<<mg.pupdate, 256, 0, h->stream>>>(ndof, d.r32, d.invd32, d.p32, d.cg, 0);
      LPM_LAUNCHED(h, "k_mx_pupdate");
    }
    LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->h_cg->done) break;
    if (batch < 64) batch *= 2;
  }
  // fold what the iterations since the last replacement added
  k_mx_fold<<<GV, 256, 0, h->stream>>>(ndof, d.x32, d.x32lo, d.x64, d.cg);
  LPM_LAUNCHED(h, "k_mx_fold");
  LPM_CUDA(h, cudaMemcpyAsync(d.disp, d.x64, sizeof(double) * ndof, cudaMemcpyDeviceToDevice, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  const CgScalars& c = *h->h_cg;
  if (pgrid > 0) {
    h->stats.persistent_solves += 1;
    if (c.pfault) {
      h->err = "persistent solve: a grid-barrier wait gave up";
      return LPM_ERR_STATE;
    }
  } else if (!timing) {
    h->stats.kernel_launches += 3 * c.graph_passes + 2 * c.ru_count;
  }
  if (timing) {
    double ms_sum = 0.0;
    long long used = 0;
    for (size_t k = ev0; k + 1 < h->ev_used && used < c.it; k += 2, ++used) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, h->ev_pool[k], h->ev_pool[k + 1]) == cudaSuccess) ms_sum += ms;
    }
    h->stats.spmv32_launches += used;
    h->stats.spmv32_ms += ms_sum;
    h->ev_used = ev0;
  }
  const double rel = c.rhs_norm2 > 0 ? sqrt(c.rr / c.rhs_norm2) : 0.0;
  h->stats.cg_iters_total += c.it;
  h->stats.refine_sweeps += c.ru_count;
  if (iters) *iters = c.it;
  if (relres) *relres = rel;
  if (c.done == 3) {
    h->err = "non-finite value in the mixed-precision CG iteration";
    return LPM_ERR_NONFINITE;
  }
  // converged only on the FP64 residual (done == 1 is set by the FP64 check
  // or by a zero right-hand side)
  return c.done == 1 ? LPM_OK : LPM_NOT_CONVERGED;
}

}  // namespace lpm
