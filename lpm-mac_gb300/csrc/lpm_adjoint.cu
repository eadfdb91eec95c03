// Adjoint of a converged load step, and device-resident step checkpoints.
//
// Response J = a . x + c . Pin(x; Kn, Tv) for given weights a, c on the
// particle DOFs (a gauge displacement, a reaction sum over a constrained
// group, ...).  At a converged step the free DOFs are in equilibrium,
// Pex_f = Pin_f(x), so with H = dPin/dx
//     dJ/dtheta = (c - lambda) . dPin/dtheta,   H_ff lambda_f = (a + H^T c)_f,
// lambda = 0 on the constrained DOFs.  The bond constants theta = (Kn_b,
// Tv_b) of every directed bond enter Pin only through the bond forces
// f_b = w_b (2 Kn_b dLe_b + 2 Tv_b D_i^l), D_i^l = sum over i's layer-l bonds
// of dLe, so that with mu = c - lambda
//     dJ/dKn_b = w_b dLe_b cs_b . (mu_i - mu_j),
//     dJ/dTv_b = w_b D_i^l cs_b . (mu_i - mu_j).
//
// H is applied matrix-free: H v is the forward-mode derivative of the force
// pass (particle.h:163-215, particle_elastic.h:38-50) with the bond damage
// held fixed,
//     d dLe_b = cs_b . (v_i - v_j),   d cs_b = ((v_i - v_j) - cs_b d dLe_b) / dis_b,
//     d f_b   = w_b (2 Kn_b d dLe_b + 2 Tv_b d D_i^l),
//     d Pin_i = sum_b d cs_b F_b + cs_b (d f_b + d f_opp(b)) / 2,   F_b = (f_b + f_opp(b)) / 2.
// It is the exact Jacobian of Pin, unlike the analytical tangent of
// derivative.h, which leaves out the change of the bond directions.  When
// every bond is either intact or broken, Pin is the gradient of the lattice
// energy  sum_b Kn_b dLe_b^2 / 2 + sum_(i,l) Tv_i (D_i^l)^2 / 2, so H is
// symmetric and H_ff lambda = g is solved by Jacobi-PCG on the exact H with
// its exact diagonal as the preconditioner.  Partially damaged bonds break
// the symmetry; the adjoint then refuses the state.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "lpm_cgvec.cuh"
#include "lpm_device.cuh"

namespace lpm {
namespace {

__device__ __forceinline__ void load_v(const double* __restrict__ v, int dim, int i, double (&o)[3]) {
  o[0] = v[(int64_t)dim * i];
  o[1] = v[(int64_t)dim * i + 1];
  o[2] = dim == 3 ? v[(int64_t)dim * i + 2] : 0.0;
}

// H v runs over a sliced copy of the bond data made once per adjoint
// (k_jac_slots, k_jac_prep): slices of 32 consecutive particles, bond k of
// particle i at slot jbase[i/32] + 32 k + i%32, so that one thread per
// particle reads its bonds with the 32 threads of a warp on consecutive
// slots.  Each slot holds what the product needs at the fixed state: the
// partner, the slot of the opposite bond, the layer, the direction cosines
// and the folded constants 2 w Kn, 2 w Tv and F/dis (F the mean bond force).
// Broken bonds and padding slots hold zeros (padding points at the particle
// itself), so every slot is processed without a branch.
__global__ void k_jac_slots(int n, const int64_t* __restrict__ bptr, const int64_t* __restrict__ jbase,
                            int* __restrict__ slot_of) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s0 = jbase[i / 32] + (i % 32);
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) slot_of[b] = (int)(s0 + 32 * (b - bptr[i]));
}

__global__ void k_jac_prep(int n, const int64_t* __restrict__ bptr, const int64_t* __restrict__ jbase,
                           const int* __restrict__ slot_of, const int* __restrict__ bp2,
                           const int* __restrict__ blayer, const int* __restrict__ opp, const double* __restrict__ cs,
                           const double* __restrict__ dis, const double* __restrict__ bdamage,
                           const double* __restrict__ bforce, const double* __restrict__ Kn,
                           const double* __restrict__ Tv, int* __restrict__ jp2, int* __restrict__ jopp,
                           int* __restrict__ jlayer, double* __restrict__ jc, double* __restrict__ jk,
                           double* __restrict__ jt, double* __restrict__ jf, int64_t nslot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sl = i / 32;
  const int len = (int)((jbase[sl + 1] - jbase[sl]) / 32);
  const int64_t s0 = jbase[sl] + (i % 32);
  const int nb = (int)(bptr[i + 1] - bptr[i]);
  for (int k = 0; k < len; ++k) {
    const int64_t s = s0 + 32 * (int64_t)k;
    if (k < nb && !is_broken(bdamage[bptr[i] + k])) {
      const int64_t b = bptr[i] + k;
      const double w = 1.0 - bdamage[b];
      jp2[s] = bp2[b];
      jopp[s] = slot_of[opp[b]];
      jlayer[s] = blayer[b];
      jc[s] = cs[3 * b];
      jc[nslot + s] = cs[3 * b + 1];
      jc[2 * nslot + s] = cs[3 * b + 2];
      jk[s] = 2.0 * w * Kn[b];
      jt[s] = 2.0 * w * Tv[b];
      jf[s] = 0.5 * (bforce[b] + bforce[opp[b]]) / dis[b];
    } else {
      jp2[s] = i;
      jopp[s] = (int)s;
      jlayer[s] = 0;
      jc[s] = jc[nslot + s] = jc[2 * nslot + s] = 0.0;
      jk[s] = jt[s] = jf[s] = 0.0;
    }
  }
}

struct JacView {
  const int64_t* __restrict__ jbase;
  const int* __restrict__ jp2;
  const int* __restrict__ jopp;
  const int* __restrict__ jlayer;
  const double* __restrict__ jc;
  const double* __restrict__ jk;
  const double* __restrict__ jt;
  const double* __restrict__ jf;
  double* __restrict__ jd;  // d dLe, then d f, per slot
  int64_t nslot;
};

// Pass 1 of H v: d dLe per slot and the per-layer sums d D_i^l, then d f.
// With dlp (per slot) the plastic stretches move too: d dLe -= d dLp; with
// dfk (per slot) the bond constants too: d f += dfk.
__global__ void k_jvp_bonds(int n, int dim, JacView J, const double* __restrict__ v, const double* __restrict__ dlp,
                            const double* __restrict__ dfk, const CgScalars* cg) {
  if (cg && cg->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sl = i / 32;
  const int len = (int)((J.jbase[sl + 1] - J.jbase[sl]) / 32);
  const int64_t s0 = J.jbase[sl] + (i % 32);
  double vi[3];
  load_v(v, dim, i, vi);
  double dD0 = 0.0, dD1 = 0.0;
  for (int k = 0; k < len; ++k) {
    const int64_t s = s0 + 32 * (int64_t)k;
    double vj[3];
    load_v(v, dim, J.jp2[s], vj);
    double dd = J.jc[s] * (vi[0] - vj[0]) + J.jc[J.nslot + s] * (vi[1] - vj[1]) +
                J.jc[2 * J.nslot + s] * (vi[2] - vj[2]);
    if (dlp) dd -= dlp[s];
    J.jd[s] = dd;
    if (J.jlayer[s] == 0)
      dD0 += dd;
    else
      dD1 += dd;
  }
  for (int k = 0; k < len; ++k) {
    const int64_t s = s0 + 32 * (int64_t)k;
    J.jd[s] = J.jk[s] * J.jd[s] + J.jt[s] * (J.jlayer[s] == 0 ? dD0 : dD1) + (dfk ? dfk[s] : 0.0);
  }
}

// Pass 2 of H v: y_i = d Pin_i (zero on constrained DOFs when `mask` is
// given).  With `cg` set it also forms p.q over the grid and, in the last
// block, alpha = (r.z) / (p.q) for the CG update.
__global__ void __launch_bounds__(256) k_jvp_particles(int n, int dim, JacView J, const double* __restrict__ v,
                                                       const int* __restrict__ mask, double* __restrict__ y,
                                                       CgScalars* cg, double* partials, unsigned int* ticket) {
  if (cg && cg->done) return;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int sl = i / 32;
    const int len = (int)((J.jbase[sl + 1] - J.jbase[sl]) / 32);
    const int64_t s0 = J.jbase[sl] + (i % 32);
    double vi[3];
    load_v(v, dim, i, vi);
    double P0 = 0.0, P1 = 0.0, P2 = 0.0;
    for (int k = 0; k < len; ++k) {
      const int64_t s = s0 + 32 * (int64_t)k;
      double vj[3];
      load_v(v, dim, J.jp2[s], vj);
      const double c0 = J.jc[s], c1 = J.jc[J.nslot + s], c2 = J.jc[2 * J.nslot + s];
      const double u0 = vi[0] - vj[0], u1 = vi[1] - vj[1], u2 = vi[2] - vj[2];
      const double dd = c0 * u0 + c1 * u1 + c2 * u2;
      const double rf = J.jf[s];
      const double dF = 0.5 * (J.jd[s] + J.jd[J.jopp[s]]);
      P0 += (u0 - c0 * dd) * rf + c0 * dF;
      P1 += (u1 - c1 * dd) * rf + c1 * dF;
      P2 += (u2 - c2 * dd) * rf + c2 * dF;
    }
    const double P[3] = {P0, P1, P2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (k >= dim) break;
      const double yk = (mask && mask[3 * i + k]) ? 0.0 : P[k];
      y[(int64_t)dim * i + k] = yk;
      acc += vi[k] * yk;
    }
  }
  if (!cg) return;
  double w[1] = {acc}, tot[1];
  if (grid_sum<1>(w, partials, ticket, tot) && threadIdx.x == 0) cg->alpha = cg->abs_new / tot[0];
}

// Exact diagonal of H (one DOF of particle i moved, its partners' layer sums
// included) as the Jacobi preconditioner; 1 on constrained DOFs.
__global__ void k_jac_invdiag(int n, int dim, const int64_t* __restrict__ bptr, const int* __restrict__ blayer,
                              const int* __restrict__ opp, const double* __restrict__ cs,
                              const double* __restrict__ dis, const double* __restrict__ bdamage,
                              const double* __restrict__ bforce, const double* __restrict__ Kn,
                              const double* __restrict__ Tv, const int* __restrict__ mask,
                              double* __restrict__ invd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b0 = bptr[i], b1 = bptr[i + 1];
  for (int k = 0; k < dim; ++k) {
    double S0 = 0.0, S1 = 0.0;  // d D_i^l for a unit move of DOF k of particle i
    for (int64_t b = b0; b < b1; ++b) {
      if (is_broken(bdamage[b])) continue;
      if (blayer[b] == 0)
        S0 += cs[3 * b + k];
      else
        S1 += cs[3 * b + k];
    }
    double h = 0.0;
    for (int64_t b = b0; b < b1; ++b) {
      if (is_broken(bdamage[b])) continue;
      const double ck = cs[3 * b + k];
      const int o = opp[b];
      const double F = 0.5 * (bforce[b] + bforce[o]);
      const double df = (1.0 - bdamage[b]) * (2.0 * Kn[b] * ck + 2.0 * Tv[b] * (blayer[b] == 0 ? S0 : S1));
      // the partner's sum moves only through this bond: d dLe = ck
      const double dfo = (1.0 - bdamage[o]) * (2.0 * Kn[o] * ck + 2.0 * Tv[o] * ck);
      h += (1.0 - ck * ck) / dis[b] * F + ck * 0.5 * (df + dfo);
    }
    invd[(int64_t)dim * i + k] = (mask[3 * i + k] || h == 0.0) ? 1.0 : 1.0 / h;
  }
}

// g = (a + y) on free DOFs, 0 on constrained ones.
__global__ void k_adj_rhs(int n, int dim, const double* __restrict__ a, const double* __restrict__ y,
                          const int* __restrict__ mask, double* __restrict__ g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * dim) return;
  const int i = t / dim, k = t % dim;
  g[t] = mask[3 * i + k] ? 0.0 : (a ? a[t] : 0.0) + (y ? y[t] : 0.0);
}

// mu = c - lambda (lambda is zero on constrained DOFs).
__global__ void k_adj_mu(int64_t m, const double* __restrict__ c, const double* __restrict__ lam,
                         double* __restrict__ mu) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  mu[t] = (c ? c[t] : 0.0) - lam[t];
}

// dJ/dKn_b and dJ/dTv_b from mu, per directed bond (stored bond order).
__global__ void k_param_grad(int n, int dim, const int64_t* __restrict__ bptr, const int* __restrict__ bp2,
                             const int* __restrict__ blayer, const double* __restrict__ cs,
                             const double* __restrict__ dLe, const double* __restrict__ dle_tot,
                             const double* __restrict__ bdamage, const double* __restrict__ mu, int accumulate,
                             double* __restrict__ gKn, double* __restrict__ gTv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double mi[3];
  load_v(mu, dim, i, mi);
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    double gk = 0.0, gt = 0.0;
    if (!is_broken(bdamage[b])) {
      double mj[3];
      load_v(mu, dim, bp2[b], mj);
      const double cd = cs[3 * b] * (mi[0] - mj[0]) + cs[3 * b + 1] * (mi[1] - mj[1]) + cs[3 * b + 2] * (mi[2] - mj[2]);
      const double w = 1.0 - bdamage[b];
      gk = w * dLe[b] * cd;
      gt = w * dle_tot[NL * i + blayer[b]] * cd;
    }
    gKn[b] = accumulate ? gKn[b] + gk : gk;
    gTv[b] = accumulate ? gTv[b] + gt : gt;
  }
}

// 1 in flag when some bond is partially damaged (EPS < d < 1 - EPS) or
// broken while its opposite bond is not.
__global__ void k_partial_damage(int64_t nb, const double* __restrict__ bdamage, const int* __restrict__ opp,
                                 int* flag) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const double d = bdamage[b];
  if ((d > EPS && d < 1.0 - EPS) || is_broken(d) != is_broken(bdamage[opp[b]])) atomicOr(flag, 1);
}

// ------------------------------------------------ tangent-linear sensitivity
// d dLp in the sliced bond layout (broken bonds 0; padding slots stay 0).
__global__ void k_dlp_slots(int n, const int64_t* __restrict__ bptr, const int* __restrict__ slot_of,
                            const double* __restrict__ bdamage, const double* __restrict__ dlp,
                            double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) out[slot_of[b]] = is_broken(bdamage[b]) ? 0.0 : dlp[b];
}

// The bond force's change from changes of the bond constants, in the
// sliced layout: d f_b = w_b (2 dKn_b dLe_b + 2 dTv_b D_i^l) (broken bonds 0).
__global__ void k_dfk_slots(int n, const int64_t* __restrict__ bptr, const int* __restrict__ slot_of,
                            const int* __restrict__ blayer, const double* __restrict__ bdamage,
                            const double* __restrict__ dLe, const double* __restrict__ dle_tot,
                            const double* __restrict__ dkn, const double* __restrict__ dtv, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    const double w = 1.0 - bdamage[b];
    out[slot_of[b]] = is_broken(bdamage[b]) ? 0.0
                                            : 2.0 * w * (dkn[b] * dLe[b] + dtv[b] * dle_tot[NL * i + blayer[b]]);
  }
}

// The bond force's change from changes of the bond constants (optional)
// and of the bond damage, in the sliced layout, for the softening law:
//   d f_b = w_b (2 dKn_b dLe_b + 2 dTv_b D_i^l) - d d_b (2 Kn_b dLe_b + 2 Tv_b D_i^l)
// (f_b = (1 - d_b)(2 Kn dLe + 2 Tv D); broken bonds 0).
__global__ void k_dfs_slots(int n, const int64_t* __restrict__ bptr, const int* __restrict__ slot_of,
                            const int* __restrict__ blayer, const double* __restrict__ bdamage,
                            const double* __restrict__ dLe, const double* __restrict__ dle_tot,
                            const double* __restrict__ Kn, const double* __restrict__ Tv,
                            const double* __restrict__ dkn, const double* __restrict__ dtv,
                            const double* __restrict__ dd, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    if (is_broken(bdamage[b])) {
      out[slot_of[b]] = 0.0;
      continue;
    }
    const double D = dle_tot[NL * i + blayer[b]];
    double v = -dd[b] * 2.0 * (Kn[b] * dLe[b] + Tv[b] * D);
    if (dkn) v += 2.0 * (1.0 - bdamage[b]) * (dkn[b] * dLe[b] + dtv[b] * D);
    out[slot_of[b]] = v;
  }
}

// Tangent of the softening law's damage update (k_softening_damage), run
// just before it on the same state: kappa = max(kappa, s) with
// s = (dis - dis0)/dis0, d = D(kappa, s_c) when that raises d, where
//   D = alpha/(alpha - 1) - alpha s_c / ((alpha - 1) kappa)   (s_c < kappa < alpha s_c),
// 0 below s_c and 1 from alpha s_c.  With dx the equilibrium's change:
//   d s = c_b . (dx_i - dx_j) / dis0,  d kappa = d s where s sets kappa,
//   d d = dD/dkappa d kappa + dD/ds_c d s_c where d rises,
// otherwise both keep their previous tangents.
__global__ void k_soft_tangent(int n, int dim, const int64_t* __restrict__ bptr, const int* __restrict__ bp2,
                               const int* __restrict__ ptype, int undamaged, const double* __restrict__ pp, int np,
                               const double* __restrict__ dis, const double* __restrict__ dis0,
                               const double* __restrict__ cs, const double* __restrict__ bcrit,
                               const double* __restrict__ bkappa, const double* __restrict__ bdamage,
                               const double* __restrict__ dx, const double* __restrict__ dsc,
                               double* __restrict__ dkappa, double* __restrict__ dd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || ptype[i] == undamaged) return;
  const double alpha = pp[(int64_t)i * np];
  double ui[3];
  load_v(dx, dim, i, ui);
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    if (is_broken(bdamage[b])) continue;  // stays broken: its tangents no longer matter
    const double s = (dis[b] - dis0[b]) / dis0[b];
    double uj[3];
    load_v(dx, dim, bp2[b], uj);
    const double ds = (cs[3 * b] * (ui[0] - uj[0]) + cs[3 * b + 1] * (ui[1] - uj[1]) +
                       cs[3 * b + 2] * (ui[2] - uj[2])) / dis0[b];
    const double kold = bkappa[b];
    const double k = fmax(kold, s);
    if (s > kold) dkappa[b] = ds;
    const double sc = bcrit[b];
    double d = 0.0;
    if (k >= alpha * sc)
      d = 1.0;
    else if (k > sc)
      d = 1.0 - (sc / k) * (alpha * sc - k) / ((alpha - 1.0) * sc);
    if (d > bdamage[b]) {
      if (k >= alpha * sc || !(k > sc)) {
        dd[b] = 0.0;
      } else {
        const double a1 = alpha / (alpha - 1.0);
        dd[b] = a1 * sc / (k * k) * dkappa[b] - a1 / k * (dsc ? dsc[b] : 0.0);
      }
    }
  }
}

// g = -q on the free DOFs, 0 on the constrained ones.
__global__ void k_tg_rhs(int n, int dim, const double* __restrict__ q, const int* __restrict__ mask,
                         double* __restrict__ g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * dim) return;
  const int i = t / dim, k = t % dim;
  g[t] = mask[3 * i + k] ? 0.0 : -q[t];
}

// The change of the particle stress (particle.h:217-240,
// sigma_pq = sum_b (1/2 V_m) dis_b F_b c_p c_q with F_b the mean bond force)
// for a change v of the positions, with d F_b from pass 1 of the Jacobian
// product (J.jd, which includes any change of dLp):
//   d dis = c . u,  d c = (u - c d dis) / dis,  u = v_i - v_j.
__global__ void k_jvp_stress(int n, int dim, JacView J, const double* __restrict__ v, const int64_t* __restrict__ bptr,
                             const int* __restrict__ bp2, const int* __restrict__ slot_of,
                             const int* __restrict__ opp, const double* __restrict__ bforce,
                             const double* __restrict__ cs, const double* __restrict__ dis,
                             const int* __restrict__ nbonds, double pvol, int nneighbors, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double hv = 0.5 / (pvol * nbonds[i] / nneighbors);
  double vi[3];
  load_v(v, dim, i, vi);
  double ds[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    double vj[3];
    load_v(v, dim, bp2[b], vj);
    const double c[3] = {cs[3 * b], cs[3 * b + 1], cs[3 * b + 2]};
    const double u[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
    const double dd = c[0] * u[0] + c[1] * u[1] + c[2] * u[2];
    const double dc[3] = {(u[0] - c[0] * dd) / dis[b], (u[1] - c[1] * dd) / dis[b], (u[2] - c[2] * dd) / dis[b]};
    const int s = slot_of[b];
    const double F = 0.5 * (bforce[b] + bforce[opp[b]]);
    const double dF = 0.5 * (J.jd[s] + J.jd[J.jopp[s]]);
    const double sf = hv * dis[b] * F, dsf = hv * (dd * F + dis[b] * dF);
    const int p[6] = {0, 1, 2, 1, 0, 0}, q[6] = {0, 1, 2, 2, 2, 1};  // xx yy zz yz xz xy
#pragma unroll
    for (int k = 0; k < 6; ++k)
      ds[k] += dsf * c[p[k]] * c[q[k]] + sf * (dc[p[k]] * c[q[k]] + c[p[k]] * dc[q[k]]);
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) out[6 * (int64_t)i + k] = ds[k];
}

// The radial return of ParticleJ2Plasticity (particle_j2plasticity.h:78-140,
// the primal in lpm_laws.cu) differentiated along one direction: inputs the
// primal stress, state (before the update) and parameters, and the tangents
// of stress, state, parameters and positions; advances the tangents of the
// state (alpha, back stress) and of each bond's dLp.  Elastic particles
// (no yield) leave their tangents unchanged.
__global__ void k_j2_tangent(int n, int dim, int np, int ns, const double* __restrict__ pp,
                             const double* __restrict__ dpp, const double* __restrict__ state,
                             double* __restrict__ tsv, const double* __restrict__ stress,
                             const double* __restrict__ dstress, const int64_t* __restrict__ bptr,
                             const int* __restrict__ bp2, const double* __restrict__ dis,
                             const double* __restrict__ cs, const double* __restrict__ tx, double* __restrict__ tdlp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* P = pp + (int64_t)i * np;
  const double* dP = dpp + (int64_t)i * np;
  const double* sv = state + (int64_t)i * ns;
  double* t = tsv + (int64_t)i * ns;
  const double E = P[0], mu = P[1], sigmay = P[2], xi = P[3], H = P[4];
  const double dE = dP[0], dmu = dP[1], dsigmay = dP[2], dxi = dP[3], dH = dP[4];
  double st[6], dst[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    st[j] = stress[6 * (int64_t)i + j];
    dst[j] = dstress[6 * (int64_t)i + j];
  }
  const double sm = (st[0] + st[1] + st[2]) / 3.0, dsm = (dst[0] + dst[1] + dst[2]) / 3.0;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    st[j] -= sm;
    dst[j] -= dsm;
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    st[j] -= sv[j + 1];
    dst[j] -= t[j + 1];
  }
  double s2 = 0.0, ds2 = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double w = j < 3 ? 1.0 : 2.0;
    s2 += w * st[j] * st[j];
    ds2 += w * st[j] * dst[j];
  }
  const double seq = sqrt(1.5 * s2);
  const double dseq = seq > 0.0 ? 1.5 * ds2 / seq : 0.0;
  const double yf = seq - (sigmay + (1.0 - xi) * H * sv[0]);
  if (!(yf > 0.0)) return;
  const double G = E / 2 / (1 + mu), dG = dE / 2 / (1 + mu) - E * dmu / (2 * (1 + mu) * (1 + mu));
  const double den = 3 * G + H;
  const double dyf = dseq - (dsigmay - dxi * H * sv[0] + (1.0 - xi) * (dH * sv[0] + H * t[0]));
  const double dl = yf / den, ddl = dyf / den - yf * (3 * dG + dH) / (den * den);
  t[0] += ddl;
  double dp[6] = {0, 0, 0, 0, 0, 0}, ddp[6] = {0, 0, 0, 0, 0, 0};
  if (fabs(seq) > EPS) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      dp[j] = dl * 1.5 * st[j] / seq;
      ddp[j] = 1.5 * (ddl * st[j] / seq + dl * (dst[j] / seq - st[j] * dseq / (seq * seq)));
      t[j + 1] += 2. / 3. * (dxi * H * dp[j] + xi * dH * dp[j] + xi * H * ddp[j]);
    }
  }
  double vi[3];
  load_v(tx, dim, i, vi);
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    double vj[3];
    load_v(tx, dim, bp2[b], vj);
    const double c0 = cs[3 * b], c1 = cs[3 * b + 1], c2 = cs[3 * b + 2];
    const double u0 = vi[0] - vj[0], u1 = vi[1] - vj[1], u2 = vi[2] - vj[2];
    const double dd = c0 * u0 + c1 * u1 + c2 * u2;
    const double e0 = (u0 - c0 * dd) / dis[b], e1 = (u1 - c1 * dd) / dis[b], e2 = (u2 - c2 * dd) / dis[b];
    const double q = dp[0] * c0 * c0 + dp[1] * c1 * c1 + dp[2] * c2 * c2 + 2 * dp[3] * c1 * c2 +
                     2 * dp[4] * c0 * c2 + 2 * dp[5] * c0 * c1;
    const double dq = ddp[0] * c0 * c0 + ddp[1] * c1 * c1 + ddp[2] * c2 * c2 + 2 * ddp[3] * c1 * c2 +
                      2 * ddp[4] * c0 * c2 + 2 * ddp[5] * c0 * c1 + dp[0] * 2 * c0 * e0 + dp[1] * 2 * c1 * e1 +
                      dp[2] * 2 * c2 * e2 + 2 * dp[3] * (e1 * c2 + c1 * e2) + 2 * dp[4] * (e0 * c2 + c0 * e2) +
                      2 * dp[5] * (e0 * c1 + c0 * e1);
    tdlp[b] += dd * q + dis[b] * dq;
  }
}

}  // namespace

// Work buffers of the adjoint, allocated on first use (gradients zeroed).
int adjoint_buffers(lpm_handle* h) {
  Dev& d = h->d;
  const size_t m = (size_t)h->n * h->dim;
  double** vecs[9] = {&d.adj_g, &d.adj_lam, &d.adj_r, &d.adj_p, &d.adj_q, &d.adj_invd, &d.adj_mu, &d.adj_a, &d.adj_c};
  for (double** v : vecs)
    if (!*v) {
      *v = (double*)dev_alloc(h, sizeof(double) * std::max<size_t>(m, 1));
      if (!*v) return LPM_ERR_NOMEM;
    }
  double** bvecs[2] = {&d.adj_gkn, &d.adj_gtv};
  for (double** v : bvecs)
    if (!*v) {
      *v = (double*)zeros_dev(h, sizeof(double) * std::max<size_t>((size_t)h->nb, 1));
      if (!*v) return LPM_ERR_NOMEM;
    }
  if (!d.adj_flag) {
    d.adj_flag = (int*)dev_alloc(h, sizeof(int));
    if (!d.adj_flag) return LPM_ERR_NOMEM;
  }
  return LPM_OK;
}

// Sliced bond data of the Jacobian at the current state (layout once per
// handle, values on every call).
static int jacobian_prepare(lpm_handle* h) {
  Dev& d = h->d;
  const int n = h->n;
  if (!d.jbase) {
    std::vector<int64_t> bptr((size_t)n + 1);
    LPM_CUDA(h, cudaMemcpy(bptr.data(), d.bptr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost));
    const int nsl = (n + 31) / 32;
    std::vector<int64_t> jb((size_t)nsl + 1, 0);
    for (int sl = 0; sl < nsl; ++sl) {
      int64_t mx = 0;
      for (int i = sl * 32; i < std::min(n, sl * 32 + 32); ++i) mx = std::max(mx, bptr[(size_t)i + 1] - bptr[(size_t)i]);
      jb[(size_t)sl + 1] = jb[(size_t)sl] + 32 * mx;
    }
    h->jslots = jb[(size_t)nsl];
    if (h->jslots >= ((int64_t)1 << 31)) {
      h->err = "adjoint: 2^31 or more bond slots";
      return LPM_ERR_ARG;
    }
    d.jbase = (int64_t*)dev_alloc(h, sizeof(int64_t) * jb.size());
    d.jslot_of = (int*)dev_alloc(h, sizeof(int) * std::max<size_t>((size_t)h->nb, 1));
    const size_t S = (size_t)std::max<int64_t>(h->jslots, 1);
    d.jp2 = (int*)dev_alloc(h, sizeof(int) * S);
    d.jopp = (int*)dev_alloc(h, sizeof(int) * S);
    d.jlayer = (int*)dev_alloc(h, sizeof(int) * S);
    d.jc = (double*)dev_alloc(h, sizeof(double) * 3 * S);
    d.jk = (double*)dev_alloc(h, sizeof(double) * S);
    d.jt = (double*)dev_alloc(h, sizeof(double) * S);
    d.jf = (double*)dev_alloc(h, sizeof(double) * S);
    d.jd = (double*)dev_alloc(h, sizeof(double) * S);
    if (!d.jbase || !d.jslot_of || !d.jp2 || !d.jopp || !d.jlayer || !d.jc || !d.jk || !d.jt || !d.jf || !d.jd)
      return LPM_ERR_NOMEM;
    LPM_CUDA(h, cudaMemcpy(d.jbase, jb.data(), sizeof(int64_t) * jb.size(), cudaMemcpyHostToDevice));
    k_jac_slots<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.jbase, d.jslot_of);
    LPM_LAUNCHED(h, "k_jac_slots");
  }
  k_jac_prep<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.jbase, d.jslot_of, d.bp2, d.blayer, d.opp, d.cs,
                                                      d.dis, d.bdamage, d.bforce, d.Kn, d.Tv, d.jp2, d.jopp,
                                                      d.jlayer, d.jc, d.jk, d.jt, d.jf, h->jslots);
  LPM_LAUNCHED(h, "k_jac_prep");
  return LPM_OK;
}

// y = H v (mask: zero the constrained rows); with cg, p.q and alpha too;
// with dlp (sliced layout) the derivative along a change of dLp as well.
static int apply_jacobian(lpm_handle* h, const double* v, double* y, bool masked, CgScalars* cg,
                          const double* dlp = nullptr, const double* dfk = nullptr) {
  Dev& d = h->d;
  const JacView J{d.jbase, d.jp2, d.jopp, d.jlayer, d.jc, d.jk, d.jt, d.jf, d.jd, h->jslots};
  k_jvp_bonds<<<grid_for(h->n, 128), 128, 0, h->stream>>>(h->n, h->dim, J, v, dlp, dfk, cg);
  LPM_LAUNCHED(h, "k_jvp_bonds");
  k_jvp_particles<<<grid_for(h->n, 256, kMaxRedBlocks), 256, 0, h->stream>>>(
      h->n, h->dim, J, v, masked ? d.mask : nullptr, y, cg, d.red.partials, d.red.ticket + 8);
  LPM_LAUNCHED(h, "k_jvp_particles");
  return LPM_OK;
}

int adjoint_apply(lpm_handle* h, const double* v_dev, double* y_dev) {
  int st = adjoint_buffers(h);
  if (st) return st;
  st = jacobian_prepare(h);
  if (st) return st;
  return apply_jacobian(h, v_dev, y_dev, false, nullptr);
}

// H_ff x = g (g zero on the constrained DOFs, x zero there too) by
// Jacobi-PCG on the exact Jacobian at the prepared state, with its exact
// diagonal as the preconditioner; the relative residual in *relres.
static int jacobian_cg(lpm_handle* h, const double* g, double* x, double tol, long long maxit, long long* iters,
                       double* relres) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t m = (int64_t)h->n * dim;
  k_jac_invdiag<<<grid_for(h->n, 128), 128, 0, h->stream>>>(h->n, dim, d.bptr, d.blayer, d.opp, d.cs, d.dis,
                                                            d.bdamage, d.bforce, d.Kn, d.Tv, d.mask, d.adj_invd);
  LPM_LAUNCHED(h, "k_jac_invdiag");
  if (maxit < 0) maxit = 2LL * m;
  const int GV = grid_for(m, 256, kMaxRedBlocks);
  k_cg_init<double><<<GV, 256, 0, h->stream>>>(m, g, x, d.adj_r, d.adj_p, d.adj_invd, d.cg, tol, maxit,
                                               d.red.partials, d.red.ticket + 2);
  LPM_LAUNCHED(h, "k_cg_init");
  long long batch = 8;
  for (;;) {
    for (long long k = 0; k < batch; ++k) {
      int st = apply_jacobian(h, d.adj_p, d.adj_q, true, d.cg);
      if (st) return st;
      k_cg_update<double><<<GV, 256, 0, h->stream>>>(m, x, d.adj_r, d.adj_p, d.adj_q, d.adj_invd, d.cg,
                                                     d.red.partials, d.red.ticket + 4);
      LPM_LAUNCHED(h, "k_cg_update");
      k_cg_pupdate<double><<<GV, 256, 0, h->stream>>>(m, d.adj_r, d.adj_invd, d.adj_p, d.cg, 0);
      LPM_LAUNCHED(h, "k_cg_pupdate");
    }
    LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->h_cg->done) break;
    if (batch < 64) batch *= 2;
  }
  const CgScalars c = *h->h_cg;
  if (iters) *iters = c.it;
  *relres = c.rhs_norm2 > 0 ? sqrt(c.rr / c.rhs_norm2) : 0.0;
  if (c.done == 3) {
    h->err = "adjoint: non-finite value in the CG iteration";
    return LPM_ERR_NONFINITE;
  }
  return LPM_OK;
}

// BiCGSTAB (van der Vorst, SIAM J. Sci. Stat. Comput. 13 (1992)) for the
// non-symmetric H_ff of a partially damaged state, right-preconditioned by
// H's exact diagonal; the vector work of one iteration in three kernels.
// Its scalars stay on the device: the dot kernels' last blocks update them
// and the vector kernels read them, so an iteration needs no host round
// trip; the host reads them once per batch of iterations.
struct BicgScalars {
  double bnorm, tol2b;  // |b| and tol^2 |b|^2
  double rho, rho_new, alpha, omega, rr;
  long long it, maxit;
  int done;  // 0 running, 1 converged, 2 iteration cap or breakdown, 3 non-finite
};

enum BicgStage { kBicgInit, kBicgAlpha, kBicgOmega, kBicgRes };

// Two dot products (a.b, c.e) folded over the grid; the last block updates
// the scalars for the stage.  Nothing once the solve has ended.
template <int STAGE>
__global__ void k_bicg_dot(int64_t m, const double* __restrict__ a, const double* __restrict__ b,
                           const double* __restrict__ c, const double* __restrict__ e, double* partials,
                           unsigned int* ticket, BicgScalars* S, double tol, long long maxit) {
  if (STAGE != kBicgInit && S->done) return;
  double v[2] = {0.0, 0.0};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
    v[0] += a[t] * b[t];
    v[1] += c[t] * e[t];
  }
  double tot[2];
  if (!(grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0)) return;
  if (STAGE == kBicgInit) {  // (g.g, rh.r) with r = rh = g
    S->bnorm = sqrt(tot[0]);
    S->tol2b = tol * tol * tot[0];
    S->rho = S->alpha = S->omega = 1.0;
    S->rho_new = tot[1];
    S->rr = tot[0];
    S->it = 0;
    S->maxit = maxit;
    S->done = !isfinite(tot[0]) ? 3 : (tot[0] == 0.0 || maxit <= 0) ? (tot[0] == 0.0 ? 1 : 2) : 0;
  } else if (STAGE == kBicgAlpha) {  // rh.v
    S->alpha = S->rho_new / tot[0];
  } else if (STAGE == kBicgOmega) {  // (t.s, t.t)
    S->omega = tot[1] > 0.0 ? tot[0] / tot[1] : 0.0;
  } else {  // (r.r, rh.r)
    S->rho = S->rho_new;
    S->rho_new = tot[1];
    S->rr = tot[0];
    S->it += 1;
    if (!isfinite(tot[0]))
      S->done = 3;
    else if (tot[0] <= S->tol2b)
      S->done = 1;
    else if (S->it >= S->maxit || S->rho_new == 0.0 || S->omega == 0.0)
      S->done = 2;
  }
}

// p = r + beta (p - omega v), phat = M p, with beta from the scalars (0 in
// the first iteration)
__global__ void k_bicg_p(int64_t m, const double* __restrict__ r, const double* __restrict__ v,
                         const double* __restrict__ invd, const BicgScalars* S, double* __restrict__ p,
                         double* __restrict__ phat) {
  if (S->done) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const double beta = S->it == 0 ? 0.0 : (S->rho_new / S->rho) * (S->alpha / S->omega);
  const double pt = r[t] + beta * (p[t] - S->omega * v[t]);
  p[t] = pt;
  phat[t] = invd[t] * pt;
}

// s = r - alpha v, shat = M s
__global__ void k_bicg_s(int64_t m, const double* __restrict__ r, const double* __restrict__ v,
                         const double* __restrict__ invd, const BicgScalars* S, double* __restrict__ sv,
                         double* __restrict__ shat) {
  if (S->done) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const double st = r[t] - S->alpha * v[t];
  sv[t] = st;
  shat[t] = invd[t] * st;
}

// x += alpha phat + omega shat, r = s - omega t
__global__ void k_bicg_xr(int64_t m, const double* __restrict__ phat, const double* __restrict__ shat,
                          const double* __restrict__ sv, const double* __restrict__ tv, const BicgScalars* S,
                          double* __restrict__ x, double* __restrict__ r) {
  if (S->done) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  x[t] += S->alpha * phat[t] + S->omega * shat[t];
  r[t] = sv[t] - S->omega * tv[t];
}

// H_ff x = g (g zero on the constrained DOFs) by right-preconditioned
// BiCGSTAB on the exact Jacobian at the prepared state.  The iterations are
// enqueued in batches; the scalars stop the vector updates on the device as
// soon as the solve has ended, so the few products left in a batch change
// nothing.
static int jacobian_bicgstab(lpm_handle* h, const double* g, double* x, double tol, long long maxit,
                             long long* iters, double* relres) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t m = (int64_t)h->n * dim;
  if (!d.tg_bicg) {
    d.tg_bicg = (double*)dev_alloc(h, sizeof(double) * (size_t)(7 * m) + sizeof(BicgScalars));
    if (!d.tg_bicg) return LPM_ERR_NOMEM;
  }
  double *r = d.tg_bicg, *rh = r + m, *p = rh + m, *ph = p + m, *v = ph + m, *sv = v + m, *sh = sv + m;
  BicgScalars* S = reinterpret_cast<BicgScalars*>(sh + m);
  double* tv = d.adj_q;  // t = H shat
  k_jac_invdiag<<<grid_for(h->n, 128), 128, 0, h->stream>>>(h->n, dim, d.bptr, d.blayer, d.opp, d.cs, d.dis,
                                                            d.bdamage, d.bforce, d.Kn, d.Tv, d.mask, d.adj_invd);
  LPM_LAUNCHED(h, "k_jac_invdiag");
  if (maxit < 0) maxit = 2LL * m;
  // right preconditioner: the exact diagonal, plus the coarse correction of
  // the assembled symmetric tangent when the user chose it
  // (lpm_set_preconditioner): the exact Jacobian differs from that tangent
  // by the bond directions' change, so its coarse space serves here too
  const bool coarse = coarse_usable(h);
  const int GV = grid_for(m, 256, kMaxRedBlocks), T = 256, GE = grid_for(m, T);
  LPM_CUDA(h, cudaMemsetAsync(x, 0, sizeof(double) * m, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(p, 0, sizeof(double) * m, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(v, 0, sizeof(double) * m, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(r, g, sizeof(double) * m, cudaMemcpyDeviceToDevice, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(rh, g, sizeof(double) * m, cudaMemcpyDeviceToDevice, h->stream));
  unsigned int* ticket = d.red.ticket + 9;
  k_bicg_dot<kBicgInit><<<GV, 256, 0, h->stream>>>(m, g, g, rh, r, d.red.partials, ticket, S, tol, maxit);
  LPM_LAUNCHED(h, "k_bicg_dot");
  BicgScalars hs{};
  long long batch = 4;
  for (;;) {
    for (long long k = 0; k < batch; ++k) {
      k_bicg_p<<<GE, T, 0, h->stream>>>(m, r, v, d.adj_invd, S, p, ph);
      LPM_LAUNCHED(h, "k_bicg_p");
      if (coarse) {
        const int st = coarse_apply64(h, p, d.adj_invd, ph);
        if (st) return st;
      }
      int st = apply_jacobian(h, ph, v, true, nullptr);
      if (st) return st;
      k_bicg_dot<kBicgAlpha><<<GV, 256, 0, h->stream>>>(m, rh, v, rh, v, d.red.partials, ticket, S, tol, maxit);
      LPM_LAUNCHED(h, "k_bicg_dot");
      k_bicg_s<<<GE, T, 0, h->stream>>>(m, r, v, d.adj_invd, S, sv, sh);
      LPM_LAUNCHED(h, "k_bicg_s");
      if (coarse) {
        st = coarse_apply64(h, sv, d.adj_invd, sh);
        if (st) return st;
      }
      st = apply_jacobian(h, sh, tv, true, nullptr);
      if (st) return st;
      k_bicg_dot<kBicgOmega><<<GV, 256, 0, h->stream>>>(m, tv, sv, tv, tv, d.red.partials, ticket, S, tol, maxit);
      LPM_LAUNCHED(h, "k_bicg_dot");
      k_bicg_xr<<<GE, T, 0, h->stream>>>(m, ph, sh, sv, tv, S, x, r);
      LPM_LAUNCHED(h, "k_bicg_xr");
      k_bicg_dot<kBicgRes><<<GV, 256, 0, h->stream>>>(m, r, r, rh, r, d.red.partials, ticket, S, tol, maxit);
      LPM_LAUNCHED(h, "k_bicg_dot");
    }
    LPM_CUDA(h, cudaMemcpyAsync(&hs, S, sizeof(BicgScalars), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hs.done) break;
    if (batch < 32) batch *= 2;
  }
  if (hs.done == 3) {
    h->err = hs.it == 0 ? "tangent: non-finite right-hand side" : "tangent: non-finite value in BiCGSTAB";
    return LPM_ERR_NONFINITE;
  }
  if (iters) *iters = hs.it;
  *relres = hs.bnorm > 0.0 ? sqrt(hs.rr) / hs.bnorm : 0.0;
  return LPM_OK;
}

// One round of the softening law's tangent (called after the round's
// Newton, before its damage update): for each direction, the equilibrium's
// change H_ff dx_f = -(dPin/d(d) . dd + dPin/d(Kn, Tv) . d(Kn, Tv))_f with
// H the exact, non-symmetric Jacobian of the partially damaged state, then
// dPin there; and the tangent of the damage update that follows.
static int tangent_soft_round(lpm_handle* h) {
  Dev& d = h->d;
  const int dim = h->dim, n = h->n;
  const int64_t m = (int64_t)n * dim;
  const size_t B = (size_t)std::max<int64_t>(h->nb, 1);
  int st = jacobian_prepare(h);
  if (st) return st;
  if (!d.tg_jdk) {
    d.tg_jdl = (double*)zeros_dev(h, sizeof(double) * (size_t)std::max<int64_t>(h->jslots, 1));
    d.tg_jdk = (double*)zeros_dev(h, sizeof(double) * (size_t)std::max<int64_t>(h->jslots, 1));
    if (!d.tg_jdl || !d.tg_jdk) return LPM_ERR_NOMEM;
  }
  LPM_CUDA(h, cudaMemsetAsync(d.adj_a, 0, sizeof(double) * m, h->stream));
  for (int k = 0; k < h->tg_ndir; ++k) {
    double* tx = d.tg_x + (size_t)k * m;
    double* tpin = d.tg_pin + (size_t)k * m;
    k_dfs_slots<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.jslot_of, d.blayer, d.bdamage, d.dLe,
                                                        d.dle_tot, d.Kn, d.Tv, h->tg_bond ? d.tg_dkn + k * B : nullptr,
                                                        h->tg_bond ? d.tg_dtv + k * B : nullptr, d.tg_dd + k * B,
                                                        d.tg_jdk);
    LPM_LAUNCHED(h, "k_dfs_slots");
    st = apply_jacobian(h, d.adj_a, d.adj_c, false, nullptr, nullptr, d.tg_jdk);
    if (st) return st;
    k_tg_rhs<<<grid_for(m, 256), 256, 0, h->stream>>>(n, dim, d.adj_c, d.mask, d.adj_g);
    LPM_LAUNCHED(h, "k_tg_rhs");
    long long it = 0;
    double rr = 0.0;
    st = jacobian_bicgstab(h, d.adj_g, tx, h->tg_tol, -1, &it, &rr);
    if (st) return st;
    h->stats.tangent_cg_iters += it;
    if (!(rr <= h->tg_tol)) {
      h->err = "tangent: the equilibrium change did not converge";
      return LPM_NOT_CONVERGED;
    }
    st = apply_jacobian(h, tx, tpin, false, nullptr, nullptr, d.tg_jdk);
    if (st) return st;
  }
  return LPM_OK;
}

// The damage update's tangent (before k_softening_damage changes the state).
int tangent_soft_damage(lpm_handle* h) {
  Dev& d = h->d;
  const int n = h->n;
  const int64_t m = (int64_t)n * h->dim;
  const size_t B = (size_t)std::max<int64_t>(h->nb, 1);
  for (int k = 0; k < h->tg_ndir; ++k) {
    k_soft_tangent<<<grid_for(n, 128), 128, 0, h->stream>>>(
        n, h->dim, d.bptr, d.bp2, d.ptype, h->undamaged, d.pp, h->law_np, d.dis, d.dis0, d.cs, d.bcrit, d.bkappa,
        d.bdamage, d.tg_x + (size_t)k * m, d.tg_dsc + k * B, d.tg_dkappa + k * B, d.tg_dd + k * B);
    LPM_LAUNCHED(h, "k_soft_tangent");
  }
  return LPM_OK;
}

// 1 in the adjoint flag (and LPM_ERR_STATE) when some bond is partially or
// one-sidedly damaged: the Jacobian is then not symmetric.
static int check_symmetric_damage(lpm_handle* h) {
  Dev& d = h->d;
  LPM_CUDA(h, cudaMemsetAsync(d.adj_flag, 0, sizeof(int), h->stream));
  k_partial_damage<<<grid_for(h->nb, 256), 256, 0, h->stream>>>(h->nb, d.bdamage, d.opp, d.adj_flag);
  LPM_LAUNCHED(h, "k_partial_damage");
  int flag = 0;
  LPM_CUDA(h, cudaMemcpyAsync(&flag, d.adj_flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (flag) {
    h->err = "adjoint: partially or one-sidedly damaged bonds make the Jacobian non-symmetric";
    return LPM_ERR_STATE;
  }
  return LPM_OK;
}

int adjoint_step(lpm_handle* h, const double* a_dev, const double* c_dev, double tol, long long maxit, int accumulate,
                 double* gKn_dev, double* gTv_dev, long long* iters, double* relres) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t m = (int64_t)h->n * dim;
  int st = adjoint_buffers(h);
  if (st) return st;
  // the symmetric solve needs every bond intact or broken
  st = check_symmetric_damage(h);
  if (st) return st;
  st = jacobian_prepare(h);
  if (st) return st;
  // g = a + H c on the free DOFs
  const int TV = 256;
  if (c_dev) {
    st = apply_jacobian(h, c_dev, d.adj_q, false, nullptr);
    if (st) return st;
  }
  k_adj_rhs<<<grid_for(m, TV), TV, 0, h->stream>>>(h->n, dim, a_dev, c_dev ? d.adj_q : nullptr, d.mask, d.adj_g);
  LPM_LAUNCHED(h, "k_adj_rhs");
  // H_ff lambda = g by Jacobi-PCG on the exact Jacobian
  double err = 0.0;
  st = jacobian_cg(h, d.adj_g, d.adj_lam, tol, maxit, iters, &err);
  if (st) return st;
  if (relres) *relres = err;
  // parameter gradients
  k_adj_mu<<<grid_for(m, TV), TV, 0, h->stream>>>(m, c_dev, d.adj_lam, d.adj_mu);
  LPM_LAUNCHED(h, "k_adj_mu");
  k_param_grad<<<grid_for(h->n, 128), 128, 0, h->stream>>>(h->n, dim, d.bptr, d.bp2, d.blayer, d.cs, d.dLe,
                                                           d.dle_tot, d.bdamage, d.adj_mu, accumulate, gKn_dev,
                                                           gTv_dev);
  LPM_LAUNCHED(h, "k_param_grad");
  return err <= tol ? LPM_OK : LPM_NOT_CONVERGED;
}

// ------------------------------------------------ tangent-linear sensitivity
int tangent_begin(lpm_handle* h, int ndir, const double* dparams_host, double tol) {
  Dev& d = h->d;
  if (ndir < 0 || !(tol > 0.0)) {
    h->err = "tangent: bad arguments";
    return LPM_ERR_ARG;
  }
  const bool soft = h->law == LPM_LAW_SOFTENING, hcf = h->law == LPM_LAW_FATIGUE_HCF;
  if (ndir > 0 && ((h->law != 2 && !soft && !hcf) || !d.pp || !d.state || (soft && (!d.bcrit || !d.bkappa)) ||
                   (hcf && !d.nl_ptr))) {
    h->err = "tangent: the J2 law (2), the HCF law with nonlocal neighbours (3) or the softening law (4) is required";
    return LPM_ERR_STATE;
  }
  if (ndir > 0 && !soft && !dparams_host) {
    h->err = "tangent: NULL parameter directions";
    return LPM_ERR_ARG;
  }

  if (ndir > h->tg_cap) {  // buffers for ndir directions (smaller ones stay owned by the handle)
    const size_t N = (size_t)h->n, B = (size_t)std::max<int64_t>(h->nb, 1), m = N * h->dim;
    d.tg_dlp = (double*)dev_alloc(h, sizeof(double) * ndir * B);
    d.tg_sv = (double*)dev_alloc(h, sizeof(double) * ndir * N * h->nstate);
    d.tg_x = (double*)dev_alloc(h, sizeof(double) * ndir * m);
    d.tg_pin = (double*)dev_alloc(h, sizeof(double) * ndir * m);
    d.tg_dp = (double*)dev_alloc(h, sizeof(double) * ndir * N * h->law_np);
    d.tg_stress = (double*)dev_alloc(h, sizeof(double) * 6 * N);
    d.tg_dkn = (double*)dev_alloc(h, sizeof(double) * ndir * B);
    d.tg_dtv = (double*)dev_alloc(h, sizeof(double) * ndir * B);
    d.tg_dd = (double*)dev_alloc(h, sizeof(double) * ndir * B);
    d.tg_dkappa = (double*)dev_alloc(h, sizeof(double) * ndir * B);
    d.tg_dsc = (double*)dev_alloc(h, sizeof(double) * ndir * B);
    d.tg_dD = (double*)dev_alloc(h, sizeof(double) * ndir * N);
    d.tg_ddot = (double*)dev_alloc(h, sizeof(double) * ndir * N);
    d.tg_dnl = (double*)dev_alloc(h, sizeof(double) * ndir * N);
    if (!d.tg_dlp || !d.tg_sv || !d.tg_x || !d.tg_pin || !d.tg_dp || !d.tg_stress || !d.tg_dkn || !d.tg_dtv ||
        !d.tg_dd || !d.tg_dkappa || !d.tg_dsc || !d.tg_dD || !d.tg_ddot || !d.tg_dnl)
      return LPM_ERR_NOMEM;
    h->tg_cap = ndir;
  }
  h->tg_ndir = 0;
  if (ndir == 0) return LPM_OK;
  const size_t N = (size_t)h->n, B = (size_t)std::max<int64_t>(h->nb, 1), m = N * h->dim;
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dlp, 0, sizeof(double) * ndir * B, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_sv, 0, sizeof(double) * ndir * N * h->nstate, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_x, 0, sizeof(double) * ndir * m, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_pin, 0, sizeof(double) * ndir * m, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dkn, 0, sizeof(double) * ndir * B, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dtv, 0, sizeof(double) * ndir * B, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dd, 0, sizeof(double) * ndir * B, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dkappa, 0, sizeof(double) * ndir * B, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dsc, 0, sizeof(double) * ndir * B, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dD, 0, sizeof(double) * ndir * N, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_ddot, 0, sizeof(double) * ndir * N, h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.tg_dnl, 0, sizeof(double) * ndir * N, h->stream));
  if (dparams_host)
    LPM_CUDA(h, cudaMemcpyAsync(d.tg_dp, dparams_host, sizeof(double) * ndir * N * h->law_np, cudaMemcpyHostToDevice,
                                h->stream));
  else
    LPM_CUDA(h, cudaMemsetAsync(d.tg_dp, 0, sizeof(double) * ndir * N * h->law_np, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->tg_ndir = ndir;
  h->tg_tol = tol;
  h->tg_bond = false;
  return LPM_OK;
}

int tangent_bond_constants(lpm_handle* h, int dir, const double* dkn_host, const double* dtv_host) {
  Dev& d = h->d;
  if (dir < 0 || dir >= h->tg_ndir || !dkn_host || !dtv_host) {
    h->err = "tangent: bad direction or NULL bond-constant changes";
    return LPM_ERR_ARG;
  }
  const size_t B = (size_t)std::max<int64_t>(h->nb, 1);
  LPM_CUDA(h, cudaMemcpyAsync(d.tg_dkn + (size_t)dir * B, dkn_host, sizeof(double) * h->nb, cudaMemcpyHostToDevice,
                              h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.tg_dtv + (size_t)dir * B, dtv_host, sizeof(double) * h->nb, cudaMemcpyHostToDevice,
                              h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->tg_bond = true;
  return LPM_OK;
}

int tangent_bond_scrit(lpm_handle* h, int dir, const double* dsc_host) {
  Dev& d = h->d;
  if (dir < 0 || dir >= h->tg_ndir || !dsc_host || h->law != LPM_LAW_SOFTENING) {
    h->err = "tangent: bad direction, NULL critical-stretch changes, or not the softening law";
    return LPM_ERR_ARG;
  }
  const size_t B = (size_t)std::max<int64_t>(h->nb, 1);
  LPM_CUDA(h, cudaMemcpyAsync(d.tg_dsc + (size_t)dir * B, dsc_host, sizeof(double) * h->nb, cudaMemcpyHostToDevice,
                              h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

// One converged step's tangents (called after Newton, before the state
// update): for each direction, the equilibrium's change, the changes of
// Pin and of the stress there, then the differentiated J2 return.
int tangent_step(lpm_handle* h) {
  Dev& d = h->d;
  const int dim = h->dim, n = h->n;
  const int64_t m = (int64_t)n * dim;
  int st = adjoint_buffers(h);
  if (st) return st;
  if (h->law == LPM_LAW_SOFTENING) return tangent_soft_round(h);
  if (h->law == LPM_LAW_FATIGUE_HCF) {  // equilibrium with the damage's tangent, then the state update's
    st = tangent_soft_round(h);
    if (st) return st;
    return tangent_hcf_state(h);
  }
  st = check_symmetric_damage(h);
  if (st) return st;
  st = jacobian_prepare(h);
  if (st) return st;
  if (!d.tg_jdl) {
    d.tg_jdl = (double*)zeros_dev(h, sizeof(double) * (size_t)std::max<int64_t>(h->jslots, 1));
    d.tg_jdk = (double*)zeros_dev(h, sizeof(double) * (size_t)std::max<int64_t>(h->jslots, 1));
    if (!d.tg_jdl || !d.tg_jdk) return LPM_ERR_NOMEM;
  }
  LPM_CUDA(h, cudaMemsetAsync(d.adj_a, 0, sizeof(double) * m, h->stream));  // a zero position change
  const JacView J{d.jbase, d.jp2, d.jopp, d.jlayer, d.jc, d.jk, d.jt, d.jf, d.jd, h->jslots};
  for (int k = 0; k < h->tg_ndir; ++k) {
    double* tdlp = d.tg_dlp + (size_t)k * std::max<int64_t>(h->nb, 1);
    double* tsv = d.tg_sv + (size_t)k * n * h->nstate;
    double* tx = d.tg_x + (size_t)k * m;
    double* tpin = d.tg_pin + (size_t)k * m;
    const double* tdp = d.tg_dp + (size_t)k * n * h->law_np;
    k_dlp_slots<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.jslot_of, d.bdamage, tdlp, d.tg_jdl);
    LPM_LAUNCHED(h, "k_dlp_slots");
    const double* dfk = nullptr;
    if (h->tg_bond) {  // the bond constants' changes (lpm_tangent_bond_constants)
      const size_t B = (size_t)std::max<int64_t>(h->nb, 1);
      k_dfk_slots<<<grid_for(n, 128), 128, 0, h->stream>>>(n, d.bptr, d.jslot_of, d.blayer, d.bdamage, d.dLe,
                                                          d.dle_tot, d.tg_dkn + (size_t)k * B,
                                                          d.tg_dtv + (size_t)k * B, d.tg_jdk);
      LPM_LAUNCHED(h, "k_dfk_slots");
      dfk = d.tg_jdk;
    }
    // H_ff dx_f = -(dPin/d dLp . d dLp + dPin/d(Kn, Tv) . d(Kn, Tv))_f
    st = apply_jacobian(h, d.adj_a, d.adj_q, false, nullptr, d.tg_jdl, dfk);
    if (st) return st;
    k_tg_rhs<<<grid_for(m, 256), 256, 0, h->stream>>>(n, dim, d.adj_q, d.mask, d.adj_g);
    LPM_LAUNCHED(h, "k_tg_rhs");
    long long it = 0;
    double rr = 0.0;
    st = jacobian_cg(h, d.adj_g, tx, h->tg_tol, -1, &it, &rr);
    if (st) return st;
    h->stats.tangent_cg_iters += it;
    if (!(rr <= h->tg_tol)) {
      h->err = "tangent: the equilibrium change did not converge";
      return LPM_NOT_CONVERGED;
    }
    // dPin and the stress change at the equilibrium (pass 1 leaves d f in J.jd)
    st = apply_jacobian(h, tx, tpin, false, nullptr, d.tg_jdl, dfk);
    if (st) return st;
    k_jvp_stress<<<grid_for(n, 128), 128, 0, h->stream>>>(n, dim, J, tx, d.bptr, d.bp2, d.jslot_of, d.opp, d.bforce,
                                                         d.cs, d.dis, d.nbonds, h->particle_volume, h->nneighbors,
                                                         d.tg_stress);
    LPM_LAUNCHED(h, "k_jvp_stress");
    k_j2_tangent<<<grid_for(n, 128), 128, 0, h->stream>>>(n, dim, h->law_np, h->nstate, d.pp, tdp, d.state, tsv,
                                                         d.stress, d.tg_stress, d.bptr, d.bp2, d.dis, d.cs, tx,
                                                         tdlp);
    LPM_LAUNCHED(h, "k_j2_tangent");
  }
  return LPM_OK;
}

// ---------------------------------------------------------------- checkpoints
namespace {
struct CkField {
  void* dev;
  size_t bytes;
};
// the arrays that define a step's state; everything else is recomputed by
// the force pass after a restore
std::vector<CkField> checkpoint_fields(lpm_handle* h) {
  Dev& d = h->d;
  const size_t N = (size_t)h->n, B = (size_t)h->nb, S = (size_t)h->nstate * N;
  std::vector<CkField> f = {{d.x, 3 * N * 8},       {d.xlast, 3 * N * 8},     {d.pex, 3 * N * 8},
                            {d.mask, 3 * N * 4},    {d.damage, N * 8},        {d.damage_last, N * 8},
                            {d.dLp, B * 8},         {d.dLp_last, B * 8},      {d.bdamage, B * 8},
                            {d.bdamage_last, B * 8}, {d.dis_last, B * 8},     {d.bforce_last, B * 8}};
  if (d.state) f.push_back({d.state, S * 8});
  if (d.state_last) f.push_back({d.state_last, S * 8});
  if (d.ddot_local) f.push_back({d.ddot_local, N * 8});
  if (d.ddot_nl) f.push_back({d.ddot_nl, N * 8});
  if (d.bkappa) f.push_back({d.bkappa, B * 8});
  if (d.bkappa_last) f.push_back({d.bkappa_last, B * 8});
  std::vector<CkField> out;
  for (const CkField& c : f)
    if (c.dev && c.bytes) out.push_back(c);
  return out;
}
}  // namespace

int checkpoint_save(lpm_handle* h, int* id) {
  std::vector<CkField> f = checkpoint_fields(h);
  size_t total = 0;
  for (const CkField& c : f) total += (c.bytes + 255) / 256 * 256;
  void* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, std::max<size_t>(total, 256));
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->err = "checkpoint: out of device memory";
    return LPM_ERR_NOMEM;
  }
  size_t off = 0;
  for (const CkField& c : f) {
    e = cudaMemcpyAsync((char*)buf + off, c.dev, c.bytes, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) {
      cudaFree(buf);
      return cuda_fail(h, e, "checkpoint copy");
    }
    off += (c.bytes + 255) / 256 * 256;
  }
  int slot = -1;
  for (size_t k = 0; k < h->checkpoints.size(); ++k)
    if (!h->checkpoints[k].buf) {
      slot = (int)k;
      break;
    }
  if (slot < 0) {
    slot = (int)h->checkpoints.size();
    h->checkpoints.push_back({});
  }
  h->checkpoints[(size_t)slot] = {buf, total};
  *id = slot;
  return LPM_OK;
}

int checkpoint_restore(lpm_handle* h, int id) {
  if (id < 0 || (size_t)id >= h->checkpoints.size() || !h->checkpoints[(size_t)id].buf) {
    h->err = "checkpoint: unknown id";
    return LPM_ERR_ARG;
  }
  const Checkpoint& ck = h->checkpoints[(size_t)id];
  std::vector<CkField> f = checkpoint_fields(h);
  size_t off = 0;
  for (const CkField& c : f) {
    LPM_CUDA(h, cudaMemcpyAsync(c.dev, (const char*)ck.buf + off, c.bytes, cudaMemcpyDeviceToDevice, h->stream));
    off += (c.bytes + 255) / 256 * 256;
  }
  h->a32_valid = false;
  return launch_geometry_force(h);
}

int checkpoint_drop(lpm_handle* h, int id) {
  if (id < 0 || (size_t)id >= h->checkpoints.size() || !h->checkpoints[(size_t)id].buf) {
    h->err = "checkpoint: unknown id";
    return LPM_ERR_ARG;
  }
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  cudaFree(h->checkpoints[(size_t)id].buf);
  h->checkpoints[(size_t)id] = {};
  return LPM_OK;
}

}  // namespace lpm
