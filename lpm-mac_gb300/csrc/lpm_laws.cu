// Material laws: state-variable updates (Assembly::updateStateVar), the
// nonlocal damage rate, and the static / fatigue damage updates.
//
// One thread per particle; each particle's sums walk its bonds and its
// nonlocal neighbours in stored (ascending) order, the order the reference
// loops use.
//   law 1 ParticleElasticDamage  params {k0, k1, damage_threshold}
//   law 2 ParticleJ2Plasticity   params {E, mu, sigmay, xi, H, A, damage_threshold}
//   law 3 ParticleFatigueHCF     params {A, B, d, damage_threshold}
//   law 4 softening bond law     params {alpha, s_c} (per-bond s_c in bcrit)
#include <algorithm>
#include <climits>

#include "lpm_device.cuh"

namespace lpm {
namespace {

struct LawView {
  int n, law, np, ns, undamaged;
  double pvol;
  int nneighbors;
  const int64_t *bptr, *lptr;
  const int *bp2, *blayer, *nbonds, *ptype;
  const double *Kn, *Tv, *dLe, *dis, *cs, *dle_tot, *tdle_tot, *stress, *pp, *x, *nonlocal_L;
  double *dLp, *state, *ddot_local, *ddot_nl, *damage, *bdamage;
  const double *state_last, *damage_last, *bstrain, *crit;
  const int64_t* nl_ptr;
  const int* nl_idx;
};

// particle_elastic_damage.h:89-104 (the total of particle_fatigue_hcf.h:82-125
// is the same sum)
__device__ double strain_energy(const LawView& v, int i) {
  const double Vm = v.pvol * v.nbonds[i] / v.nneighbors;
  double e = 0.0;
  for (int l = 0; l < NL; ++l) {
    const int64_t b0 = l == 0 ? v.bptr[i] : v.lptr[i], b1 = l == 0 ? v.lptr[i] : v.bptr[i + 1];
    for (int64_t b = b0; b < b1; ++b) e += 0.5 * (v.Kn[b] * v.dLe[b] * v.dLe[b]) / Vm;
    e += 0.5 * v.tdle_tot[NL * i + l] * v.dle_tot[NL * i + l] / Vm;
  }
  return e;
}

__global__ void k_update_state(LawView v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const double* P = v.pp + (int64_t)i * v.np;
  double* sv = v.state + (int64_t)i * v.ns;
  const double* svl = v.state_last + (int64_t)i * v.ns;
  if (v.law == 1) {  // particle_elastic_damage.h:150-161
    const double k0 = P[0], k1 = P[1];
    sv[0] = strain_energy(v, i);
    const double delta = sv[0] - svl[0];
    const double f = sv[0] - k1 * v.damage[i] - k0;
    v.ddot_local[i] = (f > 0 && delta > 0) ? (1 / k1) * delta : 0.0;
  } else if (v.law == 2) {  // particle_j2plasticity.h:78-140 (radial return)
    const double E = P[0], mu = P[1], sigmay = P[2], xi = P[3], H = P[4], A = P[5];
    double st[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) st[j] = v.stress[6 * (int64_t)i + j];
    const double sigma_m = 1.0 / 3.0 * (st[0] + st[1] + st[2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) st[j] -= sigma_m;
#pragma unroll
    for (int j = 0; j < 6; ++j) st[j] -= sv[j + 1];
    double seq = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) seq += (j < 3 ? 1.0 : 2.0) * st[j] * st[j];
    seq = sqrt(3.0 / 2.0 * seq);
    const double yf = seq - (sigmay + (1.0 - xi) * H * sv[0]);
    const double G = E / 2 / (1 + mu);
    const double dl = yf > 0.0 ? yf / (3 * G + H) : 0.0;
    sv[0] += dl;
    double dp[6] = {0, 0, 0, 0, 0, 0};
    if (fabs(seq) > EPS) {
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        dp[j] = dl * 1.5 * st[j] / seq;
        sv[j + 1] += 2. / 3. * xi * H * dp[j];
      }
    }
    if (dl != 0.0)
      for (int64_t b = v.bptr[i]; b < v.bptr[i + 1]; ++b) {
        const double c0 = v.cs[3 * b], c1 = v.cs[3 * b + 1], c2 = v.cs[3 * b + 2];
        v.dLp[b] += v.dis[b] * (dp[0] * c0 * c0 + dp[1] * c1 * c1 + dp[2] * c2 * c2 + 2 * dp[3] * c1 * c2 +
                                2 * dp[4] * c0 * c2 + 2 * dp[5] * c0 * c1);
      }
    const double tri = seq > EPS ? sigma_m / seq : 0.0;
    v.ddot_local[i] = dl * (1.0 + A * tri);
  } else if (v.law == 3) {  // particle_fatigue_hcf.h:127-145
    const double A = P[0], B = P[1], d = P[2];
    const double u = strain_energy(v, i);
    sv[1] = fmin(u, sv[1]);
    sv[2] = fmax(u, sv[2]);
    sv[0] = fmax(sv[2], sv[0]);
    v.ddot_local[i] = (sv[2] - sv[1] > 0) ? A * pow(sv[0], B) * pow(sv[2] - sv[1], d) : 0.0;
  }
}

// func_phi (lpm.h:45-49) and the nonlocal damage rate of
// SolverStatic::updateStaticDamage / SolverFatigue::updateFatigueDamage
// (solver_static.h:34-54, solver_fatigue.h:79-116).
__device__ __forceinline__ double phi(double x, double L) {
  const double t = x / L;
  const double t2 = t * t, t4 = t2 * t2;
  const double g = 1 / (1 + t4 * t4);
  return g * g;
}

__global__ void k_nonlocal_rate(LawView v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || v.ptype[i] == v.undamaged) return;
  double A = 0.0, D = 0.0;
  const double x0 = v.x[3 * i], x1 = v.x[3 * i + 1], x2 = v.x[3 * i + 2];
  const double L = v.nonlocal_L[i];
  for (int64_t q = v.nl_ptr[i]; q < v.nl_ptr[i + 1]; ++q) {
    const int j = v.nl_idx[q];
    if (v.ptype[j] == v.undamaged) continue;
    const double dx = x0 - v.x[3 * j], dy = x1 - v.x[3 * j + 1], dz = x2 - v.x[3 * j + 2];
    const double w = phi(bond_length(dx, dy, dz), L) * (v.pvol * v.nbonds[j] / v.nneighbors);
    D += v.ddot_local[j] * w;
    A += w;
  }
  v.ddot_nl[i] = D / A;
}

// updateParticleStaticDamage of each law (particle_elastic.h:52-68,
// particle_elastic_damage.h:163-173, particle_j2plasticity.h:142-152).
__global__ void k_static_damage(LawView v, int* any) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || v.ptype[i] == v.undamaged) return;
  bool hit = false;
  if (v.law == 0) {
    const double c = v.crit[i];
    for (int64_t b = v.bptr[i]; b < v.bptr[i + 1]; ++b)
      if (v.bstrain[b] >= c && fabs(v.bdamage[b] - 1.0) > EPS) {
        v.bdamage[b] = 1.0;
        hit = true;
      }
  } else if (v.law == 1 || v.law == 2) {
    const double thr = v.pp[(int64_t)i * v.np + (v.law == 1 ? 2 : 6)];
    double d = v.damage[i] + v.ddot_nl[i];
    if (d >= thr) d = 1.0;
    v.damage[i] = d;
    hit = fabs(d - v.damage_last[i]) > 1e-3;
  }
  if (hit) atomicOr(any, 1);
}

// Softening bond law: kappa = max(kappa, stretch), d(kappa) linear softening
// between s_c and alpha s_c; bdamage never decreases.  Thread per particle,
// its own bonds (both directed copies of a bond see the same stretch).
__global__ void k_softening_damage(int n, const int64_t* __restrict__ bptr, const int* __restrict__ ptype,
                                   int undamaged, const double* __restrict__ pp, int np,
                                   const double* __restrict__ dis, const double* __restrict__ dis0,
                                   const double* __restrict__ bcrit, double* __restrict__ bkappa,
                                   double* __restrict__ bdamage, int* any) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || ptype[i] == undamaged) return;
  const double alpha = pp[(int64_t)i * np];
  bool hit = false;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    const double s = (dis[b] - dis0[b]) / dis0[b];
    const double k = fmax(bkappa[b], s);
    bkappa[b] = k;
    const double sc = bcrit[b];
    double d = 0.0;
    if (k >= alpha * sc)
      d = 1.0;
    else if (k > sc)
      d = 1.0 - (sc / k) * (alpha * sc - k) / ((alpha - 1.0) * sc);
    const double old = bdamage[b];
    if (d > old) {
      bdamage[b] = d;
      if (d - old > 1e-3) hit = true;
    }
  }
  if (hit) atomicOr(any, 1);
}

// ParticleFatigueHCF::updateParticleFatigueDamage (particle_fatigue_hcf.h:147-160).
__global__ void k_fatigue_damage(LawView v, double dt, int* any) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || v.ptype[i] == v.undamaged || v.law != 3) return;
  const double thr = v.pp[(int64_t)i * v.np + 3];
  double d = v.damage[i] + v.ddot_nl[i] * dt;
  if (d >= thr) d = 1.0;
  v.damage[i] = d;
  v.state[(int64_t)i * v.ns + 1] = (double)INT_MAX;
  v.state[(int64_t)i * v.ns + 2] = 0.0;
  if (fabs(d - v.damage_last[i]) > 1e-3) atomicOr(any, 1);
}

// ---- forward-mode tangents of the HCF law (lpm_tangent_begin with law 3)
// Per direction: dx the step's equilibrium change, dp the parameter
// directions [n][np], tsv the state tangents [n][3] (U_hist, U_min, U_max),
// tdd the local rate's tangent, tdnl the nonlocal rate's, tdD the damage's.

__device__ __forceinline__ void load_dv(const double* __restrict__ v, int dim, int i, double (&o)[3]) {
  o[0] = v[(int64_t)dim * i];
  o[1] = v[(int64_t)dim * i + 1];
  o[2] = dim == 3 ? v[(int64_t)dim * i + 2] : 0.0;
}

// Tangent of ParticleFatigueHCF::updateParticleStateVariables (k_update_state,
// law 3), run before it on the same state.  U = sum Kn dLe^2/(2 Vm) +
// sum_l T_l D_l/(2 Vm) with d dLe = c . (dx_i - dx_j); U_min, U_max, U_hist
// follow the branch the update takes; the local rate
// A U_hist^B (U_max - U_min)^d is differentiated along A, B, d and the states.
__global__ void k_hcf_tangent_state(LawView v, int dim, const double* __restrict__ dx,
                                    const double* __restrict__ dp, double* __restrict__ tsv,
                                    double* __restrict__ tdd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const double Vm = v.pvol * v.nbonds[i] / v.nneighbors;
  double ui[3];
  load_dv(dx, dim, i, ui);
  double dU = 0.0;
  for (int l = 0; l < NL; ++l) {
    const int64_t b0 = l == 0 ? v.bptr[i] : v.lptr[i], b1 = l == 0 ? v.lptr[i] : v.bptr[i + 1];
    double dD = 0.0, dT = 0.0;
    for (int64_t b = b0; b < b1; ++b) {
      double uj[3];
      load_dv(dx, dim, v.bp2[b], uj);
      const double de = v.cs[3 * b] * (ui[0] - uj[0]) + v.cs[3 * b + 1] * (ui[1] - uj[1]) +
                        v.cs[3 * b + 2] * (ui[2] - uj[2]);
      dU += v.Kn[b] * v.dLe[b] * de / Vm;
      dD += de;
      dT += v.Tv[b] * de;
    }
    dU += 0.5 * (dT * v.dle_tot[NL * i + l] + v.tdle_tot[NL * i + l] * dD) / Vm;
  }
  const double u = strain_energy(v, i);
  const double* sv = v.state + (int64_t)i * v.ns;
  double* ts = tsv + (int64_t)i * v.ns;
  if (u < sv[1]) ts[1] = dU;
  if (u > sv[2]) ts[2] = dU;
  const double umin = fmin(u, sv[1]), umax = fmax(u, sv[2]);
  if (umax > sv[0]) ts[0] = ts[2];
  const double uh = fmax(umax, sv[0]);
  const double* P = v.pp + (int64_t)i * v.np;
  const double* dP = dp + (int64_t)i * v.np;
  const double r = umax - umin;
  if (r > 0) {
    const double A = P[0], B = P[1], d = P[2];
    const double g = pow(uh, B) * pow(r, d);
    const double dg = g * (log(uh) * dP[1] + B * ts[0] / uh + log(r) * dP[2] + d * (ts[2] - ts[1]) / r);
    tdd[i] = dP[0] * g + A * dg;
  } else {
    tdd[i] = 0.0;
  }
}

// Tangent of the nonlocal rate (k_nonlocal_rate) at the same positions:
// weights w_ij = phi(r_ij, L) Vm_j move with the positions,
// d r = (x_i - x_j).(dx_i - dx_j)/r, d phi/d r = -16 t^7 g^3 / L (t = r/L, g = 1/(1+t^8)).
__global__ void k_hcf_tangent_nonlocal(LawView v, int dim, const double* __restrict__ dx,
                                       const double* __restrict__ tdd, double* __restrict__ tdnl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || v.ptype[i] == v.undamaged) return;
  double A = 0.0, D = 0.0, dA = 0.0, dD = 0.0;
  const double x0 = v.x[3 * i], x1 = v.x[3 * i + 1], x2 = v.x[3 * i + 2];
  double ui[3];
  load_dv(dx, dim, i, ui);
  const double L = v.nonlocal_L[i];
  for (int64_t q = v.nl_ptr[i]; q < v.nl_ptr[i + 1]; ++q) {
    const int j = v.nl_idx[q];
    if (v.ptype[j] == v.undamaged) continue;
    const double ex = x0 - v.x[3 * j], ey = x1 - v.x[3 * j + 1], ez = x2 - v.x[3 * j + 2];
    const double rr = bond_length(ex, ey, ez);
    const double vm = v.pvol * v.nbonds[j] / v.nneighbors;
    const double w = phi(rr, L) * vm;
    double dw = 0.0;
    if (rr > 0.0) {
      double uj[3];
      load_dv(dx, dim, j, uj);
      const double dr = (ex * (ui[0] - uj[0]) + ey * (ui[1] - uj[1]) + ez * (ui[2] - uj[2])) / rr;
      const double t = rr / L, t2 = t * t, t4 = t2 * t2, t7 = t4 * t2 * t;
      const double g = 1 / (1 + t4 * t4);
      dw = -16.0 * t7 * g * g * g / L * dr * vm;
    }
    D += v.ddot_local[j] * w;
    dD += tdd[j] * w + v.ddot_local[j] * dw;
    A += w;
    dA += dw;
  }
  tdnl[i] = (dD - (D / A) * dA) / A;
}

// Tangent of ParticleFatigueHCF::updateParticleFatigueDamage (k_fatigue_damage),
// run before it: D += Ddot_nl dt unless it reaches the threshold (then 1);
// the reset U_min, U_max are constants.
__global__ void k_hcf_tangent_damage(LawView v, double dt, const double* __restrict__ tdnl, double* __restrict__ tdD,
                                     double* __restrict__ tsv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || v.ptype[i] == v.undamaged) return;
  const double thr = v.pp[(int64_t)i * v.np + 3];
  const double d = v.damage[i] + v.ddot_nl[i] * dt;
  tdD[i] = d >= thr ? 0.0 : tdD[i] + tdnl[i] * dt;
  tsv[(int64_t)i * v.ns + 1] = 0.0;
  tsv[(int64_t)i * v.ns + 2] = 0.0;
}

// Tangent of the bond damage the force pass raises to the larger particle
// damage (bdamage = max(bdamage, D_i, D_j), particle_fatigue_hcf.h:74),
// run before the force pass.
__global__ void k_hcf_tangent_bdamage(int n, const int64_t* __restrict__ bptr, const int* __restrict__ bp2,
                                      const double* __restrict__ bdamage, const double* __restrict__ damage,
                                      const double* __restrict__ tdD, double* __restrict__ tdd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double di = damage[i];
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    const int j = bp2[b];
    const double dj = damage[j];
    const double m = fmax(di, dj);
    if (m > bdamage[b]) tdd[b] = di >= dj ? tdD[i] : tdD[j];
  }
}

LawView law_view(lpm_handle* h) {
  Dev& d = h->d;
  LawView v;
  v.n = h->n;
  v.law = h->law;
  v.np = h->law_np;
  v.ns = h->nstate;
  v.undamaged = h->undamaged;
  v.pvol = h->particle_volume;
  v.nneighbors = h->nneighbors;
  v.bptr = d.bptr;
  v.lptr = d.lptr;
  v.bp2 = d.bp2;
  v.blayer = d.blayer;
  v.nbonds = d.nbonds;
  v.ptype = d.ptype;
  v.Kn = d.Kn;
  v.Tv = d.Tv;
  v.dLe = d.dLe;
  v.dis = d.dis;
  v.cs = d.cs;
  v.dle_tot = d.dle_tot;
  v.tdle_tot = d.tdle_tot;
  v.stress = d.stress;
  v.pp = d.pp;
  v.x = d.x;
  v.nonlocal_L = d.nonlocal_L;
  v.dLp = d.dLp;
  v.state = d.state;
  v.ddot_local = d.ddot_local;
  v.ddot_nl = d.ddot_nl;
  v.damage = d.damage;
  v.bdamage = d.bdamage;
  v.state_last = d.state_last;
  v.damage_last = d.damage_last;
  v.bstrain = d.bstrain;
  v.crit = d.crit;
  v.nl_ptr = d.nl_ptr;
  v.nl_idx = d.nl_idx;
  return v;
}

int read_flag(lpm_handle* h, int* flag, int* out) {
  int v = 0;
  LPM_CUDA(h, cudaMemcpyAsync(&v, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  *out = v;
  return LPM_OK;
}

}  // namespace

// HCF tangents (lpm_tangent_begin with law 3), one launch per direction.
int tangent_hcf_state(lpm_handle* h) {
  const int T = 128;
  const int64_t m = (int64_t)h->n * h->dim;
  const LawView v = law_view(h);
  Dev& d = h->d;
  for (int k = 0; k < h->tg_ndir; ++k) {
    k_hcf_tangent_state<<<grid_for(h->n, T), T, 0, h->stream>>>(
        v, h->dim, d.tg_x + k * m, d.tg_dp + (int64_t)k * h->n * h->law_np, d.tg_sv + (int64_t)k * h->n * h->nstate,
        d.tg_ddot + (int64_t)k * h->n);
    LPM_LAUNCHED(h, "k_hcf_tangent_state");
  }
  return LPM_OK;
}

int tangent_hcf_bdamage(lpm_handle* h) {
  const int T = 128;
  Dev& d = h->d;
  const size_t B = (size_t)std::max<int64_t>(h->nb, 1);
  for (int k = 0; k < h->tg_ndir; ++k) {
    k_hcf_tangent_bdamage<<<grid_for(h->n, T), T, 0, h->stream>>>(h->n, d.bptr, d.bp2, d.bdamage, d.damage,
                                                                 d.tg_dD + (int64_t)k * h->n, d.tg_dd + k * B);
    LPM_LAUNCHED(h, "k_hcf_tangent_bdamage");
  }
  return LPM_OK;
}

int launch_update_state(lpm_handle* h) {
  // with tangent directions on, their step comes first: it needs the state
  // before the update (lpm_tangent_begin)
  if (h->tg_ndir > 0) {
    const int st = tangent_step(h);
    if (st) return st;
  }
  if (h->law == 0) return LPM_OK;  // ParticleElastic has no state update
  const int T = 128;
  k_update_state<<<grid_for(h->n, T), T, 0, h->stream>>>(law_view(h));
  LPM_LAUNCHED(h, "k_update_state");
  return LPM_OK;
}

int launch_static_damage(lpm_handle* h, int* any_new) {
  int* flag = (int*)h->d.red.ticket + 15;
  LPM_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
  const int T = 128;
  const LawView v = law_view(h);
  if (h->law == 1 || h->law == 2) {
    if (!h->d.nl_ptr) {
      h->err = "damage law without nonlocal neighbours (lpm_set_nonlocal)";
      return LPM_ERR_STATE;
    }
    k_nonlocal_rate<<<grid_for(h->n, T), T, 0, h->stream>>>(v);
    LPM_LAUNCHED(h, "k_nonlocal_rate");
  }
  if (h->law <= 2) {
    k_static_damage<<<grid_for(h->n, T), T, 0, h->stream>>>(v, flag);
    LPM_LAUNCHED(h, "k_static_damage");
  }
  if (h->law == LPM_LAW_SOFTENING) {
    if (h->tg_ndir > 0) {  // the update's tangent reads the state before it
      const int st = tangent_soft_damage(h);
      if (st) return st;
    }
    const Dev& d = h->d;
    k_softening_damage<<<grid_for(h->n, T), T, 0, h->stream>>>(h->n, d.bptr, d.ptype, h->undamaged, d.pp, h->law_np,
                                                               d.dis, d.dis0, d.bcrit, d.bkappa, d.bdamage, flag);
    LPM_LAUNCHED(h, "k_softening_damage");
  }
  return read_flag(h, flag, any_new);
}

int launch_fatigue_damage(lpm_handle* h, double dt, int* any_new) {
  int* flag = (int*)h->d.red.ticket + 15;
  LPM_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
  if (h->law == 3) {
    if (!h->d.nl_ptr) {
      h->err = "fatigue law without nonlocal neighbours (lpm_set_nonlocal)";
      return LPM_ERR_STATE;
    }
    const int T = 128;
    const LawView v = law_view(h);
    k_nonlocal_rate<<<grid_for(h->n, T), T, 0, h->stream>>>(v);
    LPM_LAUNCHED(h, "k_nonlocal_rate");
    const int64_t m = (int64_t)h->n * h->dim;
    Dev& d = h->d;
    for (int k = 0; k < h->tg_ndir; ++k) {  // tangents first: they read the state before the update
      k_hcf_tangent_nonlocal<<<grid_for(h->n, T), T, 0, h->stream>>>(v, h->dim, d.tg_x + k * m,
                                                                     d.tg_ddot + (int64_t)k * h->n,
                                                                     d.tg_dnl + (int64_t)k * h->n);
      LPM_LAUNCHED(h, "k_hcf_tangent_nonlocal");
      k_hcf_tangent_damage<<<grid_for(h->n, T), T, 0, h->stream>>>(v, dt, d.tg_dnl + (int64_t)k * h->n,
                                                                   d.tg_dD + (int64_t)k * h->n,
                                                                   d.tg_sv + (int64_t)k * h->n * h->nstate);
      LPM_LAUNCHED(h, "k_hcf_tangent_damage");
    }
    k_fatigue_damage<<<grid_for(h->n, T), T, 0, h->stream>>>(v, dt, flag);
    LPM_LAUNCHED(h, "k_fatigue_damage");
  }
  return read_flag(h, flag, any_new);
}

}  // namespace lpm
