// Force path: bond geometry and nonlocal dilatation sums, bond forces,
// particle forces / stress / damage_visual, residual and boundary conditions.
//
// One thread owns one particle and walks its bonds in stored order, so every
// per-particle sum adds its terms in the order Particle::bond_layers lists
// them (particle.h:163-181, 197-240).
#include "lpm_device.cuh"

namespace lpm {
namespace {

// Bond geometry + per-layer sums (bond.h:30-39, particle.h:163-181), then
// the elastic bond force (particle_elastic.h:38-50), which needs the owner's
// complete dLe_total: bforce = (2 Kn dLe + 2 Tv dLe_total[layer]) (1 - bdamage).
__global__ void k_geometry_force(int n, const double* __restrict__ x, const int64_t* __restrict__ bptr,
                                 const int* __restrict__ bp2, const int* __restrict__ blayer,
                                 const double* __restrict__ dis0, const double* __restrict__ dLp,
                                 double* __restrict__ bdamage, const double* __restrict__ Kn,
                                 const double* __restrict__ Tv, double* __restrict__ dis, double* __restrict__ bstrain,
                                 double* __restrict__ dLe, double* __restrict__ cs, double* __restrict__ bforce,
                                 double* __restrict__ dle_tot, double* __restrict__ tdle_tot,
                                 double* __restrict__ cs_sum, const double* __restrict__ damage, int damage_law,
                                 double* __restrict__ tsum, double* __restrict__ msum) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xi0 = x[3 * i], xi1 = x[3 * i + 1], xi2 = x[3 * i + 2];
  double dlt[NL] = {0.0, 0.0}, tdlt[NL] = {0.0, 0.0};
  double css[NL][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  const int64_t b0 = bptr[i], b1 = bptr[i + 1];
  for (int64_t b = b0; b < b1; ++b) {
    const int j = bp2[b];
    const double dx = xi0 - x[3 * j], dy = xi1 - x[3 * j + 1], dz = xi2 - x[3 * j + 2];
    const double d = bond_length(dx, dy, dz);
    const bool br = is_broken(bdamage[b]);
    const double d0 = dis0[b];
    const double dl = br ? 0.0 : (d - d0);
    const double e = br ? 0.0 : (d - d0 - dLp[b]);
    // the direction cosines use one reciprocal per bond (products, within
    // an ulp of dx/dis); the strain is the quotient dL/dis itself, so that
    // the brittle test bstrain >= critical (particle_elastic.h:60) sees the
    // reference's value bit for bit
    const double rd = 1.0 / d;
    const double c0 = br ? 0.0 : dx * rd, c1 = br ? 0.0 : dy * rd, c2 = br ? 0.0 : dz * rd;
    dis[b] = d;
    bstrain[b] = br ? 0.0 : dl / d;
    dLe[b] = e;
    cs[3 * b] = c0;
    cs[3 * b + 1] = c1;
    cs[3 * b + 2] = c2;
    const double te = Tv[b] * e;
    if (blayer[b] == 0) {
      dlt[0] += e;
      tdlt[0] += te;
      css[0][0] += c0;
      css[0][1] += c1;
      css[0][2] += c2;
    } else {
      dlt[1] += e;
      tdlt[1] += te;
      css[1][0] += c0;
      css[1][1] += c1;
      css[1][2] += c2;
    }
  }
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    dle_tot[NL * i + l] = dlt[l];
    tdle_tot[NL * i + l] = tdlt[l];
    cs_sum[(NL * i + l) * 3 + 0] = css[l][0];
    cs_sum[(NL * i + l) * 3 + 1] = css[l][1];
    cs_sum[(NL * i + l) * 3 + 2] = css[l][2];
  }
  // the damage laws raise the bond damage to the larger particle damage
  // first (particle_elastic_damage.h:83, particle_j2plasticity.h:72,
  // particle_fatigue_hcf.h:74)
  const double di = damage_law ? damage[i] : 0.0;
  // the tangent's per-particle sums use the final bond damage (the tangent
  // is assembled after this pass): T = sum w Tv n, M = sum w (2 Kn + Tv) n n^T
  double T[2 * 3] = {0, 0, 0, 0, 0, 0}, M[2 * 6] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t b = b0; b < b1; ++b) {
    const bool l1 = blayer[b] != 0;
    double f = 2. * Kn[b] * dLe[b] + 2. * Tv[b] * (l1 ? dlt[1] : dlt[0]);
    double bd = bdamage[b];
    if (damage_law) {
      bd = fmax(bd, fmax(di, damage[bp2[b]]));
      bdamage[b] = bd;
    }
    const double w = 1.0 - bd;
    f *= w;
    bforce[b] = f;
    const double c0 = cs[3 * b], c1 = cs[3 * b + 1], c2 = cs[3 * b + 2];
    const double wt = w * Tv[b], wk = w * (2.0 * Kn[b] + Tv[b]);
    const double t[3] = {wt * c0, wt * c1, wt * c2};
    const double m[6] = {wk * c0 * c0, wk * c0 * c1, wk * c0 * c2, wk * c1 * c1, wk * c1 * c2, wk * c2 * c2};
    if (l1) {
#pragma unroll
      for (int k = 0; k < 3; ++k) T[3 + k] += t[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) M[6 + k] += m[k];
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) T[k] += t[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) M[k] += m[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) tsum[NL * 3 * i + k] = T[k];
#pragma unroll
  for (int k = 0; k < 12; ++k) msum[NL * 6 * i + k] = M[k];
}

// Pin = sum cs * (f + f_opposite)/2 (particle.h:197-215); stress from the
// averaged bond force (particle.h:217-240); damage_visual (particle.h:151-161).
__global__ void k_particle_force(int n, const int64_t* __restrict__ bptr, const int* __restrict__ opp,
                                 const double* __restrict__ bforce, const double* __restrict__ cs,
                                 const double* __restrict__ dis, const double* __restrict__ bdamage,
                                 const int* __restrict__ nbonds, double pvol, int nneighbors, double* __restrict__ pin,
                                 double* __restrict__ stress, double* __restrict__ dvis) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double P0 = 0, P1 = 0, P2 = 0, s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0, dv = 0;
  const double Vm = pvol * nbonds[i] / nneighbors;
  const double hv = 0.5 / Vm;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    const double f = 0.5 * (bforce[b] + bforce[opp[b]]);
    const double c0 = cs[3 * b], c1 = cs[3 * b + 1], c2 = cs[3 * b + 2];
    P0 += c0 * f;
    P1 += c1 * f;
    P2 += c2 * f;
    const double sf = hv * dis[b] * f;
    s0 += sf * c0 * c0;
    s1 += sf * c1 * c1;
    s2 += sf * c2 * c2;
    s3 += sf * c1 * c2;
    s4 += sf * c0 * c2;
    s5 += sf * c0 * c1;
    dv += bdamage[b];
  }
  pin[3 * i] = P0;
  pin[3 * i + 1] = P1;
  pin[3 * i + 2] = P2;
  stress[6 * i + 0] = s0;
  stress[6 * i + 1] = s1;
  stress[6 * i + 2] = s2;
  stress[6 * i + 3] = s3;
  stress[6 * i + 4] = s4;
  stress[6 * i + 5] = s5;
  dvis[i] = dv / (double)nbonds[i];
}

// r = (1 - mask) (Pex - Pin) on the dim DOFs of each particle, |r|^2 and
// |reaction|^2 (solver.h:108-128, 62-63).
__global__ void k_residual(int n, int dim, const int* __restrict__ mask, const double* __restrict__ pex,
                           const double* __restrict__ pin, double* __restrict__ r, double* partials,
                           unsigned int* ticket, double* norms) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int k = 0; k < dim; ++k) {
      const int m = mask[3 * i + k];
      const double p = pin[3 * i + k];
      const double ri = (1 - m) * (pex[3 * i + k] - p);
      r[dim * i + k] = ri;
      v[0] += ri * ri;
      if (m == 1) v[1] += p * p;
    }
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    norms[0] = sqrt(tot[0]);
    norms[1] = sqrt(tot[1]);
  }
}

// Particle::moveBy with Solver::disp (solver.h:97-105): all particles move.
__global__ void k_move_by(int n, int dim, const double* __restrict__ d, double* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < dim; ++k) x[3 * i + k] += d[dim * i + k];
}

// DispBC (solver.h:130-166).
__global__ void k_disp_bc(const int* __restrict__ ids, int count, int axis, int mode, double value, double* x,
                          int* mask) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = ids[t];
  if (mode == 0) {
    x[3 * i + axis] += value;
  } else {
    x[3 * i + 0] = axis == 0 ? value : 0.0;
    x[3 * i + 1] = axis == 1 ? value : 0.0;
    x[3 * i + 2] = axis == 2 ? value : 0.0;
  }
  mask[3 * i + axis] = 1;
}

// ForceBC (solver.h:168-190).
__global__ void k_force_bc(const int* __restrict__ ids, int count, int mode, double fx, double fy, double fz,
                           double* pex) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = ids[t];
  const double a = fx / count, b = fy / count, c = fz / count;
  if (mode == 0) {
    pex[3 * i] += a;
    pex[3 * i + 1] += b;
    pex[3 * i + 2] += c;
  } else {
    pex[3 * i] = a;
    pex[3 * i + 1] = b;
    pex[3 * i + 2] = c;
  }
}

// Load increments of cycle N of a spectrum held on the device
// (SolverFatigue::generateLoadCycle, solver_fatigue.h:128-172): the loading
// half steps by (f1 - f0)/n_interval, the unloading half by (f2 - f1)/n_interval,
// with f0, f1, f2 = spectrum[2N], spectrum[2N+1], spectrum[2N+2].
__global__ void k_cycle_increments(const double* __restrict__ spectrum, long long N, int n_interval,
                                   double* __restrict__ inc) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double f0 = spectrum[2 * N], f1 = spectrum[2 * N + 1], f2 = spectrum[2 * N + 2];
    inc[0] = (f1 - f0) / n_interval;
    inc[1] = (f2 - f1) / n_interval;
  }
}

// DispBC / ForceBC with the unit load scaled by a factor read from device
// memory (the cycle's increment), so the host never reads the spectrum.
__global__ void k_disp_bc_scaled(const int* __restrict__ ids, int count, int axis, int mode, double unit,
                                 const double* __restrict__ scale, double* x, int* mask) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = ids[t];
  const double value = unit * scale[0];
  if (mode == 0) {
    x[3 * i + axis] += value;
  } else {
    x[3 * i + 0] = axis == 0 ? value : 0.0;
    x[3 * i + 1] = axis == 1 ? value : 0.0;
    x[3 * i + 2] = axis == 2 ? value : 0.0;
  }
  mask[3 * i + axis] = 1;
}

__global__ void k_force_bc_scaled(const int* __restrict__ ids, int count, int mode, double fx, double fy, double fz,
                                  const double* __restrict__ scale, double* pex) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = ids[t];
  const double s = scale[0];
  const double a = fx * s / count, b = fy * s / count, c = fz * s / count;
  if (mode == 0) {
    pex[3 * i] += a;
    pex[3 * i + 1] += b;
    pex[3 * i + 2] += c;
  } else {
    pex[3 * i] = a;
    pex[3 * i + 1] = b;
    pex[3 * i + 2] = c;
  }
}

// Mean of the first state variable (the HCF law's strain energy) over the
// particles that damage (SolverFatigue::solveProblemCyclic,
// solver_fatigue.h:201-212).
__global__ void k_mean_state0(int n, int ns, const double* __restrict__ state, const int* __restrict__ ptype,
                              int undamaged, double* partials, unsigned int* ticket, double* out) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (ptype[i] != undamaged) {
      v[0] += state[(int64_t)i * ns];
      v[1] += 1.0;
    }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) *out = tot[1] > 0 ? tot[0] / tot[1] : 0.0;
}

}  // namespace

int launch_cycle_increments(lpm_handle* h, const double* spectrum, long long N, int n_interval, double* inc) {
  k_cycle_increments<<<1, 32, 0, h->stream>>>(spectrum, N, n_interval, inc);
  LPM_LAUNCHED(h, "k_cycle_increments");
  return LPM_OK;
}

int launch_disp_bc_scaled(lpm_handle* h, const Group& g, int axis, int mode, double unit, const double* scale) {
  if (g.count == 0) return LPM_OK;
  const int T = 256;
  k_disp_bc_scaled<<<grid_for(g.count, T), T, 0, h->stream>>>(g.ids, g.count, axis, mode, unit, scale, h->d.x,
                                                              h->d.mask);
  LPM_LAUNCHED(h, "k_disp_bc_scaled");
  return LPM_OK;
}

int launch_force_bc_scaled(lpm_handle* h, const Group& g, int mode, double fx, double fy, double fz,
                           const double* scale) {
  if (g.count == 0) return LPM_OK;
  const int T = 256;
  k_force_bc_scaled<<<grid_for(g.count, T), T, 0, h->stream>>>(g.ids, g.count, mode, fx, fy, fz, scale, h->d.pex);
  LPM_LAUNCHED(h, "k_force_bc_scaled");
  return LPM_OK;
}

int launch_mean_state0(lpm_handle* h, double* out_dev) {
  const int G = grid_for(h->n, kRedThreads, kMaxRedBlocks);
  k_mean_state0<<<G, kRedThreads, 0, h->stream>>>(h->n, h->nstate, h->d.state, h->d.ptype, h->undamaged,
                                                  h->d.red.partials, h->d.red.ticket + 12, out_dev);
  LPM_LAUNCHED(h, "k_mean_state0");
  return LPM_OK;
}

int launch_geometry_force(lpm_handle* h) {
  if (h->tg_ndir > 0 && h->law == LPM_LAW_FATIGUE_HCF) {  // the bond damage's tangent reads it before the pass
    const int st = tangent_hcf_bdamage(h);
    if (st) return st;
  }
  const Dev& d = h->d;
  const int T = 128;
  k_geometry_force<<<grid_for(h->n, T), T, 0, h->stream>>>(h->n, d.x, d.bptr, d.bp2, d.blayer, d.dis0, d.dLp,
                                                           d.bdamage, d.Kn, d.Tv, d.dis, d.bstrain, d.dLe, d.cs,
                                                           d.bforce, d.dle_tot, d.tdle_tot, d.cs_sum, d.damage,
                                                           (h->law >= 1 && h->law <= 3) ? 1 : 0, d.tsum, d.msum);
  LPM_LAUNCHED(h, "k_geometry_force");
  k_particle_force<<<grid_for(h->n, T), T, 0, h->stream>>>(h->n, d.bptr, d.opp, d.bforce, d.cs, d.dis, d.bdamage,
                                                           d.nbonds, h->particle_volume, h->nneighbors, d.pin,
                                                           d.stress, d.dvis);
  LPM_LAUNCHED(h, "k_particle_force");
  return LPM_OK;
}

int launch_residual(lpm_handle* h, double* norm_r, double* norm_R) {
  const Dev& d = h->d;
  const int G = grid_for(h->n, kRedThreads, kMaxRedBlocks);
  k_residual<<<G, kRedThreads, 0, h->stream>>>(h->n, h->dim, d.mask, d.pex, d.pin, d.rhs, d.red.partials,
                                               d.red.ticket + 0, d.norms);
  LPM_LAUNCHED(h, "k_residual");
  LPM_CUDA(h, cudaMemcpyAsync(h->h_norms, d.norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (norm_r) *norm_r = h->h_norms[0];
  if (norm_R) *norm_R = h->h_norms[1];
  return LPM_OK;
}

int launch_move_by_disp(lpm_handle* h) {
  const int T = 256;
  k_move_by<<<grid_for(h->n, T), T, 0, h->stream>>>(h->n, h->dim, h->d.disp, h->d.x);
  LPM_LAUNCHED(h, "k_move_by");
  return LPM_OK;
}

int launch_disp_bc(lpm_handle* h, const Group& g, int axis, int mode, double value) {
  if (g.count == 0) return LPM_OK;
  const int T = 256;
  k_disp_bc<<<grid_for(g.count, T), T, 0, h->stream>>>(g.ids, g.count, axis, mode, value, h->d.x, h->d.mask);
  LPM_LAUNCHED(h, "k_disp_bc");
  return LPM_OK;
}

int launch_force_bc(lpm_handle* h, const Group& g, int mode, double fx, double fy, double fz) {
  if (g.count == 0) return LPM_OK;
  const int T = 256;
  k_force_bc<<<grid_for(g.count, T), T, 0, h->stream>>>(g.ids, g.count, mode, fx, fy, fz, h->d.pex);
  LPM_LAUNCHED(h, "k_force_bc");
  return LPM_OK;
}

}  // namespace lpm
