// CPU oracle for the LPM quasi-static Newton load step (TEST INFRASTRUCTURE).
//
// A restatement of the reference algorithm in plain C++ over flat arrays.
// Only tests/, the smoke check and bench.py's CPU-baseline leg use it; the
// product never does.  Floating-point expressions keep the reference's
// operation order (and are compiled without FMA contraction) so that
// topology, force state and tangent agree bit for bit with the reference
// headers on the same inputs; the CG dot products are sequential for the
// same reason.  Particle loops and the sparse products run under OpenMP with
// a fixed per-row order, so results do not depend on the thread count.
#include "lpm_oracle.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double EPS_ = 1e-6;  // lpm.h:37
const int NL = 2;          // two neighbour layers (all reference examples)

}  // namespace

struct lo_sys {
  int dim = 3, n = 0;
  long nb = 0;
  double particle_volume = 0;
  int nneighbors = 1;
  // particles
  std::vector<double> x, x0, xlast, pin, pex, stress, dvis, dle_tot, tdle_tot, cs_sum;
  std::vector<double> damage, damage_last, ddot_local;
  std::vector<int> mask, nbonds;
  int nstate = 1;
  std::vector<double> state, state_last;
  // bonds (CSR by p1)
  std::vector<long> bptr, bsrc, opp;
  std::vector<int> bp2, blayer;
  std::vector<double> Kn, Tv, dis0, dis, dis_last, dL, dLe, dLp, dLp_last, bstrain, cs, bforce, bforce_last, bdamage,
      bdamage_last;
  // pattern + tangent (BSR by block-row i)
  std::vector<long> cptr, tpos;
  std::vector<int> cidx;
  std::vector<double> K;
  // law: 0 elastic, 1 elastic damage, 2 J2 plasticity, 3 HCF fatigue,
  // 4 softening bond law (no reference class; restated from its definition)
  int law = 0;
  std::vector<double> bcrit, bkappa, bkappa_last;  // softening law, per bond
  int np = 0;                // parameters per particle
  std::vector<double> pp;    // [n * np] per-particle law parameters
  std::vector<double> crit;  // per-particle critical bond strain (elastic law)
  std::vector<int> ptype;    // particle type (undamaged type skips damage)
  int undamaged = -1;
  // nonlocal neighbours (Assembly::searchNonlocalNeighbors) and length scale
  std::vector<long> nl_ptr;
  std::vector<int> nl_idx;
  std::vector<double> nonlocal_L, ddot_nl;
  // log
  std::vector<double> log;
};

namespace {

inline bool broken(double bd) { return std::abs(bd - 1.0) < EPS_; }

// bond.h:30-39 + particle.h:163-181
void update_geometry(lo_sys* s) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s->n; ++i) {
    double dlt[NL] = {0, 0}, tdlt[NL] = {0, 0}, css[NL][3] = {{0, 0, 0}, {0, 0, 0}};
    const double* xi = &s->x[3 * (size_t)i];
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
      const double* xj = &s->x[3 * (size_t)s->bp2[b]];
      double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
      double d = std::sqrt(dx * dx + dy * dy + dz * dz);
      s->dis[b] = d;
      bool br = broken(s->bdamage[b]);
      s->dL[b] = br ? 0.0 : (d - s->dis0[b]);
      s->bstrain[b] = br ? 0.0 : (s->dL[b] / d);
      s->dLe[b] = br ? 0.0 : (d - s->dis0[b] - s->dLp[b]);
      s->cs[3 * b + 0] = br ? 0.0 : (dx / d);
      s->cs[3 * b + 1] = br ? 0.0 : (dy / d);
      s->cs[3 * b + 2] = br ? 0.0 : (dz / d);
      int l = s->blayer[b];
      dlt[l] += s->dLe[b];
      tdlt[l] += s->Tv[b] * s->dLe[b];
      css[l][0] += s->cs[3 * b + 0];
      css[l][1] += s->cs[3 * b + 1];
      css[l][2] += s->cs[3 * b + 2];
    }
    for (int l = 0; l < NL; ++l) {
      s->dle_tot[NL * (size_t)i + l] = dlt[l];
      s->tdle_tot[NL * (size_t)i + l] = tdlt[l];
      for (int k = 0; k < 3; ++k) s->cs_sum[(NL * (size_t)i + l) * 3 + k] = css[l][k];
    }
  }
}

// particle_elastic.h:38-50 (law 0); the damage laws first raise the bond
// damage to the larger particle damage (particle_elastic_damage.h:74-87,
// particle_j2plasticity.h:63-76, particle_fatigue_hcf.h:65-80).
void update_bond_force(lo_sys* s) {
  const bool dmg = s->law >= 1 && s->law <= 3;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s->n; ++i) {
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
      double f = 2. * s->Kn[b] * s->dLe[b] + 2. * s->Tv[b] * s->dle_tot[NL * (size_t)i + s->blayer[b]];
      if (dmg) s->bdamage[b] = std::max(s->bdamage[b], std::max(s->damage[i], s->damage[s->bp2[b]]));
      f *= (1.0 - s->bdamage[b]);
      s->bforce[b] = f;
    }
  }
}

// particle.h:197-240, 151-161
void update_particle_force(lo_sys* s) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s->n; ++i) {
    double P[3] = {0, 0, 0}, st[6] = {0, 0, 0, 0, 0, 0}, dv = 0;
    double Vm = s->particle_volume * s->nbonds[i] / s->nneighbors;
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
      double fo = s->bforce[s->opp[b]];
      double f = s->bforce[b];
      const double* c = &s->cs[3 * b];
      P[0] += c[0] * 0.5 * (f + fo);
      P[1] += c[1] * 0.5 * (f + fo);
      P[2] += c[2] * 0.5 * (f + fo);
      double d = s->dis[b];
      st[0] += 0.5 / Vm * d * 0.5 * (f + fo) * c[0] * c[0];
      st[1] += 0.5 / Vm * d * 0.5 * (f + fo) * c[1] * c[1];
      st[2] += 0.5 / Vm * d * 0.5 * (f + fo) * c[2] * c[2];
      st[3] += 0.5 / Vm * d * 0.5 * (f + fo) * c[1] * c[2];
      st[4] += 0.5 / Vm * d * 0.5 * (f + fo) * c[0] * c[2];
      st[5] += 0.5 / Vm * d * 0.5 * (f + fo) * c[0] * c[1];
      dv += s->bdamage[b];
    }
    for (int k = 0; k < 3; ++k) s->pin[3 * (size_t)i + k] = P[k];
    for (int k = 0; k < 6; ++k) s->stress[6 * (size_t)i + k] = st[k];
    s->dvis[i] = dv / (double)s->nbonds[i];
  }
}

// ---- tangent (derivative.h), restated with the reference's loop order ----
typedef double Blk[3][3];

inline double pprod(double kt, const double* n, int r, int c) {
  // (Kn+Tv) * n_r * n_c as derivative.h writes it: pow() on the diagonal,
  // the larger index multiplied first off the diagonal.
  if (r == c) return kt * (n[r] * n[r]);
  int hi = r > c ? r : c, lo = r > c ? c : r;
  return kt * n[hi] * n[lo];
}

// derivative.h:8-45
void diag_block(const lo_sys* s, int i, int sym, Blk K) {
  std::memset(K, 0, sizeof(Blk));
  for (int l = 0; l < NL; ++l) {
    const double* S = &s->cs_sum[(NL * (size_t)i + l) * 3];
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
      if (s->blayer[b] != l) continue;
      const double* n = &s->cs[3 * b];
      double w = 1 - s->bdamage[b], kn = s->Kn[b], tv = s->Tv[b];
      for (int r = 0; r < 3; ++r)
        for (int c = r; c < 3; ++c) K[r][c] += w * ((kn * n[c] + tv * S[c]) * n[r] + pprod(kn + tv, n, r, c));
    }
  }
  K[1][0] = sym ? K[0][1] : K[1][0];
  K[2][0] = K[0][2];
  K[2][1] = K[1][2];
}

// derivative.h:47-142 (layer 0) and 144-239 (layer 1)
void offdiag_block_layer(const lo_sys* s, int i, int j, int l, Blk K) {
  std::memset(K, 0, sizeof(Blk));
  for (long b1 = s->bptr[i]; b1 < s->bptr[i + 1]; ++b1) {
    if (s->blayer[b1] != l || s->bp2[b1] != j) continue;
    const double* n1 = &s->cs[3 * b1];
    double w1t = (1 - s->bdamage[b1]) * s->Tv[b1];
    for (long b2 = s->bptr[i]; b2 < s->bptr[i + 1]; ++b2) {
      if (s->blayer[b2] != l) continue;
      const double* n2 = &s->cs[3 * b2];
      double w2 = 1 - s->bdamage[b2];
      if (s->bp2[b2] == j) {
        const double* Sj = &s->cs_sum[(NL * (size_t)j + l) * 3];
        double kn = s->Kn[b2], tv = s->Tv[b2];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) K[r][c] += w2 * ((-kn * n2[c] + tv * Sj[c]) * n2[r] - pprod(kn + tv, n2, r, c));
      } else {
        double w2t = w2 * s->Tv[b2];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) K[r][c] -= 0.5 * (w1t + w2t) * n2[r] * n1[c];
        int k = s->bp2[b2];
        for (long b3 = s->bptr[k]; b3 < s->bptr[k + 1]; ++b3) {
          if (s->blayer[b3] != l || s->bp2[b3] != j) continue;
          const double* n3 = &s->cs[3 * b3];
          double w3t = (1 - s->bdamage[b3]) * s->Tv[b3];
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) K[r][c] -= 0.5 * (w3t + w2t) * n2[r] * n3[c];
        }
      }
    }
    return;
  }
  for (long b1 = s->bptr[i]; b1 < s->bptr[i + 1]; ++b1) {
    if (s->blayer[b1] != l) continue;
    const double* n1 = &s->cs[3 * b1];
    double w1t = (1 - s->bdamage[b1]) * s->Tv[b1];
    int k = s->bp2[b1];
    for (long b2 = s->bptr[k]; b2 < s->bptr[k + 1]; ++b2) {
      if (s->blayer[b2] != l || s->bp2[b2] != j) continue;
      const double* n2 = &s->cs[3 * b2];
      double w2t = (1 - s->bdamage[b2]) * s->Tv[b2];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) K[r][c] -= 0.5 * (w2t + w1t) * n1[r] * n2[c];
    }
  }
}

// stiffness.h:67-101 + 228-263
void assemble(lo_sys* s, int sym) {
  const int dim = s->dim;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < s->n; ++i) {
    for (long q = s->cptr[i]; q < s->cptr[i + 1]; ++q) {
      int j = s->cidx[q];
      Blk B;
      if (j == i) {
        diag_block(s, i, sym, B);
      } else {
        Blk B0, B1;
        offdiag_block_layer(s, i, j, 0, B0);
        offdiag_block_layer(s, i, j, 1, B1);
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) B[r][c] = B0[r][c] + B1[r][c];
      }
      double* dst = &s->K[(size_t)q * dim * dim];
      for (int r = 0; r < dim; ++r)
        for (int c = 0; c < dim; ++c) dst[r * dim + c] = B[r][c];
    }
  }
}

// stiffness.h:265-294
void apply_bc(lo_sys* s) {
  const int dim = s->dim;
  double ss = 0;
  for (int i = 0; i < s->n; ++i)
    for (long q = s->cptr[i]; q < s->cptr[i + 1]; ++q)
      if (s->cidx[q] == i)
        for (int r = 0; r < dim; ++r) {
          double v = s->K[(size_t)q * dim * dim + r * dim + r];
          ss += v * v;
        }
  double nd = std::sqrt(ss);
  std::vector<char> fixed((size_t)s->n * dim, 0);
  for (int i = 0; i < s->n; ++i)
    for (int k = 0; k < dim; ++k)
      fixed[(size_t)i * dim + k] = (s->mask[3 * (size_t)i + k] == 1 || std::abs(s->dvis[i] - 1.0) < EPS_) ? 1 : 0;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s->n; ++i)
    for (long q = s->cptr[i]; q < s->cptr[i + 1]; ++q) {
      int j = s->cidx[q];
      double* blk = &s->K[(size_t)q * dim * dim];
      for (int r = 0; r < dim; ++r)
        for (int c = 0; c < dim; ++c) {
          bool fr = fixed[(size_t)i * dim + r], fc = fixed[(size_t)j * dim + c];
          if (fr || fc) blk[r * dim + c] = (i == j && r == c && fr) ? nd : 0.0;
        }
    }
}

void compute_tpos(lo_sys* s) {
  // tpos[q] for block (i, j): index of block (j, i) in block-row j
  s->tpos.assign(s->cidx.size(), -1);
  for (int i = 0; i < s->n; ++i)
    for (long q = s->cptr[i]; q < s->cptr[i + 1]; ++q) {
      int j = s->cidx[q];
      const int* b = &s->cidx[s->cptr[j]];
      const int* e = &s->cidx[s->cptr[j + 1]];
      const int* f = std::lower_bound(b, e, i);
      s->tpos[q] = (f != e && *f == i) ? s->cptr[j] + (f - b) : -1;
    }
}

// y = K^T p.  Entry (j, c) sums column (j, c) of K over rows (i, r) in
// ascending order, as a column-major SparseMatrix column walk does.
void apply_KT(const lo_sys* s, const std::vector<double>& p, std::vector<double>& y) {
  const int dim = s->dim;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < s->n; ++j) {
    for (int c = 0; c < dim; ++c) {
      double acc = 0.0;
      for (long q = s->cptr[j]; q < s->cptr[j + 1]; ++q) {
        int i = s->cidx[q];
        const double* blk = &s->K[(size_t)s->tpos[q] * dim * dim];  // block (i, j)
        for (int r = 0; r < dim; ++r) acc += blk[r * dim + c] * p[(size_t)i * dim + r];
      }
      y[(size_t)j * dim + c] = acc;
    }
  }
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

// strain energy density, particle_elastic_damage.h:89-104 (and the total
// of particle_fatigue_hcf.h:82-125, which returns the same sum)
double strain_energy(const lo_sys* s, int i) {
  const double Vm = s->particle_volume * s->nbonds[i] / s->nneighbors;
  double e = 0;
  for (int l = 0; l < NL; ++l) {
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b)
      if (s->blayer[b] == l) e += 0.5 * (s->Kn[b] * s->dLe[b] * s->dLe[b]) / Vm;
    e += 0.5 * s->tdle_tot[NL * (size_t)i + l] * s->dle_tot[NL * (size_t)i + l] / Vm;
  }
  return e;
}

// Assembly::updateStateVar -> Particle*::updateParticleStateVariables
void update_state(lo_sys* s) {
  const int ns = s->nstate;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s->n; ++i) {
    const double* P = &s->pp[(size_t)i * s->np];
    double* sv = &s->state[(size_t)i * ns];
    const double* svl = &s->state_last[(size_t)i * ns];
    if (s->law == 1) {  // particle_elastic_damage.h:150-161
      const double k0 = P[0], k1 = P[1];
      sv[0] = strain_energy(s, i);
      const double delta = sv[0] - svl[0];
      const double f = sv[0] - k1 * s->damage[i] - k0;
      s->ddot_local[i] = (f > 0 && delta > 0) ? (1 / k1) * delta : 0;
    } else if (s->law == 2) {  // particle_j2plasticity.h:78-140
      const double E = P[0], mu = P[1], sigmay = P[2], xi = P[3], H = P[4], A = P[5];
      double st[6];
      for (int j = 0; j < 6; ++j) st[j] = s->stress[6 * (size_t)i + j];
      const double sigma_m = 1.0 / 3.0 * (st[0] + st[1] + st[2]);
      for (int j = 0; j < 3; ++j) st[j] -= sigma_m;
      for (int j = 0; j < 6; ++j) st[j] -= sv[j + 1];
      double seq = 0;
      for (int j = 0; j < 6; ++j) seq += (j < 3 ? 1.0 : 2.0) * st[j] * st[j];
      seq = std::sqrt(3.0 / 2.0 * seq);
      const double yf = seq - (sigmay + (1.0 - xi) * H * sv[0]);
      const double G = E / 2 / (1 + mu);
      double dl = 0.0;
      if (yf > 0.0) dl = yf / (3 * G + H);
      sv[0] += dl;
      double dp[6] = {0, 0, 0, 0, 0, 0};
      for (int j = 0; j < 6; ++j)
        if (std::fabs(seq) > EPS_) {
          dp[j] = dl * 1.5 * st[j] / seq;
          sv[j + 1] += 2. / 3. * xi * H * dp[j];
        }
      for (int l = 0; l < NL; ++l)
        for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
          if (s->blayer[b] != l) continue;
          const double* c = &s->cs[3 * b];
          const double ddLp = s->dis[b] * (dp[0] * c[0] * c[0] + dp[1] * c[1] * c[1] + dp[2] * c[2] * c[2] +
                                           2 * dp[3] * c[1] * c[2] + 2 * dp[4] * c[0] * c[2] + 2 * dp[5] * c[0] * c[1]);
          s->dLp[b] += ddLp;
        }
      const double tri = seq > EPS_ ? sigma_m / seq : 0.0;
      s->ddot_local[i] = dl * (1.0 + A * tri);
    } else if (s->law == 3) {  // particle_fatigue_hcf.h:127-145
      const double A = P[0], B = P[1], d = P[2];
      const double u = strain_energy(s, i);
      sv[1] = std::min(u, sv[1]);
      sv[2] = std::max(u, sv[2]);
      sv[0] = std::max(sv[2], sv[0]);
      s->ddot_local[i] = (sv[2] - sv[1] > 0) ? A * std::pow(sv[0], B) * std::pow(sv[2] - sv[1], d) : 0;
    }
  }
}

// func_phi, lpm.h:45-49
inline double phi(double x, double L) { return std::pow(1 / (1 + std::pow(x / L, 8.0)), 2.0); }

// nonlocal damage rate, solver_static.h:34-54 / solver_fatigue.h:79-116
void nonlocal_rate(lo_sys* s) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s->n; ++i) {
    if (s->ptype[i] == s->undamaged) continue;
    double A = 0, D = 0;
    const double* xi = &s->x[3 * (size_t)i];
    for (long q = s->nl_ptr[i]; q < s->nl_ptr[i + 1]; ++q) {
      const int j = s->nl_idx[q];
      if (s->ptype[j] == s->undamaged) continue;
      const double* xj = &s->x[3 * (size_t)j];
      const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
      const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
      const double Vm = s->particle_volume * s->nbonds[j] / s->nneighbors;
      D += s->ddot_local[j] * phi(dis, s->nonlocal_L[i]) * Vm;
      A += phi(dis, s->nonlocal_L[i]) * Vm;
    }
    s->ddot_nl[i] = D / A;
  }
}

// SolverStatic::updateStaticDamage (solver_static.h:31-62)
bool static_damage(lo_sys* s) {
  nonlocal_rate(s);
  bool any = false;
  for (int i = 0; i < s->n; ++i) {
    if (s->ptype[i] == s->undamaged) continue;
    if (s->law == 0) {  // particle_elastic.h:52-68
      for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b)
        if (s->bstrain[b] >= s->crit[i] && std::abs(s->bdamage[b] - 1.0) > EPS_) {
          s->bdamage[b] = 1;
          any = true;
        }
    } else if (s->law == 1 || s->law == 2) {  // particle_elastic_damage.h:163-173, particle_j2plasticity.h:142-152
      const double thr = s->pp[(size_t)i * s->np + (s->law == 1 ? 2 : 6)];
      s->damage[i] += s->ddot_nl[i];
      if (s->damage[i] >= thr) s->damage[i] = 1;
      any = (std::abs(s->damage[i] - s->damage_last[i]) > 1e-3) || any;
    } else if (s->law == 4) {
      // softening bond law: kappa = max(kappa, (dis - dis0)/dis0);
      // d = 1 - (s_c/kappa)(alpha s_c - kappa)/((alpha - 1) s_c) between s_c
      // and alpha s_c, 0 below, 1 above; bdamage never decreases
      const double alpha = s->pp[(size_t)i * s->np];
      for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
        const double st = (s->dis[b] - s->dis0[b]) / s->dis0[b];
        const double k = std::max(s->bkappa[b], st);
        s->bkappa[b] = k;
        const double sc = s->bcrit[b];
        double d = 0.0;
        if (k >= alpha * sc)
          d = 1.0;
        else if (k > sc)
          d = 1.0 - (sc / k) * (alpha * sc - k) / ((alpha - 1.0) * sc);
        const double old = s->bdamage[b];
        if (d > old) {
          s->bdamage[b] = d;
          if (d - old > 1e-3) any = true;
        }
      }
    }
  }
  return any;
}

// SolverFatigue::updateFatigueDamage (solver_fatigue.h:75-126) with
// ParticleFatigueHCF::updateParticleFatigueDamage (particle_fatigue_hcf.h:147-160)
bool fatigue_damage(lo_sys* s, double dt) {
  nonlocal_rate(s);
  bool any = false;
  for (int i = 0; i < s->n; ++i) {
    if (s->ptype[i] == s->undamaged || s->law != 3) continue;
    const double thr = s->pp[(size_t)i * s->np + 3];
    s->damage[i] += s->ddot_nl[i] * dt;
    if (s->damage[i] >= thr) s->damage[i] = 1;
    s->state[(size_t)i * s->nstate + 1] = INT_MAX;
    s->state[(size_t)i * s->nstate + 2] = 0;
    any = (std::abs(s->damage[i] - s->damage_last[i]) > 1e-3) || any;
  }
  return any;
}

}  // namespace

extern "C" {

void lo_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

lo_sys* lo_create(int dim, int n, long nb, const double* xyz, const int* p1, const int* p2, const int* layer,
                  const double* Kn, const double* Tv, double particle_volume, int nneighbors, int* err) {
  *err = 0;
  if ((dim != 2 && dim != 3) || n <= 0 || nb < 0 || nneighbors <= 0) {
    *err = -1;
    return nullptr;
  }
  for (long b = 0; b < nb; ++b)
    if (p1[b] < 0 || p1[b] >= n || p2[b] < 0 || p2[b] >= n || layer[b] < 0 || layer[b] >= NL) {
      *err = -1;
      return nullptr;
    }
  lo_sys* s = new lo_sys();
  s->dim = dim;
  s->n = n;
  s->nb = nb;
  s->particle_volume = particle_volume;
  s->nneighbors = nneighbors;
  size_t N = (size_t)n;
  s->x.assign(xyz, xyz + 3 * N);
  s->x0 = s->x;
  s->xlast = s->x;
  s->pin.assign(3 * N, 0);
  s->pex.assign(3 * N, 0);
  s->stress.assign(6 * N, 0);
  s->dvis.assign(N, 0);
  s->dle_tot.assign(NL * N, 0);
  s->tdle_tot.assign(NL * N, 0);
  s->cs_sum.assign(NL * 3 * N, 0);
  s->damage.assign(N, 0);
  s->damage_last.assign(N, 0);
  s->ddot_local.assign(N, 0);
  s->mask.assign(3 * N, 0);
  s->state.assign(N * s->nstate, 0);
  s->state_last = s->state;
  s->crit.assign(N, 1.0);
  s->ptype.assign(N, 0);
  s->nonlocal_L.assign(N, 0.0);
  s->ddot_nl.assign(N, 0.0);
  s->nl_ptr.assign(N + 1, 0);
  // bond CSR: stable counting sort by (p1, layer)
  std::vector<long> cnt(N * NL + 1, 0);
  for (long b = 0; b < nb; ++b) cnt[(size_t)p1[b] * NL + layer[b] + 1]++;
  for (size_t k = 1; k < cnt.size(); ++k) cnt[k] += cnt[k - 1];
  s->bsrc.assign((size_t)nb, 0);
  {
    std::vector<long> pos(cnt.begin(), cnt.end() - 1);
    for (long b = 0; b < nb; ++b) s->bsrc[(size_t)pos[(size_t)p1[b] * NL + layer[b]]++] = b;
  }
  s->bptr.assign(N + 1, 0);
  for (size_t i = 0; i <= N; ++i) s->bptr[i] = cnt[i * NL];
  s->bp2.resize((size_t)nb);
  s->blayer.resize((size_t)nb);
  s->Kn.resize((size_t)nb);
  s->Tv.resize((size_t)nb);
  s->dis0.resize((size_t)nb);
  for (long b = 0; b < nb; ++b) {
    long src = s->bsrc[(size_t)b];
    s->bp2[(size_t)b] = p2[src];
    s->blayer[(size_t)b] = layer[src];
    s->Kn[(size_t)b] = Kn[src];
    s->Tv[(size_t)b] = Tv[src];
  }
  s->nbonds.assign(N, 0);
  for (int i = 0; i < n; ++i) s->nbonds[i] = (int)(s->bptr[i + 1] - s->bptr[i]);
  // initial bond length (Bond ctor, bond.h:59-72, from Particle::distanceTo)
  for (int i = 0; i < n; ++i)
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
      const double *xi = &s->x[3 * (size_t)i], *xj = &s->x[3 * (size_t)s->bp2[b]];
      double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
      s->dis0[b] = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  s->dis = s->dis0;
  s->dis_last = s->dis0;
  s->dL.assign((size_t)nb, 0);
  s->dLe.assign((size_t)nb, 0);
  s->dLp.assign((size_t)nb, 0);
  s->dLp_last.assign((size_t)nb, 0);
  s->bstrain.assign((size_t)nb, 0);
  s->cs.assign(3 * (size_t)nb, 0);
  s->bforce.assign((size_t)nb, 0);
  s->bforce_last.assign((size_t)nb, 0);
  s->bdamage.assign((size_t)nb, 0);
  s->bdamage_last.assign((size_t)nb, 0);
  // opposite bond: first bond of p2 in the same layer that points back
  // (particle.h:207-209)
  s->opp.assign((size_t)nb, -1);
  for (int i = 0; i < n; ++i)
    for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
      int j = s->bp2[b];
      for (long c = s->bptr[j]; c < s->bptr[j + 1]; ++c)
        if (s->blayer[c] == s->blayer[b] && s->bp2[c] == i) {
          s->opp[b] = c;
          break;
        }
      if (s->opp[b] < 0) {
        *err = -2;
        delete s;
        return nullptr;
      }
    }
  // conns (assembly.h:236-266): direct and two-hop neighbours per layer,
  // sorted and unique
  s->cptr.assign(N + 1, 0);
  std::vector<std::vector<int>> rows(N);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    std::vector<int>& c = rows[(size_t)i];
    for (int l = 0; l < NL; ++l)
      for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) {
        if (s->blayer[b] != l) continue;
        int k = s->bp2[b];
        c.push_back(k);
        for (long b2 = s->bptr[k]; b2 < s->bptr[k + 1]; ++b2)
          if (s->blayer[b2] == l) c.push_back(s->bp2[b2]);
      }
    std::sort(c.begin(), c.end());
    c.erase(std::unique(c.begin(), c.end()), c.end());
  }
  for (int i = 0; i < n; ++i) s->cptr[i + 1] = s->cptr[i] + (long)rows[(size_t)i].size();
  s->cidx.resize((size_t)s->cptr[N]);
  for (int i = 0; i < n; ++i) std::copy(rows[(size_t)i].begin(), rows[(size_t)i].end(), s->cidx.begin() + s->cptr[i]);
  compute_tpos(s);
  s->K.assign((size_t)s->cptr[N] * dim * dim, 0.0);
  return s;
}

void lo_destroy(lo_sys* s) { delete s; }
long lo_num_bonds(const lo_sys* s) { return s->nb; }
long lo_num_blocks(const lo_sys* s) { return (long)s->cidx.size(); }

void lo_get_topology(const lo_sys* s, long* bptr, int* bp2, int* blayer, long* bsrc, long* opp, long* cptr, int* cidx) {
  if (bptr) std::copy(s->bptr.begin(), s->bptr.end(), bptr);
  if (bp2) std::copy(s->bp2.begin(), s->bp2.end(), bp2);
  if (blayer) std::copy(s->blayer.begin(), s->blayer.end(), blayer);
  if (bsrc) std::copy(s->bsrc.begin(), s->bsrc.end(), bsrc);
  if (opp) std::copy(s->opp.begin(), s->opp.end(), opp);
  if (cptr) std::copy(s->cptr.begin(), s->cptr.end(), cptr);
  if (cidx) std::copy(s->cidx.begin(), s->cidx.end(), cidx);
}

static std::vector<double>* pfield(lo_sys* s, int f) {
  switch (f) {
    case LO_XYZ: return &s->x;
    case LO_XYZ0: return &s->x0;
    case LO_PIN: return &s->pin;
    case LO_PEX: return &s->pex;
    case LO_STRESS: return &s->stress;
    case LO_DVIS: return &s->dvis;
    case LO_DLE_TOT: return &s->dle_tot;
    case LO_TDLE_TOT: return &s->tdle_tot;
    case LO_CS_SUM: return &s->cs_sum;
    case LO_DAMAGE: return &s->damage;
    case LO_XYZ_LAST: return &s->xlast;
    case LO_STATE: return &s->state;
    case LO_DDOT_LOCAL: return &s->ddot_local;
  }
  return nullptr;
}
static std::vector<double>* bfield(lo_sys* s, int f) {
  switch (f) {
    case LO_BFORCE: return &s->bforce;
    case LO_BDAMAGE: return &s->bdamage;
    case LO_DLE: return &s->dLe;
    case LO_DIS: return &s->dis;
    case LO_BSTRAIN: return &s->bstrain;
    case LO_CS: return &s->cs;
    case LO_KN: return &s->Kn;
    case LO_TV: return &s->Tv;
    case LO_DIS0: return &s->dis0;
    case LO_DLP: return &s->dLp;
    case LO_SCRIT: return &s->bcrit;
    case LO_KAPPA: return &s->bkappa;
  }
  return nullptr;
}

void lo_get_particle(const lo_sys* s, int field, double* out) {
  auto* v = pfield(const_cast<lo_sys*>(s), field);
  if (v) std::copy(v->begin(), v->end(), out);
}
void lo_set_particle(lo_sys* s, int field, const double* in) {
  auto* v = pfield(s, field);
  if (v) std::copy(in, in + v->size(), v->begin());
}
void lo_get_bond(const lo_sys* s, int field, double* out) {
  auto* v = bfield(const_cast<lo_sys*>(s), field);
  if (v) std::copy(v->begin(), v->end(), out);
}
void lo_set_bond(lo_sys* s, int field, const double* in) {
  auto* v = bfield(s, field);
  if (v) std::copy(in, in + v->size(), v->begin());
}
void lo_set_mask(lo_sys* s, const int* mask) { std::copy(mask, mask + 3 * (size_t)s->n, s->mask.begin()); }

void lo_set_law(lo_sys* s, int law, const double* params, int nparams, int per_particle) {
  s->law = law;
  s->np = nparams;
  const size_t N = (size_t)s->n;
  s->pp.assign(N * (size_t)nparams, 0.0);
  for (size_t i = 0; i < N; ++i)
    for (int k = 0; k < nparams; ++k) s->pp[i * nparams + k] = per_particle ? params[i * nparams + k] : params[k];
  if (law == 0 && nparams >= 1)
    for (size_t i = 0; i < N; ++i) s->crit[i] = s->pp[i * nparams];
  if (law == 4) {
    const size_t B = s->bp2.size();
    s->bcrit.assign(B, 0.0);
    for (size_t i = 0; i < N; ++i)
      for (long b = s->bptr[i]; b < s->bptr[i + 1]; ++b) s->bcrit[(size_t)b] = s->pp[i * nparams + 1];
    s->bkappa.assign(B, 0.0);
    s->bkappa_last.assign(B, 0.0);
  }
  // state variables (constructors of the particle classes)
  s->nstate = law == 2 ? 7 : (law == 3 ? 3 : 1);
  s->state.assign(N * s->nstate, 0.0);
  if (law == 3)
    for (size_t i = 0; i < N; ++i) s->state[i * 3 + 1] = INT_MAX;
  s->state_last = s->state;
}

void lo_set_types(lo_sys* s, const int* types, int undamaged) {
  std::copy(types, types + s->n, s->ptype.begin());
  s->undamaged = undamaged;
}

void lo_set_nonlocal(lo_sys* s, const long* ptr, const int* idx, const double* L) {
  s->nl_ptr.assign(ptr, ptr + s->n + 1);
  s->nl_idx.assign(idx, idx + ptr[s->n]);
  s->nonlocal_L.assign(L, L + s->n);
}

void lo_update_state(lo_sys* s) { update_state(s); }
int lo_static_damage(lo_sys* s) { return static_damage(s) ? 1 : 0; }
int lo_fatigue_damage(lo_sys* s, double dt) { return fatigue_damage(s, dt) ? 1 : 0; }
void lo_get_ddot(const lo_sys* s, double* local, double* nonlocal) {
  if (local) std::copy(s->ddot_local.begin(), s->ddot_local.end(), local);
  if (nonlocal) std::copy(s->ddot_nl.begin(), s->ddot_nl.end(), nonlocal);
}
int lo_num_state(const lo_sys* s) { return s->nstate; }

void lo_update_geometry_force(lo_sys* s) {
  update_geometry(s);
  update_bond_force(s);
  update_particle_force(s);
}

void lo_residual(lo_sys* s, double* r, double* norm_r, double* norm_R) {
  const int dim = s->dim;
  double sr = 0, sR = 0;
  for (int i = 0; i < s->n; ++i)
    for (int k = 0; k < dim; ++k) {
      size_t q = 3 * (size_t)i + k;
      double v = (1 - s->mask[q]) * (s->pex[q] - s->pin[q]);
      if (r) r[(size_t)i * dim + k] = v;
      sr += v * v;
      if (s->mask[q] == 1) sR += s->pin[q] * s->pin[q];
    }
  if (norm_r) *norm_r = std::sqrt(sr);
  if (norm_R) *norm_R = std::sqrt(sR);
}

void lo_assemble(lo_sys* s, int sym, int bc) {
  assemble(s, sym);
  if (bc) apply_bc(s);
}

void lo_get_K(const lo_sys* s, double* vals) { std::copy(s->K.begin(), s->K.end(), vals); }

int lo_cg(lo_sys* s, const double* b, double* x, double tol, long maxit, long* iters, double* err) {
  const size_t n = (size_t)s->n * s->dim;
  const int dim = s->dim;
  if (maxit < 0) maxit = 2 * (long)n;
  std::vector<double> invd(n, 1.0);
  for (int i = 0; i < s->n; ++i)
    for (long q = s->cptr[i]; q < s->cptr[i + 1]; ++q)
      if (s->cidx[q] == i)
        for (int r = 0; r < dim; ++r) {
          double v = s->K[(size_t)q * dim * dim + r * dim + r];
          if (v != 0.0) invd[(size_t)i * dim + r] = 1.0 / v;
        }
  std::vector<double> r(b, b + n), p(n), z(n), tmp(n), xx(n, 0.0);
  double rhsNorm2 = dot(r, r);
  long it = 0;
  double resNorm2 = rhsNorm2;
  int status = 0;
  if (rhsNorm2 == 0.0) {
    *iters = 0;
    *err = 0.0;
    std::fill(x, x + n, 0.0);
    return 0;
  }
  const double threshold = std::max(tol * tol * rhsNorm2, 2.2250738585072014e-308);
  if (resNorm2 >= threshold) {
    for (size_t i = 0; i < n; ++i) p[i] = invd[i] * r[i];
    double absNew = dot(r, p);
    while (it < maxit) {
      apply_KT(s, p, tmp);
      double alpha = absNew / dot(p, tmp);
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)n; ++i) {
        xx[(size_t)i] += alpha * p[(size_t)i];
        r[(size_t)i] -= alpha * tmp[(size_t)i];
      }
      resNorm2 = dot(r, r);
      if (resNorm2 < threshold) break;
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)n; ++i) z[(size_t)i] = invd[(size_t)i] * r[(size_t)i];
      double absOld = absNew;
      absNew = dot(r, z);
      double beta = absNew / absOld;
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)n; ++i) p[(size_t)i] = z[(size_t)i] + beta * p[(size_t)i];
      ++it;
    }
  }
  *iters = it;
  *err = std::sqrt(resNorm2 / rhsNorm2);
  status = (*err <= tol) ? 0 : 1;
  std::copy(xx.begin(), xx.end(), x);
  return status;
}

int lo_newton(lo_sys* s, int max_iter, double tol, double cg_tol, long cg_maxit) {
  const int dim = s->dim;
  const size_t n = (size_t)s->n * dim;
  std::vector<double> r(n), d(n);
  lo_update_geometry_force(s);
  double nr, nR;
  lo_residual(s, r.data(), &nr, &nR);
  double mult = std::max(nr, nR);
  int ni = 0;
  while (nr > tol * mult) {
    if (++ni > max_iter) return max_iter;
    long it = 0;
    double err = 0;
    lo_cg(s, r.data(), d.data(), cg_tol, cg_maxit, &it, &err);
    for (int i = 0; i < s->n; ++i)
      for (int k = 0; k < dim; ++k) s->x[3 * (size_t)i + k] += d[(size_t)i * dim + k];
    lo_update_geometry_force(s);
    lo_residual(s, r.data(), &nr, &nR);
    s->log.push_back((double)it);
    s->log.push_back(err);
    s->log.push_back(nr);
  }
  return ni;
}

long lo_log_size(const lo_sys* s) { return (long)s->log.size() / 3; }
void lo_get_log(const lo_sys* s, double* out) { std::copy(s->log.begin(), s->log.end(), out); }
void lo_clear_log(lo_sys* s) { s->log.clear(); }

void lo_apply_disp_bc(lo_sys* s, const int* apply, const double* d) {
  for (size_t q = 0; q < 3 * (size_t)s->n; ++q)
    if (apply[q]) {
      s->x[q] += d[q];
      s->mask[q] = 1;
    }
}
void lo_add_pex(lo_sys* s, const double* f) {
  for (size_t q = 0; q < 3 * (size_t)s->n; ++q) s->pex[q] += f[q];
}

void lo_store_state(lo_sys* s) {
  s->xlast = s->x;
  s->damage_last = s->damage;
  s->state_last = s->state;
  s->dis_last = s->dis;
  s->bdamage_last = s->bdamage;
  s->bforce_last = s->bforce;
  s->dLp_last = s->dLp;
  s->bkappa_last = s->bkappa;
}
void lo_reset_state(lo_sys* s, int reset_xyz) {
  if (reset_xyz) s->x = s->xlast;
  s->damage = s->damage_last;
  s->state = s->state_last;
  s->dis = s->dis_last;
  s->bdamage = s->bdamage_last;
  s->bforce = s->bforce_last;
  s->dLp = s->dLp_last;
  s->bkappa = s->bkappa_last;
}

int lo_load_step(lo_sys* s, const int* apply, const double* d, const double* f, int sym, int bc_elim, int max_iter,
                 double tol, double cg_tol, long cg_maxit, int max_cuts) {
  std::vector<double> dd(d, d + 3 * (size_t)s->n), ff(f ? f : d, (f ? f : d) + 3 * (size_t)s->n);
  if (!f) std::fill(ff.begin(), ff.end(), 0.0);
  // A failed step is halved and solved twice (solver_static.h:79-87): the
  // pending list holds the scale of each sub-step still to solve, front first.
  std::vector<double> pending{1.0};
  int cuts = 0, last_n = 0;
  std::vector<double> ds(dd.size()), fs(ff.size());
  while (!pending.empty()) {
    double scale = pending.front();
    for (size_t q = 0; q < dd.size(); ++q) {
      ds[q] = dd[q] * scale;
      fs[q] = ff[q] * scale;
    }
    lo_add_pex(s, fs.data());
    lo_apply_disp_bc(s, apply, ds.data());
    int nn = 0;
    bool damaged = false;
    do {
      lo_assemble(s, sym, bc_elim != 0 ? 1 : 0);
      nn = lo_newton(s, max_iter, tol, cg_tol, cg_maxit);
      if (nn >= max_iter) break;
      damaged = false;
      update_state(s);  // Assembly::updateStateVar
      if (bc_elim != 1) damaged = static_damage(s);
      lo_store_state(s);
      if (damaged) lo_update_geometry_force(s);
    } while (damaged);
    if (nn >= max_iter) {
      if (++cuts > max_cuts) return -1;
      lo_reset_state(s, 1);
      pending.front() = 0.5 * scale;
      pending.insert(pending.begin(), 0.5 * scale);
      continue;
    }
    last_n = nn;
    pending.erase(pending.begin());
  }
  return last_n;
}

}  // extern "C"
