// Oracle driver around the UNMODIFIED LPM reference headers (test infrastructure).
//
// Built by oracle/Makefile only where the reference sources are present: the
// reference's include/ directory is put on the include path together with the
// Eigen/Boost stand-ins in oracle/shim/.  Nothing here is shipped or timed on
// the product path; the binary writes golden files that tests/golden/ keeps.
//
// It sets up lattices the way the reference examples do
// (examples/ex1_isoelasticity_2d_hex.cpp:9-93, ex1_isoelasticity_3d_sc.cpp:31-122)
// and dumps the quantities the GPU path must reproduce:
//   topology        Assembly::createBonds / updateConnections (assembly.h:212-266)
//   force state     Assembly::updateGeometry / updateForceState (assembly.h:132-191)
//   tangent         Stiffness::calcStiffness (stiffness.h:228-263)
//   BC elimination  Stiffness::updateStiffnessDispBC (stiffness.h:265-294)
//   linear solve    Solver::LPM_CG (solver.h:192-217)
//   load steps      SolverStatic::solveProblem (solver_static.h:64-149)
//
// Usage: ref_driver <case> <out.bin> [key=value ...]
#include "lpm.h"
#include "particle.h"
#include "assembly.h"
#include "utilities.h"
#include "stiffness.h"
#include "load_step.h"
#include "solver_static.h"
#include "solver_fatigue.h"

#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <string>

namespace {

// ---------------------------------------------------------------- output file
// Format: repeated records  "<name> <dtype> <count>\n" + raw little-endian data.
struct Out {
  FILE* f;
  explicit Out(const char* path) { f = std::fopen(path, "wb"); }
  ~Out() {
    if (f) std::fclose(f);
  }
  void f64(const std::string& name, const std::vector<double>& v) {
    std::fprintf(f, "%s f8 %zu\n", name.c_str(), v.size());
    std::fwrite(v.data(), sizeof(double), v.size(), f);
  }
  void i64(const std::string& name, const std::vector<long long>& v) {
    std::fprintf(f, "%s i8 %zu\n", name.c_str(), v.size());
    std::fwrite(v.data(), sizeof(long long), v.size(), f);
  }
  void scalar(const std::string& name, double x) { f64(name, std::vector<double>{x}); }
};

std::map<std::string, std::string> g_opts;
double opt(const char* k, double d) {
  auto it = g_opts.find(k);
  return it == g_opts.end() ? d : std::atof(it->second.c_str());
}
std::string opts(const char* k, const char* d) {
  auto it = g_opts.find(k);
  return it == g_opts.end() ? std::string(d) : it->second;
}

const int NL = 2;
typedef Particle<NL> P;

// Lattice point sets: same row/column rules as utilities.h createPlateHEX2D
// (alternating full / offset rows) and createCuboidSC3D, anchored at the origin.
std::vector<std::array<double, NDIM>> hex_points(int ncol, int nrow, double a) {
  std::vector<std::array<double, NDIM>> xyz;
  double hy = a * std::sqrt(3.0) / 2.0;
  for (int j = 0; j < nrow; ++j) {
    if (j % 2 == 0)
      for (int i = 0; i < ncol; ++i) xyz.push_back({a * i, hy * j, 0.0});
    else
      for (int i = 0; i < ncol - 1; ++i) xyz.push_back({a * (2 * i + 1) / 2.0, hy * j, 0.0});
  }
  return xyz;
}
std::vector<std::array<double, NDIM>> sc_points(int nx, int ny, int nz, double a) {
  std::vector<std::array<double, NDIM>> xyz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) xyz.push_back({a * i, a * j, a * k});
  return xyz;
}

// Kn/Tv as the reference computes them (el_mapping read through a column-major
// Map) or with the mapping rows applied as written ("row"), which gives the
// physical constants.  Both feed the same per-bond arrays.
void set_elastic(Assembly<NL>& ass, UnitCell& cell, bool plane_stress, double E, double nu, double crit,
                 const std::string& mapping) {
  for (P* p : ass.pt_sys) {
    auto* el = dynamic_cast<ParticleElastic<NL>*>(p);
    el->setParticleProperty(0.0, plane_stress, E, nu, crit);
  }
  if (mapping == "row") {
    double C11, C12, C44;
    if (!plane_stress) {
      C11 = E * (1.0 - nu) / (1.0 + nu) / (1.0 - 2.0 * nu);
      C12 = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
      C44 = E / 2.0 / (1.0 + nu);
    } else {
      C11 = E / (1.0 - nu) / (1.0 + nu);
      C12 = E * nu / (1.0 + nu) / (1.0 - nu);
      C44 = E / 2.0 / (1.0 + nu);
    }
    double Ce[3] = {C11, C12, C44}, k[3];
    for (int i = 0; i < 3; ++i) {
      // row i of the written data = column i of the column-major Map
      double s = 0;
      for (int j = 0; j < 3; ++j) s += cell.el_mapping(j, i) * Ce[j];
      k[i] = (cell.dim == 2 ? 1.0 : cell.radius) * s;
    }
    for (P* p : ass.pt_sys)
      for (int l = 0; l < NL; ++l)
        for (Bond<NL>* b : p->bond_layers[l]) {
          if (cell.lattice == LatticeType::Hexagon2D) {
            b->Kn = k[0];
            b->Tv = k[1];
          } else {
            b->Kn = k[b->layer];
            b->Tv = k[2];
          }
        }
  }
}

// ------------------------------------------------------------------ dumpers
void dump_topology(Out& o, Assembly<NL>& ass) {
  std::vector<long long> p1, p2, layer, cptr{0}, cidx, nbv;
  std::vector<double> Kn, Tv, dis0, xyz;
  for (P* p : ass.pt_sys) {
    for (int l = 0; l < NL; ++l)
      for (Bond<NL>* b : p->bond_layers[l]) {
        p1.push_back(b->p1->id);
        p2.push_back(b->p2->id);
        layer.push_back(b->layer);
        Kn.push_back(b->Kn);
        Tv.push_back(b->Tv);
        dis0.push_back(b->dis_initial);
      }
    for (P* q : p->conns) cidx.push_back(q->id);
    cptr.push_back((long long)cidx.size());
    nbv.push_back(p->nb);
    for (int k = 0; k < 3; ++k) xyz.push_back(p->xyz_initial[k]);
  }
  o.i64("bond_p1", p1);
  o.i64("bond_p2", p2);
  o.i64("bond_layer", layer);
  o.f64("Kn", Kn);
  o.f64("Tv", Tv);
  o.f64("dis0", dis0);
  o.i64("conn_ptr", cptr);
  o.i64("conn_idx", cidx);
  o.i64("nb", nbv);
  o.f64("xyz0", xyz);
}

void dump_state(Out& o, const std::string& pfx, Assembly<NL>& ass) {
  std::vector<double> xyz, Pin, stress, dv, dLe_t, TdLe_t, cs, bforce, bdamage, dLe;
  for (P* p : ass.pt_sys) {
    for (int k = 0; k < 3; ++k) xyz.push_back(p->xyz[k]);
    for (int k = 0; k < 3; ++k) Pin.push_back(p->Pin[k]);
    for (int k = 0; k < 6; ++k) stress.push_back(p->stress.size() == 6 ? p->stress[k] : 0.0);
    dv.push_back(p->damage_visual);
    for (int l = 0; l < NL; ++l) {
      dLe_t.push_back(p->dLe_total[l]);
      TdLe_t.push_back(p->TdLe_total[l]);
      cs.push_back(p->cs_sumx[l]);
      cs.push_back(p->cs_sumy[l]);
      cs.push_back(p->cs_sumz[l]);
      for (Bond<NL>* b : p->bond_layers[l]) {
        bforce.push_back(b->bforce);
        bdamage.push_back(b->bdamage);
        dLe.push_back(b->dLe);
      }
    }
  }
  o.f64(pfx + "xyz", xyz);
  o.f64(pfx + "Pin", Pin);
  o.f64(pfx + "stress", stress);
  o.f64(pfx + "damage_visual", dv);
  o.f64(pfx + "dLe_total", dLe_t);
  o.f64(pfx + "TdLe_total", TdLe_t);
  o.f64(pfx + "cs_sum", cs);
  o.f64(pfx + "bforce", bforce);
  o.f64(pfx + "bdamage", bdamage);
  o.f64(pfx + "dLe", dLe);
}

void dump_sparse(Out& o, const std::string& pfx, Eigen::SparseMatrix<double>& K) {
  if (!K.compressed) K.makeCompressed();
  std::vector<long long> outer(K.outer.begin(), K.outer.end()), inner(K.inner.begin(), K.inner.end());
  o.i64(pfx + "csc_outer", outer);
  o.i64(pfx + "csc_inner", inner);
  o.f64(pfx + "csc_values", K.values);
}

void perturb(Assembly<NL>& ass, double amp, unsigned seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  for (P* p : ass.pt_sys) {
    std::array<double, NDIM> d{amp * U(rng), amp * U(rng), p->cell.dim == 3 ? amp * U(rng) : 0.0};
    p->moveBy(d);
  }
}

// --------------------------------------------------------------------- cases
struct Setup {
  UnitCell cell;
  Assembly<NL>* ass;
  std::vector<P*> top, bottom, corner;
  int dim;
};

Setup build(const std::string& lattice) {
  double a = opt("a", 0.5);
  std::vector<std::array<double, NDIM>> xyz;
  LatticeType lt;
  if (lattice == "hex") {
    lt = LatticeType::Hexagon2D;
    xyz = hex_points((int)opt("ncol", 41), (int)opt("nrow", 41), a);
  } else {
    lt = LatticeType::SimpleCubic3D;
    int n = (int)opt("n", 6);
    xyz = sc_points((int)opt("nx", n), (int)opt("ny", n), (int)opt("nz", n), a);
  }
  Setup s{UnitCell(lt, a / 2.0), nullptr, {}, {}, {}, 0};
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (auto& p : xyz)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], p[k]);
      hi[k] = std::max(hi[k], p[k]);
    }
  std::array<double, 2 * NDIM> box{lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]};
  s.ass = new Assembly<NL>(xyz, box, s.cell, ParticleType::Elastic);
  s.dim = s.cell.dim;
  int ax = s.dim == 2 ? 1 : 2;  // loading axis
  double tolp = 1e-6 * a;
  for (P* p : s.ass->pt_sys) {
    if (p->xyz[ax] > hi[ax] - tolp) s.top.push_back(p);
    if (p->xyz[ax] < lo[ax] + tolp) s.bottom.push_back(p);
  }
  // bottom-left particle (lowest id on the bottom row)
  s.corner.push_back(s.bottom.front());
  bool ps = s.dim == 2 && opt("plane_stress", 1) != 0;
  double E = opt("E", s.dim == 2 ? 69e3 : 200e3), nu = opt("nu", 0.3);
  set_elastic(*s.ass, s.cell, ps, E, nu, opt("crit", 1.0), opts("mapping", "row"));
  return s;
}

std::vector<LoadStep<NL>> make_load(Setup& s, int nsteps, double du) {
  std::vector<LoadStep<NL>> load;
  for (int i = 0; i < nsteps; ++i) {
    LoadStep<NL> st;
    if (s.dim == 2) {
      // config-1 form: bottom y fixed, bottom-left x fixed, top y ramped
      st.dispBCs.push_back(DispBC<NL>(s.bottom, LoadMode::Relative, 'y', 0.0));
      st.dispBCs.push_back(DispBC<NL>(s.corner, LoadMode::Relative, 'x', 0.0));
      st.dispBCs.push_back(DispBC<NL>(s.top, LoadMode::Relative, 'y', du));
    } else {
      // config-2 form: bottom face clamped, top face pulled in z
      st.dispBCs.push_back(DispBC<NL>(s.bottom, LoadMode::Relative, 'x', 0.0));
      st.dispBCs.push_back(DispBC<NL>(s.bottom, LoadMode::Relative, 'y', 0.0));
      st.dispBCs.push_back(DispBC<NL>(s.bottom, LoadMode::Relative, 'z', 0.0));
      st.dispBCs.push_back(DispBC<NL>(s.top, LoadMode::Relative, 'z', du));
    }
    load.push_back(st);
  }
  return load;
}

// "kernels": topology, force state and tangent at a perturbed configuration,
// the BC-eliminated tangent, and one CG solve of each.
int case_kernels(Out& o, const std::string& lattice) {
  Setup s = build(lattice);
  dump_topology(o, *s.ass);
  perturb(*s.ass, opt("amp", 0.02) * opt("a", 0.5), (unsigned)opt("seed", 7));
  // damage a few bonds (bdamage feeds geometry, forces and the tangent)
  int every = (int)opt("damage_every", 0);
  if (every > 0) {
    long idx = 0;
    for (P* p : s.ass->pt_sys)
      for (int l = 0; l < NL; ++l)
        for (Bond<NL>* b : p->bond_layers[l]) {
          if (idx % every == 3) b->bdamage = (idx % (2 * every) == 3) ? 1.0 : 0.375;
          ++idx;
        }
  }
  Solver<NL> solv(*s.ass, StiffnessMode::Analytical, SolverMode::CG, "/dev/null", 30, 1e-5);
  auto load = make_load(s, 1, opt("du", 1e-3));
  solv.updateForceBC(load[0]);
  solv.updateDisplacementBC(load[0]);
  s.ass->updateGeometry();
  s.ass->updateForceState();
  solv.updateRR();
  dump_state(o, "s_", *s.ass);
  std::vector<long long> mask;
  for (P* p : s.ass->pt_sys)
    for (int k = 0; k < s.dim; ++k) mask.push_back(p->disp_constraint[k]);
  o.i64("mask", mask);
  o.f64("residual", solv.stiffness.residual.v);
  o.f64("reaction", solv.reaction_force.v);
  solv.stiffness.reset(s.ass->pt_sys);
  solv.stiffness.calcStiffness(s.ass->pt_sys);
  dump_sparse(o, "K_", solv.stiffness.K_matrix);
  Eigen::shim_cg_log().clear();
  solv.LPM_CG();
  o.f64("cg_disp", solv.disp.v);
  o.scalar("cg_iters", (double)Eigen::shim_cg_log().back().iterations);
  o.scalar("cg_error", Eigen::shim_cg_log().back().error);
  // BC elimination (fatigue path) and its solve
  solv.stiffness.updateStiffnessDispBC(s.ass->pt_sys);
  dump_sparse(o, "Kbc_", solv.stiffness.K_matrix);
  solv.LPM_CG();
  o.f64("cgbc_disp", solv.disp.v);
  o.scalar("cgbc_iters", (double)Eigen::shim_cg_log().back().iterations);
  o.scalar("cgbc_error", Eigen::shim_cg_log().back().error);
  return 0;
}

// "steps": SolverStatic::solveProblem over n displacement steps
int case_steps(Out& o, const std::string& lattice) {
  Setup s = build(lattice);
  dump_topology(o, *s.ass);
  s.ass->updateGeometry();
  s.ass->updateForceState();
  SolverStatic<NL> solv(-1, *s.ass, StiffnessMode::Analytical, SolverMode::CG, opts("dump", "/dev/null"),
                        (int)opt("max_iter", 30), opt("tol", 1e-5));
  // solver=fatigue: the static steps of SolverFatigue (solver_fatigue.h:243-298),
  // which apply Stiffness::updateStiffnessDispBC before each Newton solve.
  SolverFatigue<NL> solvf(-1, *s.ass, StiffnessMode::Analytical, SolverMode::CG, TimeMapMode::Linear, 1.0,
                          opts("dump", "/dev/null"), (int)opt("max_iter", 30), opt("tol", 1e-5));
  bool use_fatigue = opts("solver", "static") == "fatigue";
  int nsteps = (int)opt("steps", 10);
  std::vector<double> react, xyz_steps;
  std::vector<long long> cg_iters;
  int ax = s.dim == 2 ? 1 : 2;
  Eigen::shim_cg_log().clear();
  for (int i = 0; i < nsteps; ++i) {
    auto load = make_load(s, 1, opt("du", 1e-3));
    int start = i;
    if (use_fatigue)
      solvf.solveProblemStatic(load, start);
    else
      solv.solveProblem(load, start);
    double rt = 0, rb = 0;
    for (P* p : s.top) rt += p->Pin[ax];
    for (P* p : s.bottom) rb += p->Pin[ax];
    react.push_back(rt);
    react.push_back(rb);
    if (opt("all_xyz", 0) != 0 || i == nsteps - 1)
      for (P* p : s.ass->pt_sys)
        for (int k = 0; k < 3; ++k) xyz_steps.push_back(p->xyz[k]);
  }
  for (auto& r : Eigen::shim_cg_log()) cg_iters.push_back(r.iterations);
  o.f64("reaction_top_bottom", react);
  o.f64("xyz_steps", xyz_steps);
  o.i64("cg_iters", cg_iters);
  std::vector<double> cg_err;
  for (auto& r : Eigen::shim_cg_log()) cg_err.push_back(r.error);
  o.f64("cg_error", cg_err);
  dump_state(o, "f_", *s.ass);
  return 0;
}

// "laws": one update of each material law at a deformed, perturbed state.
//   law=damage  ParticleElasticDamage  (particle_elastic_damage.h)
//   law=j2      ParticleJ2Plasticity   (particle_j2plasticity.h)
//   law=hcf     ParticleFatigueHCF     (particle_fatigue_hcf.h)
// Sequence: updateGeometry/updateForceState, updateStateVar, the nonlocal
// damage update of SolverStatic (or SolverFatigue for hcf), and a second
// updateForceState that carries particle damage into the bonds.
void dump_laws_state(Out& o, const std::string& pfx, Assembly<NL>& ass) {
  std::vector<double> sv, ddl, ddn, dmg, dlp;
  for (P* p : ass.pt_sys) {
    for (double v : p->state_var) sv.push_back(v);
    ddl.push_back(p->Ddot_local);
    ddn.push_back(p->Ddot_nonlocal);
    dmg.push_back(p->damage);
    for (int l = 0; l < NL; ++l)
      for (Bond<NL>* b : p->bond_layers[l]) dlp.push_back(b->dLp);
  }
  o.f64(pfx + "state_var", sv);
  o.f64(pfx + "ddot_local", ddl);
  o.f64(pfx + "ddot_nonlocal", ddn);
  o.f64(pfx + "damage", dmg);
  o.f64(pfx + "dLp", dlp);
}

int case_laws(Out& o, const std::string& lattice) {
  double a = opt("a", 0.5);
  std::vector<std::array<double, NDIM>> xyz;
  LatticeType lt;
  if (lattice == "hex") {
    lt = LatticeType::Hexagon2D;
    xyz = hex_points((int)opt("ncol", 11), (int)opt("nrow", 11), a);
  } else {
    lt = LatticeType::SimpleCubic3D;
    int n = (int)opt("n", 5);
    xyz = sc_points(n, n, n, a);
  }
  UnitCell cell(lt, a / 2.0);
  std::array<double, 2 * NDIM> box{0, 1, 0, 1, 0, 1};
  std::string law = opts("law", "damage");
  ParticleType pt = law == "damage" ? ParticleType::ElasticDamage
                                    : (law == "j2" ? ParticleType::J2Plasticity : ParticleType::FatigueHCF);
  Assembly<NL> ass(xyz, box, cell, pt);
  bool ps = cell.dim == 2;
  double nl = opt("nonlocal_L", 0.6);
  int undamaged = (int)opt("undamaged", 4);
  int k = 0;
  for (P* p : ass.pt_sys) {
    p->type = (k % 9 == 4) ? undamaged : 0;  // a sprinkling of undamaged particles
    ++k;
    if (law == "damage")
      dynamic_cast<ParticleElasticDamage<NL>*>(p)->setParticleProperty(nl, ps, opt("E", 3.2e3), opt("nu", 0.28),
                                                                       opt("k0", 0.1936), opt("k1", 1.0), 10.0,
                                                                       opt("dthr", 0.99));
    else if (law == "j2")
      dynamic_cast<ParticleJ2Plasticity<NL>*>(p)->setParticleProperty(nl, ps, opt("E", 110e3), opt("nu", 0.34),
                                                                      opt("sigmay", 900.0), opt("xi", 0.3),
                                                                      opt("H", 1e3), opt("A", 0.5), 1.0);
    else
      dynamic_cast<ParticleFatigueHCF<NL>*>(p)->setParticleProperty(nl, ps, opt("E", 71.7e3), opt("nu", 0.306),
                                                                    opt("fA", 1.94e-4), opt("fB", 0.581),
                                                                    opt("fd", 1.079), opt("dthr", 1.0), 1.108);
  }
  ass.searchNonlocalNeighbors(opt("cutoff_ratio", 1.5));
  dump_topology(o, ass);
  std::vector<long long> types, nlp{0}, nli;
  for (P* p : ass.pt_sys) {
    types.push_back(p->type);
    for (P* q : p->neighbors_nonlocal) nli.push_back(q->id);
    nlp.push_back((long long)nli.size());
  }
  o.i64("types", types);
  o.i64("nl_ptr", nlp);
  o.i64("nl_idx", nli);
  // deformed state: uniform stretch along the loading axis plus noise
  int ax = cell.dim == 2 ? 1 : 2;
  auto deform = [&](double stretch, unsigned seed) {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    double amp = opt("amp", 0.01) * a;
    for (P* p : ass.pt_sys) {
      std::array<double, NDIM> x = p->xyz_initial;
      x[ax] *= (1.0 + stretch);
      x[0] += amp * U(rng);
      x[1] += amp * U(rng);
      if (cell.dim == 3) x[2] += amp * U(rng);
      p->moveTo(x);
    }
  };
  SolverStatic<NL> ss(undamaged, ass, StiffnessMode::Analytical, SolverMode::CG, "/dev/null", 30, 1e-5);
  SolverFatigue<NL> sf(undamaged, ass, StiffnessMode::Analytical, SolverMode::CG, TimeMapMode::Linear, 1.0,
                       "/dev/null", 30, 1e-5);
  double s1 = opt("stretch", 0.015);
  deform(s1, 11);
  ass.updateGeometry();
  ass.updateForceState();
  dump_state(o, "a_", ass);
  ass.updateStateVar();
  dump_laws_state(o, "a_", ass);
  if (law == "hcf") {
    // a second, smaller deformation inside the same cycle, then the cycle's damage
    deform(0.3 * s1, 12);
    ass.updateGeometry();
    ass.updateForceState();
    dump_state(o, "b_", ass);
    ass.updateStateVar();
    dump_laws_state(o, "b_", ass);
    bool any = sf.updateFatigueDamage(opt("dNdt", 1000));
    o.scalar("any_damaged", any ? 1.0 : 0.0);
  } else {
    bool any = ss.updateStaticDamage();
    o.scalar("any_damaged", any ? 1.0 : 0.0);
  }
  dump_laws_state(o, "c_", ass);
  ass.updateGeometry();
  ass.updateForceState();
  dump_state(o, "c_", ass);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <kernels-hex|kernels-sc|steps-hex|steps-sc> <out.bin> [k=v ...]\n", argv[0]);
    return 2;
  }
  for (int i = 3; i < argc; ++i) {
    const char* eq = std::strchr(argv[i], '=');
    if (eq) g_opts[std::string(argv[i], eq - argv[i])] = eq + 1;
  }
  std::string c = argv[1];
  Out o(argv[2]);
  if (!o.f) return 3;
  if (c == "kernels-hex") return case_kernels(o, "hex");
  if (c == "kernels-sc") return case_kernels(o, "sc");
  if (c == "steps-hex") return case_steps(o, "hex");
  if (c == "steps-sc") return case_steps(o, "sc");
  if (c == "laws-hex") return case_laws(o, "hex");
  if (c == "laws-sc") return case_laws(o, "sc");
  std::fprintf(stderr, "unknown case %s\n", c.c_str());
  return 2;
}
