// Assembly: the particle system (assembly.h:40-425 of the reference) with
// its hot methods on the GPU.
//
// The host keeps the reference's objects (Particle*, Bond*) so that example
// code reads and writes the same members.  The first device operation
// creates one device lattice from them (lpm_create); from then on the
// device holds the state and Assembly copies positions, forces, stress,
// damage and state variables back into the particles after every device
// update (bond state on demand, pullBonds()).  Copies of an Assembly share
// the device lattice, as copies of the reference's Assembly share their
// particles.
#pragma once

#include <memory>

#include "dump_writer.h"
#include "particle.h"

template <int nlayer>
class Assembly {
 public:
  ParticleType ptype;
  int nparticle{0};
  std::vector<Particle<nlayer>*> pt_sys;
  std::array<double, 2 * NDIM> box{};

  Assembly(std::vector<std::array<double, NDIM>>& p_xyz, std::array<double, 2 * NDIM>& p_box, UnitCell& p_cell,
           const ParticleType& p_ptype)
      : ptype(p_ptype), box(p_box) {
    createParticles(p_xyz, p_cell);
    createBonds();
    nparticle = (int)pt_sys.size();
  }
  Assembly(const std::string& dumpFile, UnitCell& p_cell, const ParticleType& p_ptype) : ptype(p_ptype) {
    printf("Reading data ...\n");
    readDump(dumpFile, p_cell);
    createBonds();
  }
  Assembly(const std::string& dumpFile, const std::string& bondFile, UnitCell& p_cell, const ParticleType& p_ptype)
      : ptype(p_ptype) {
    printf("Reading data ...\n");
    readDump(dumpFile, p_cell);
    readBond(bondFile);
    for (Particle<nlayer>* p1 : pt_sys) p1->nb = (int)p1->neighbors.size();
  }

  // ------------------------------------------------------------ set-up
  void createParticles(std::vector<std::array<double, NDIM>>& p_xyz, UnitCell& cell) {
    for (auto x : p_xyz) pt_sys.push_back(newParticle(x[0], x[1], x[2], cell, -1));
  }

  // Assembly::createBonds (assembly.h:212-234), searched on the device
  // (lpm_find_bonds: a cell grid with the reference's distance arithmetic,
  // bonds in ascending partner id per particle)
  void createBonds() {
    const int n = (int)pt_sys.size();
    if (!n) return;
    const UnitCell& c = pt_sys[0]->cell;
    std::vector<double> x(3 * (size_t)n);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) x[3 * (size_t)i + k] = pt_sys[(size_t)i]->xyz[(size_t)k];
    int64_t nb = 0;
    lpm_check(lpm_find_bonds(n, x.data(), c.neighbor_cutoff[0], c.neighbor_cutoff[1], 0, nullptr, nullptr, nullptr,
                             &nb),
              "lpm_find_bonds");
    std::vector<int> p1((size_t)nb), p2((size_t)nb), layer((size_t)nb);
    lpm_check(lpm_find_bonds(n, x.data(), c.neighbor_cutoff[0], c.neighbor_cutoff[1], nb, p1.data(), p2.data(),
                             layer.data(), &nb),
              "lpm_find_bonds");
    for (int64_t b = 0; b < nb; ++b) {
      Particle<nlayer>* a = pt_sys[(size_t)p1[(size_t)b]];
      Particle<nlayer>* q = pt_sys[(size_t)p2[(size_t)b]];
      a->bond_layers[layer[(size_t)b]].push_back(new Bond<nlayer>(a, q, layer[(size_t)b], a->distanceTo(q)));
      a->neighbors.push_back(q);
    }
    for (Particle<nlayer>* p : pt_sys) p->nb = (int)p->neighbors.size();
  }

  // Assembly::updateConnections (assembly.h:236-266), on the host.  The
  // device builds its own copy of this pattern; call this only when the
  // host lists are wanted.
  void updateConnections() {
    for (Particle<nlayer>* p1 : pt_sys) {
      p1->conns.clear();
      for (int i = 0; i < nlayer; i++)
        for (auto* fw : p1->bond_layers[i]) {
          p1->conns.push_back(fw->p2);
          for (auto* bw : fw->p2->bond_layers[i]) p1->conns.push_back(bw->p2);
        }
      std::sort(p1->conns.begin(), p1->conns.end(),
                [](Particle<nlayer>* a, Particle<nlayer>* b) { return a->id < b->id; });
      p1->conns.erase(std::unique(p1->conns.begin(), p1->conns.end()), p1->conns.end());
      p1->nconn = (int)p1->conns.size();
      auto cur = std::find(p1->conns.begin(), p1->conns.end(), p1);
      p1->nconn_largeq = (int)std::distance(cur, p1->conns.end());
    }
  }

  // Assembly::searchNonlocalNeighbors (assembly.h:117-130) on the device
  void searchNonlocalNeighbors(double cutoff_ratio) {
    const int n = (int)pt_sys.size();
    if (!n) return;
    std::vector<double> x(3 * (size_t)n), r((size_t)n);
    for (int i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) x[3 * (size_t)i + k] = pt_sys[(size_t)i]->xyz[(size_t)k];
      r[(size_t)i] = cutoff_ratio * (pt_sys[(size_t)i]->nonlocal_L);
    }
    std::vector<int64_t> ptr((size_t)n + 1);
    int64_t total = 0;
    lpm_check(lpm_find_neighbors(n, x.data(), r.data(), 0, ptr.data(), nullptr, &total), "lpm_find_neighbors");
    std::vector<int> idx((size_t)total);
    lpm_check(lpm_find_neighbors(n, x.data(), r.data(), total, ptr.data(), idx.data(), &total), "lpm_find_neighbors");
    for (int i = 0; i < n; ++i)
      for (int64_t q = ptr[(size_t)i]; q < ptr[(size_t)i + 1]; ++q)
        pt_sys[(size_t)i]->neighbors_nonlocal.push_back(pt_sys[(size_t)idx[(size_t)q]]);
    g_->nonlocal_dirty = true;
  }

  std::map<int, Particle<nlayer>*> toMap() {
    std::map<int, Particle<nlayer>*> m;
    for (Particle<nlayer>* pt : pt_sys) m[pt->id] = pt;
    return m;
  }

  // --------------------------------------------------- device operations
  // Assembly::updateGeometry + updateForceState (assembly.h:132-191): one
  // device pass computes both, so either call brings the force state up to
  // date.
  void updateGeometry() { updateForceState(); }
  // The device force pass without the copy back to the particles, for the
  // solvers' inner loops; pullParticles() brings the particles up to date.
  void refreshForceState() { lpm_check(lpm_update_geometry_force(device()), "lpm_update_geometry_force"); }
  void updateForceState() {
    lpm_check(lpm_update_geometry_force(device()), "lpm_update_geometry_force");
    pullParticles();
  }
  void storeStateVar() {
    lpm_check(lpm_store_state(device()), "lpm_store_state");
    for (Particle<nlayer>* pt : pt_sys) {
      pt->xyz_last = pt->xyz;
      pt->damage_last = pt->damage;
      pt->state_var_last = pt->state_var;
    }
  }
  void resetStateVar(bool reset_xyz) {
    lpm_check(lpm_reset_state(device(), reset_xyz ? 1 : 0), "lpm_reset_state");
    pullParticles();
  }
  void updateStateVar() {
    lpm_check(lpm_update_state(device()), "lpm_update_state");
    pullParticles();
  }

  // -------------------------------------------------------------- files
  void writeBond(const std::string& bondFile) {
    pullBonds();
    FILE* f = fopen(bondFile.c_str(), "w+");
    for (Particle<nlayer>* pt : pt_sys)
      for (int i = 0; i < nlayer; ++i)
        for (Bond<nlayer>* bd : pt->bond_layers[i]) fprintf(f, "%d %d %d %d\n", bd->id, bd->layer, bd->p1->id, bd->p2->id);
    fclose(f);
  }
  void writeConfigurationDump(const std::string& dumpFile) {
    FILE* f = fopen(dumpFile.c_str(), "w+");
    header(f, 0);
    fprintf(f, "ITEM: ATOMS id type x y z\n");
    for (auto pt : pt_sys) fprintf(f, "%d %d %.4e %.4e %.4e \n", pt->id, pt->type, pt->xyz[0], pt->xyz[1], pt->xyz[2]);
    fclose(f);
  }
  // LAMMPS dump, the columns of assembly.h:309-335.  The particle columns
  // are copied here and written by the asynchronous dump writer
  // (dump_writer.h), so the load steps go on while the text is formatted and
  // appended; flushDumps() waits for it.
  void writeDump(const std::string& dumpFile, int step) {
    DumpRecord r;
    r.file = dumpFile;
    r.step = step;
    r.nparticle = nparticle;
    for (int k = 0; k < 6; ++k) r.box[k] = box[(size_t)k];
    r.id.reserve(pt_sys.size());
    r.type.reserve(pt_sys.size());
    r.cols.reserve(pt_sys.size() * DumpWriter::kCols);
    for (auto pt : pt_sys) {
      r.id.push_back(pt->id);
      r.type.push_back(pt->type);
      const double c[DumpWriter::kCols] = {pt->xyz[0], pt->xyz[1], pt->xyz[2], pt->xyz[0] - pt->xyz_initial[0],
                                           pt->xyz[1] - pt->xyz_initial[1], pt->xyz[2] - pt->xyz_initial[2],
                                           pt->stress[0], pt->stress[1], pt->stress[2], pt->stress[3], pt->stress[4],
                                           pt->stress[5], pt->damage, pt->damage_visual, pt->state_var[0]};
      r.cols.insert(r.cols.end(), c, c + DumpWriter::kCols);
    }
    DumpWriter::instance().submit(std::move(r));
  }
  // readDump (assembly.h:337-388): id type x y z, ids 0..N-1
  void readDump(const std::string& dumpFile, UnitCell& cell) {
    FILE* f = fopen(dumpFile.c_str(), "r");
    if (!f) {
      printf("'%s' does not exist!\n", dumpFile.c_str());
      exit(1);
    }
    char line[500];
    for (int k = 0; k < 3; ++k)
      if (!fgets(line, sizeof line, f)) break;
    if (fscanf(f, "%d\n", &nparticle) != 1) nparticle = 0;
    if (!fgets(line, sizeof line, f)) line[0] = 0;
    for (int k = 0; k < 3; ++k)
      if (fscanf(f, "%lf %lf\n", &box[2 * k], &box[2 * k + 1]) != 2) break;
    if (!fgets(line, sizeof line, f)) line[0] = 0;
    int id, type;
    double x[NDIM];
    while (fscanf(f, "%d %d %lf %lf %lf", &id, &type, &x[0], &x[1], &x[2]) > 0) {
      Particle<nlayer>* pt = newParticle(x[0], x[1], x[2], cell, type);
      pt->id = id;
      pt_sys.push_back(pt);
    }
    fclose(f);
  }
  // readBond (assembly.h:390-424): "id layer p1 p2" per directed bond
  void readBond(const std::string& bondFile) {
    FILE* f = fopen(bondFile.c_str(), "r");
    if (!f) {
      printf("'%s' does not exist!\n", bondFile.c_str());
      exit(1);
    }
    std::map<int, Particle<nlayer>*> m = toMap();
    int id, layer, a, b;
    while (fscanf(f, "%d %d %d %d", &id, &layer, &a, &b) == 4) {
      Particle<nlayer>*p1 = m[a], *p2 = m[b];
      p1->bond_layers[layer].push_back(new Bond<nlayer>(p1, p2, layer, p1->distanceTo(p2)));
      p1->neighbors.push_back(p2);
    }
    fclose(f);
  }

  // ------------------------------------------------------ device glue
  // The device lattice, created from the host objects on first use.
  lpm_handle* device() {
    if (!g_->h) attach();
    if (g_->nonlocal_dirty) uploadNonlocal();
    return g_->h;
  }
  // Device group id of a BC group (registered once per distinct id list).
  int groupId(const std::vector<Particle<nlayer>*>& group) {
    std::vector<int> ids;
    for (Particle<nlayer>* p : group) ids.push_back(p->id);
    auto it = g_->groups.find(ids);
    if (it != g_->groups.end()) return it->second;
    int gid = -1;
    lpm_check(lpm_add_group(device(), ids.data(), (int)ids.size(), &gid), "lpm_add_group");
    g_->groups[ids] = gid;
    return gid;
  }
  void setUndamagedType(int t) {
    std::vector<int> types;
    for (Particle<nlayer>* p : pt_sys) types.push_back(p->type);
    lpm_check(lpm_set_types(device(), types.data(), t), "lpm_set_types");
  }
  // device -> particles: positions, forces, stress, damage, state variables
  void pullParticles() {
    lpm_handle* h = g_->h;
    if (!h) return;
    const size_t n = pt_sys.size();
    std::vector<double> x(3 * n), pin(3 * n), st(6 * n), dm(n), dv(n), dl(2 * n);
    lpm_check(lpm_download(h, LPM_F_XYZ, x.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_F_PIN, pin.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_F_STRESS, st.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_F_DAMAGE, dm.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_F_DVIS, dv.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_F_DLE_TOT, dl.data()), "lpm_download");
    const size_t ns = pt_sys.empty() ? 0 : pt_sys[0]->state_var.size();
    std::vector<double> sv(ns * n);
    if (ns) lpm_check(lpm_download(h, LPM_F_STATE, sv.data()), "lpm_download");
    for (size_t i = 0; i < n; ++i) {
      Particle<nlayer>* p = pt_sys[i];
      for (int k = 0; k < 3; ++k) {
        p->xyz[(size_t)k] = x[3 * i + k];
        p->Pin[(size_t)k] = pin[3 * i + k];
      }
      for (int k = 0; k < 6; ++k) p->stress[(size_t)k] = st[6 * i + k];
      p->damage = dm[i];
      p->damage_visual = dv[i];
      for (int l = 0; l < nlayer && l < 2; ++l) p->dLe_total[(size_t)l] = dl[2 * i + l];
      for (size_t k = 0; k < ns; ++k) p->state_var[k] = sv[i * ns + k];
    }
  }
  // device -> bonds: force, damage, length, stretch, plastic stretch
  void pullBonds() {
    lpm_handle* h = g_->h;
    if (!h) return;
    const size_t nb = (size_t)g_->nb;
    std::vector<double> f(nb), d(nb), dis(nb), dle(nb), dlp(nb), bs(nb), cs(3 * nb);
    lpm_check(lpm_download(h, LPM_B_BFORCE, f.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_B_BDAMAGE, d.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_B_DIS, dis.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_B_DLE, dle.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_B_DLP, dlp.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_B_BSTRAIN, bs.data()), "lpm_download");
    lpm_check(lpm_download(h, LPM_B_CS, cs.data()), "lpm_download");
    size_t b = 0;  // device order = bond_layers order
    for (Particle<nlayer>* pt : pt_sys)
      for (int l = 0; l < nlayer; ++l)
        for (Bond<nlayer>* bd : pt->bond_layers[l]) {
          bd->bforce = f[b];
          bd->bdamage = d[b];
          bd->dis = dis[b];
          bd->dLe = dle[b];
          bd->dLp = dlp[b];
          bd->bstrain = bs[b];
          bd->csx = cs[3 * b];
          bd->csy = cs[3 * b + 1];
          bd->csz = cs[3 * b + 2];
          ++b;
        }
  }

 private:
  struct GpuState {
    lpm_handle* h = nullptr;
    int64_t nb = 0;
    bool nonlocal_dirty = false;
    std::map<std::vector<int>, int> groups;
    ~GpuState() {
      if (h) lpm_destroy(h);
    }
  };
  std::shared_ptr<GpuState> g_ = std::make_shared<GpuState>();

  Particle<nlayer>* newParticle(double x, double y, double z, UnitCell& cell, int type) {
    Particle<nlayer>* pt = nullptr;
    if (ptype == ParticleType::Elastic)
      pt = type < 0 ? new ParticleElastic<nlayer>(x, y, z, cell) : new ParticleElastic<nlayer>(x, y, z, cell, type);
    if (ptype == ParticleType::ElasticDamage)
      pt = type < 0 ? new ParticleElasticDamage<nlayer>(x, y, z, cell)
                    : new ParticleElasticDamage<nlayer>(x, y, z, cell, type);
    if (ptype == ParticleType::J2Plasticity)
      pt = type < 0 ? new ParticleJ2Plasticity<nlayer>(x, y, z, cell)
                    : new ParticleJ2Plasticity<nlayer>(x, y, z, cell, type);
    if (ptype == ParticleType::FatigueHCF)
      pt = type < 0 ? new ParticleFatigueHCF<nlayer>(x, y, z, cell) : new ParticleFatigueHCF<nlayer>(x, y, z, cell, type);
    return pt;
  }

  void header(FILE* f, int step) {
    fprintf(f, "ITEM: TIMESTEP\n%d\nITEM: NUMBER OF ATOMS\n%d\nITEM: BOX BOUNDS pp pp pp\n", step, nparticle);
    fprintf(f, "%8.8f %8.8f\n%8.8f %8.8f\n%8.8f %8.8f\n", box[0], box[1], box[2], box[3], box[4], box[5]);
  }

  void attach() {
    const size_t n = pt_sys.size();
    std::vector<double> x0(3 * n), Kn, Tv;
    std::vector<int> p1, p2, layer;
    for (size_t i = 0; i < n; ++i) {
      Particle<nlayer>* pt = pt_sys[i];
      if (pt->id != (int)i) {
        fprintf(stderr, "liblpmgpu: particle ids must be 0..N-1 in pt_sys order\n");
        exit(1);
      }
      for (int k = 0; k < 3; ++k) x0[3 * i + k] = pt->xyz_initial[(size_t)k];
      for (int l = 0; l < nlayer; ++l)
        for (Bond<nlayer>* bd : pt->bond_layers[l]) {
          p1.push_back(pt->id);
          p2.push_back(bd->p2->id);
          layer.push_back(l);
          Kn.push_back(bd->Kn);
          Tv.push_back(bd->Tv);
        }
    }
    const UnitCell& c = pt_sys[0]->cell;
    lpm_check(lpm_create(c.dim, (int)n, (int64_t)p1.size(), x0.data(), p1.data(), p2.data(), layer.data(), Kn.data(),
                         Tv.data(), c.particle_volume, c.nneighbors, &g_->h),
              "lpm_create");
    g_->nb = (int64_t)p1.size();
    if (lpm_gpu_options().precond != LPM_PRECOND_JACOBI)
      lpm_check(lpm_set_preconditioner(g_->h, lpm_gpu_options().precond, lpm_gpu_options().precond_box),
                "lpm_set_preconditioner");
    // material law and per-particle parameters
    std::vector<double> prm, all;
    pt_sys[0]->gpuParams(prm);
    const int np = (int)prm.size();
    for (Particle<nlayer>* pt : pt_sys) {
      pt->gpuParams(prm);
      all.insert(all.end(), prm.begin(), prm.end());
    }
    lpm_check(lpm_set_law(g_->h, pt_sys[0]->gpuLaw(), all.data(), np, 1), "lpm_set_law");
    // current state: positions, loads, constraints, damage, state variables
    std::vector<double> x(3 * n), pex(3 * n), dm(n), st;
    std::vector<int> mask(3 * n), types(n);
    for (size_t i = 0; i < n; ++i) {
      Particle<nlayer>* pt = pt_sys[i];
      for (int k = 0; k < 3; ++k) {
        x[3 * i + k] = pt->xyz[(size_t)k];
        pex[3 * i + k] = pt->Pex[(size_t)k];
        mask[3 * i + k] = pt->disp_constraint[(size_t)k];
      }
      dm[i] = pt->damage;
      types[i] = pt->type;
      st.insert(st.end(), pt->state_var.begin(), pt->state_var.end());
    }
    lpm_check(lpm_upload(g_->h, LPM_F_XYZ, x.data()), "lpm_upload");
    lpm_check(lpm_upload(g_->h, LPM_F_PEX, pex.data()), "lpm_upload");
    lpm_check(lpm_upload(g_->h, LPM_F_DAMAGE, dm.data()), "lpm_upload");
    lpm_check(lpm_upload(g_->h, LPM_F_STATE, st.data()), "lpm_upload");
    lpm_check(lpm_set_mask(g_->h, mask.data()), "lpm_set_mask");
    lpm_check(lpm_set_types(g_->h, types.data(), INT_MIN), "lpm_set_types");
    // bond damage and plastic stretch the host may have set
    std::vector<double> bd, lp;
    for (Particle<nlayer>* pt : pt_sys)
      for (int l = 0; l < nlayer; ++l)
        for (Bond<nlayer>* b : pt->bond_layers[l]) {
          bd.push_back(b->bdamage);
          lp.push_back(b->dLp);
        }
    if (!bd.empty()) {
      lpm_check(lpm_upload(g_->h, LPM_B_BDAMAGE, bd.data()), "lpm_upload");
      lpm_check(lpm_upload(g_->h, LPM_B_DLP, lp.data()), "lpm_upload");
    }
    lpm_check(lpm_store_state(g_->h), "lpm_store_state");
    g_->nonlocal_dirty = true;
  }

  void uploadNonlocal() {
    g_->nonlocal_dirty = false;
    bool any = false;
    for (Particle<nlayer>* p : pt_sys) any = any || !p->neighbors_nonlocal.empty();
    if (!any || !g_->h) return;
    std::vector<int64_t> ptr{0};
    std::vector<int> idx;
    std::vector<double> L;
    for (Particle<nlayer>* p : pt_sys) {
      for (Particle<nlayer>* q : p->neighbors_nonlocal) idx.push_back(q->id);
      ptr.push_back((int64_t)idx.size());
      L.push_back(p->nonlocal_L);
    }
    lpm_check(lpm_set_nonlocal(g_->h, ptr.data(), idx.data(), L.data()), "lpm_set_nonlocal");
  }
};
