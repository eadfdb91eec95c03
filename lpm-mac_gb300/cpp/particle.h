// Particle and its material-law subclasses: host view of the particle state
// (particle.h:13-281, particle_elastic.h, particle_elastic_damage.h,
// particle_j2plasticity.h, particle_fatigue_hcf.h of the reference).
//
// setParticleProperty computes the bond constants exactly as the reference
// does (el_mapping applied to (C11, C12, C44)); the force, stress, state and
// damage updates run on the GPU through Assembly.  Each class reports the
// law id and parameters the device needs.
#pragma once

#include "bond.h"
#include "unit_cell.h"

template <int nlayer>
class Particle {
 protected:
  static int _ID;

 public:
  int id{0};
  int type{0};
  int nconn_largeq{0};
  int nb{0}, nconn{0};
  double nonlocal_L{0.};
  double damage_last{0.}, damage{0.}, damage_visual{0.};
  double Ddot_local{0}, Ddot_nonlocal{0};
  UnitCell cell;
  std::vector<double> state_var, state_var_last;
  std::array<int, NDIM> disp_constraint{0};
  std::array<double, nlayer> TdLe_total{}, dLe_total{}, cs_sumx{}, cs_sumy{}, cs_sumz{};
  std::array<double, NDIM> xyz, xyz_initial, xyz_last;
  std::array<double, NDIM> Pin{0}, Pex{0};
  std::array<std::vector<Bond<nlayer>*>, nlayer> bond_layers;
  std::vector<Particle<nlayer>*> neighbors;
  std::vector<Particle<nlayer>*> conns;
  std::vector<Particle<nlayer>*> neighbors_nonlocal;
  std::vector<double> stress, strain;

  Particle(const double& x, const double& y, const double& z, const UnitCell& c, const int& p_type) : cell{c} {
    xyz = {x, y, z};
    xyz_initial = xyz_last = xyz;
    type = p_type;
    id = _ID++;
    stress.assign(2 * NDIM, 0.0);
  }
  Particle(const double& x, const double& y, const double& z, const UnitCell& c) : cell{c} {
    xyz = {x, y, z};
    xyz_initial = xyz_last = xyz;
    id = _ID++;
    stress.assign(2 * NDIM, 0.0);
  }
  virtual ~Particle() {}

  void moveTo(const double& nx, const double& ny, const double& nz) { xyz = {nx, ny, nz}; }
  void moveTo(const std::array<double, NDIM>& n) { xyz = n; }
  void moveBy(const std::array<double, NDIM>& d) { xyz = {xyz[0] + d[0], xyz[1] + d[1], xyz[2] + d[2]}; }
  double distanceTo(Particle<nlayer>* A) {
    return sqrt(pow((xyz[0] - A->xyz[0]), 2) + pow((xyz[1] - A->xyz[1]), 2) + pow((xyz[2] - A->xyz[2]), 2));
  }
  bool operator==(const Particle<nlayer>& o) { return id == o.id; }
  // particle.h:242-256
  bool hasAFEMneighbor(Particle<nlayer>* pj, int layer) {
    for (Bond<nlayer>* b1 : bond_layers[layer]) {
      if (b1->p2->id == pj->id) return true;
      for (Bond<nlayer>* b2 : b1->p2->bond_layers[layer])
        if (b2->p2->id == pj->id) return true;
    }
    return false;
  }

  // the device law this class runs (LPM_LAW_*) and its parameters
  virtual int gpuLaw() const { return LPM_LAW_ELASTIC; }
  virtual void gpuParams(std::vector<double>& out) const { out = {1.0}; }

 protected:
  // ParticleX::setParticleProperty: KnTv = [r] el_mapping (C11, C12, C44)
  void setBondConstants(bool is_plane_stress, double E, double mu, const double* C = nullptr) {
    Eigen::VectorXd KnTv(NDIM), Ce(NDIM);
    if (C) {
      Ce << C[0], C[1], C[2];
    } else if (!is_plane_stress) {
      Ce(0) = E * (1.0 - mu) / (1.0 + mu) / (1.0 - 2.0 * mu);
      Ce(1) = E * mu / (1.0 + mu) / (1.0 - 2.0 * mu);
      Ce(2) = E / 2.0 / (1.0 + mu);
    } else {
      Ce(0) = E / (1.0 - mu) / (1.0 + mu);
      Ce(1) = E * mu / (1.0 + mu) / (1.0 - mu);
      Ce(2) = E / 2.0 / (1.0 + mu);
    }
    if (cell.dim == 2)
      KnTv = cell.el_mapping * Ce;
    else
      KnTv = cell.radius * cell.el_mapping * Ce;
    for (int i = 0; i < nlayer; ++i)
      for (Bond<nlayer>* bd : bond_layers[i]) {
        if (cell.lattice == LatticeType::Hexagon2D) {
          bd->Kn = KnTv(0);
          bd->Tv = KnTv(1);
        } else {
          bd->Kn = KnTv(bd->layer);
          bd->Tv = KnTv(2);
        }
      }
  }
};

template <int nlayer>
int Particle<nlayer>::_ID = 0;

template <int nlayer>
class ParticleElastic : public Particle<nlayer> {
  double critical_bstrain{0};

 public:
  ParticleElastic(const double& x, const double& y, const double& z, const UnitCell& c) : Particle<nlayer>{x, y, z, c} {
    this->state_var = {0};
    this->state_var_last = {0};
  }
  ParticleElastic(const double& x, const double& y, const double& z, const UnitCell& c, const int& t)
      : Particle<nlayer>{x, y, z, c, t} {
    this->state_var = {0};
    this->state_var_last = {0};
  }
  void setParticleProperty(double nl, bool ps, double E, double mu, double crit) {
    critical_bstrain = crit;
    this->nonlocal_L = nl;
    this->setBondConstants(ps, E, mu);
  }
  void setParticleProperty(double nl, double C11, double C12, double C44, double crit) {
    critical_bstrain = crit;
    this->nonlocal_L = nl;
    const double C[3] = {C11, C12, C44};
    this->setBondConstants(false, 0, 0, C);
  }
  int gpuLaw() const override { return LPM_LAW_ELASTIC; }
  void gpuParams(std::vector<double>& out) const override { out = {critical_bstrain}; }
};

template <int nlayer>
class ParticleElasticDamage : public Particle<nlayer> {
 public:
  double k0{0}, k1{0};
  double damage_threshold{0}, comp_tensile_ratio{0};
  ParticleElasticDamage(const double& x, const double& y, const double& z, const UnitCell& c)
      : Particle<nlayer>{x, y, z, c} {
    this->state_var = std::vector<double>(1, 0.);
    this->state_var_last = std::vector<double>(1, 0.);
  }
  ParticleElasticDamage(const double& x, const double& y, const double& z, const UnitCell& c, const int& t)
      : Particle<nlayer>{x, y, z, c, t} {
    this->state_var = std::vector<double>(1, 0.);
    this->state_var_last = std::vector<double>(1, 0.);
  }
  void setParticleProperty(double nl, bool ps, double E, double mu, double p_k0, double p_k1, double ct, double thr) {
    k0 = p_k0;
    k1 = p_k1;
    damage_threshold = thr;
    comp_tensile_ratio = ct;
    this->nonlocal_L = nl;
    this->setBondConstants(ps, E, mu);
  }
  void setParticleProperty(double nl, double C11, double C12, double C44, double p_k0, double p_k1, double ct,
                           double thr) {
    k0 = p_k0;
    k1 = p_k1;
    damage_threshold = thr;
    comp_tensile_ratio = ct;
    this->nonlocal_L = nl;
    const double C[3] = {C11, C12, C44};
    this->setBondConstants(false, 0, 0, C);
  }
  int gpuLaw() const override { return LPM_LAW_DAMAGE; }
  void gpuParams(std::vector<double>& out) const override { out = {k0, k1, damage_threshold}; }
};

template <int nlayer>
class ParticleJ2Plasticity : public Particle<nlayer> {
 public:
  double E{0}, mu{0}, sigmay{0}, xi{0}, H{0}, A{0};
  double damage_threshold{0}, critical_bstrain{0};  // damage_threshold is never set (stays 0), as in the reference
  ParticleJ2Plasticity(const double& x, const double& y, const double& z, const UnitCell& c)
      : Particle<nlayer>{x, y, z, c} {
    this->state_var = std::vector<double>(7, 0.);
    this->state_var_last = std::vector<double>(7, 0.);
  }
  ParticleJ2Plasticity(const double& x, const double& y, const double& z, const UnitCell& c, const int& t)
      : Particle<nlayer>{x, y, z, c, t} {
    this->state_var = std::vector<double>(7, 0.);
    this->state_var_last = std::vector<double>(7, 0.);
  }
  void setParticleProperty(double nl, bool ps, double p_E, double p_mu, double p_sy, double p_xi, double p_H,
                           double p_A, double crit) {
    E = p_E;
    mu = p_mu;
    sigmay = p_sy;
    xi = p_xi;
    H = p_H;
    A = p_A;
    critical_bstrain = crit;
    this->nonlocal_L = nl;
    this->setBondConstants(ps, p_E, p_mu);
  }
  int gpuLaw() const override { return LPM_LAW_J2; }
  void gpuParams(std::vector<double>& out) const override { out = {E, mu, sigmay, xi, H, A, damage_threshold}; }
};

template <int nlayer>
class ParticleFatigueHCF : public Particle<nlayer> {
 public:
  double A{0}, B{0}, d{0};
  double E{0}, mu{0}, fatigue_limit_ratio{1.108};
  double damage_threshold{1};
  ParticleFatigueHCF(const double& x, const double& y, const double& z, const UnitCell& c)
      : Particle<nlayer>{x, y, z, c} {
    this->state_var = {0, INT_MAX, 0};
    this->state_var_last = {0, INT_MAX, 0};
  }
  ParticleFatigueHCF(const double& x, const double& y, const double& z, const UnitCell& c, const int& t)
      : Particle<nlayer>{x, y, z, c, t} {
    this->state_var = {0, INT_MAX, 0};
    this->state_var_last = {0, INT_MAX, 0};
  }
  void setParticleProperty(double nl, bool ps, double p_E, double p_mu, double p_A, double p_B, double p_d,
                           double thr, double flr) {
    E = p_E;
    mu = p_mu;
    A = p_A;
    B = p_B;
    d = p_d;
    damage_threshold = thr;
    fatigue_limit_ratio = flr;
    this->nonlocal_L = nl;
    this->setBondConstants(ps, p_E, p_mu);
  }
  int gpuLaw() const override { return LPM_LAW_FATIGUE_HCF; }
  void gpuParams(std::vector<double>& out) const override { out = {A, B, d, damage_threshold}; }
};
