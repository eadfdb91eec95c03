// Fatigue load-step templates (load_step_fatigue.h:13-85 of the reference).
#pragma once

#include "load_step.h"

enum class FatigueLoadType : char { LoadUniaxialDisp, LoadUniaxialForce, LoadDogBoneDisp, LoadCTForce };

template <int nlayer>
class LoadUniaxialForce : public LoadStep<nlayer> {
 public:
  LoadUniaxialForce(double fy, std::vector<Particle<nlayer>*>& left, std::vector<Particle<nlayer>*>& top,
                    std::vector<Particle<nlayer>*>& bottom) {
    this->dispBCs.push_back(DispBC<nlayer>(left, LoadMode::Relative, 'x', 0.0));
    this->forceBCs.push_back(ForceBC<nlayer>(top, LoadMode::Relative, 0.0, fy, 0.0));
    this->dispBCs.push_back(DispBC<nlayer>(bottom, LoadMode::Relative, 'y', 0.0));
  }
};

template <int nlayer>
class LoadUniaxialDisp : public LoadStep<nlayer> {
 public:
  LoadUniaxialDisp(double dy, std::vector<Particle<nlayer>*>& left, std::vector<Particle<nlayer>*>& top,
                   std::vector<Particle<nlayer>*>& bottom) {
    this->dispBCs.push_back(DispBC<nlayer>(left, LoadMode::Relative, 'x', 0.0));
    this->dispBCs.push_back(DispBC<nlayer>(top, LoadMode::Relative, 'y', dy));
    this->dispBCs.push_back(DispBC<nlayer>(bottom, LoadMode::Relative, 'y', 0.0));
  }
};

template <int nlayer>
class LoadDogBoneDisp : public LoadStep<nlayer> {
 public:
  LoadDogBoneDisp(double x, double y, double z, std::vector<Particle<nlayer>*>& g1, std::vector<Particle<nlayer>*>& g2) {
    this->dispBCs.push_back(DispBC<nlayer>(g1, LoadMode::Relative, 'x', x));
    this->dispBCs.push_back(DispBC<nlayer>(g1, LoadMode::Relative, 'y', y));
    this->dispBCs.push_back(DispBC<nlayer>(g1, LoadMode::Relative, 'z', z));
    this->dispBCs.push_back(DispBC<nlayer>(g2, LoadMode::Relative, 'x', 0.0));
    this->dispBCs.push_back(DispBC<nlayer>(g2, LoadMode::Relative, 'y', 0.0));
    this->dispBCs.push_back(DispBC<nlayer>(g2, LoadMode::Relative, 'z', 0.0));
  }
};

template <int nlayer>
class LoadCTForce : public LoadStep<nlayer> {
 public:
  LoadCTForce(double fy, std::vector<Particle<nlayer>*>& mid, std::vector<Particle<nlayer>*>& top,
              std::vector<Particle<nlayer>*>& bottom) {
    this->dispBCs.push_back(DispBC<nlayer>(mid, LoadMode::Relative, 'y', 0));
    this->dispBCs.push_back(DispBC<nlayer>(top, LoadMode::Relative, 'x', 0.0));
    this->dispBCs.push_back(DispBC<nlayer>(bottom, LoadMode::Relative, 'x', 0.0));
    this->forceBCs.push_back(ForceBC<nlayer>(top, LoadMode::Relative, 0.0, fy, 0.0));
    this->forceBCs.push_back(ForceBC<nlayer>(bottom, LoadMode::Relative, 0.0, -fy, 0.0));
  }
};
