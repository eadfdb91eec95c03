// DispBC / ForceBC (boundary.h:10-44 of the reference).
#pragma once

#include "particle.h"

template <int nlayer>
class DispBC {
 public:
  std::vector<Particle<nlayer>*> group;
  LoadMode load_mode;
  char flag;
  double step;
  DispBC(std::vector<Particle<nlayer>*> g, LoadMode m, char f, double s) : group{g}, load_mode{m}, flag{f}, step{s} {}
  void cutHalf() { step /= 2.0; }
};

template <int nlayer>
class ForceBC {
 public:
  std::vector<Particle<nlayer>*> group;
  LoadMode load_mode;
  double fx, fy, fz;
  ForceBC(std::vector<Particle<nlayer>*> g, LoadMode m, double x, double y, double z)
      : group{g}, load_mode{m}, fx{x}, fy{y}, fz{z} {}
  void cutHalf() { fx /= 2.0, fy /= 2.0, fz /= 2.0; }
};
