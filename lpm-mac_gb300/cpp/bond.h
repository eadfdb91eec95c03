// Bond: host view of one directed bond (bond.h:13-74 of the reference).
// On the GPU path the device holds the bond state; Assembly copies it back
// into these objects after each device update.
#pragma once

#include "lpm.h"

template <int nlayer>
class Particle;

template <int nlayer>
class Bond {
 protected:
  static int _ID;

 public:
  int id{0};
  int layer{-1};
  double dis_initial{0}, dis_last{0}, dis{0};
  double dL{0}, dLe{0}, dLp{0}, dLp_last{0};
  double dLe_dis{0};
  double bstrain{0};
  double Kn{0}, Tv{0};
  double csx{0}, csy{0}, csz{0};
  double bforce_last{0}, bforce{0}, bdamage{0}, bdamage_last{0};
  Particle<nlayer>*p1, *p2;

  Bond(Particle<nlayer>* a, Particle<nlayer>* b, int p_layer, double p_dis) : p1(a), p2(b) {
    id = _ID++;
    dis = dis_initial = dis_last = p_dis;
    layer = p_layer;
    csx = (p1->xyz[0] - p2->xyz[0]) / dis;
    csy = (p1->xyz[1] - p2->xyz[1]) / dis;
    csz = (p1->xyz[2] - p2->xyz[2]) / dis;
  }
};

template <int nlayer>
int Bond<nlayer>::_ID = 0;
