// LoadStep (load_step.h:12-29 of the reference).
#pragma once

#include "boundary.h"

template <int nlayer>
class LoadStep {
 public:
  std::vector<DispBC<nlayer>> dispBCs;
  std::vector<ForceBC<nlayer>> forceBCs;
  LoadStep() {}
  void loadCutHalf() {
    for (DispBC<nlayer>& d : dispBCs) d.cutHalf();
    for (ForceBC<nlayer>& f : forceBCs) f.cutHalf();
  }
};
