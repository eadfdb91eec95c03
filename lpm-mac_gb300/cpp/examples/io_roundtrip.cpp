// Dump and bond files through the LPM class interface.
//
//   io_roundtrip write <dir>   a hexagonal plate (createPlateHEX2D, bonds by
//                              createBonds) written as its configuration dump
//                              and bond file (Assembly::writeConfigurationDump,
//                              writeBond)
//   io_roundtrip read <dir>    an Assembly rebuilt from those two files
//                              (readDump, readBond), written again as a bond
//                              file, a configuration dump, and three LAMMPS
//                              dumps appended to one file (writeDump)
//
// Compiled against the original header set or against these headers; the
// files must come out the same byte for byte.  Read mode makes no device call.
#include <cmath>
#include <cstdio>
#include <string>

#include "lpm.h"
#include "particle.h"
#include "assembly.h"
#include "utilities.h"

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s write|read <dir>\n", argv[0]);
    return 2;
  }
  const std::string mode = argv[1], dir = argv[2];
  UnitCell cell(LatticeType::Hexagon2D, 0.25);
  if (mode == "write") {
    double angles[] = {0.0, 0.0, 0.0};
    Eigen::MatrixXd R = createRMatrix(0, angles);
    std::array<double, 2 * NDIM> box{0.0, 4.0, 0.0, 3.5, 0.0, 1.0};
    std::vector<std::array<double, NDIM>> xyz = createPlateHEX2D(box, cell, R);
    Assembly<2> ass{xyz, box, cell, ParticleType::Elastic};
    ass.writeConfigurationDump(dir + "/config.dump");
    ass.writeBond(dir + "/plate.bond");
    return 0;
  }
  Assembly<2> ass{dir + "/config.dump", dir + "/plate.bond", cell, ParticleType::Elastic};
  printf("Particle number is %d\n", ass.nparticle);
  ass.writeBond(dir + "/rt.bond");
  ass.writeConfigurationDump(dir + "/rt_config.dump");
  // deterministic particle fields so that every dump column carries data
  // (the force state is not computed in this mode)
  for (int s = 0; s < 3; ++s) {
    for (Particle<2>* pt : ass.pt_sys) {
      const double a = 0.1 * pt->id + s;
      for (int k = 0; k < 2; ++k) pt->xyz[(size_t)k] = pt->xyz_initial[(size_t)k] + 1e-3 * (k + 1) * sin(a);
      pt->stress.assign(6, 0.0);
      for (int k = 0; k < 6; ++k) pt->stress[(size_t)k] = 10.0 * (k + 1) * cos(a + k);
      pt->damage = (pt->id % 7) / 7.0;
      pt->damage_visual = (pt->id % 5) / 5.0;
      pt->state_var[0] = 0.25 * pt->id + s;
    }
    ass.writeDump(dir + "/rt.dump", s);
  }
  return 0;
}
