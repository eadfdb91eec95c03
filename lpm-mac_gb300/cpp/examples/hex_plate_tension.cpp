// Hexagonal plate stretched by displacing its top edge with the bottom edge
// clamped: a program written against the LPM class interface (Assembly, ParticleElastic,
// LoadStep, SolverStatic / SolverFatigue).  Compiled against these headers it
// runs on the GPU; the same source compiles against the original header set.
//
//   hex_plate_tension <out.txt> [static|fatigue] [n_steps]
//
// writes "id x y z x0 y0 z0" per particle (17 significant digits) after the
// last step, x0 being the initial position.
#include <cstdio>
#include <cstdlib>
#include <string>

// the include order of the original examples (its headers need it)
#include "lpm.h"
#include "particle.h"
#include "assembly.h"
#include "utilities.h"
#include "stiffness.h"
#include "load_step.h"
#include "solver_static.h"
#include "solver_fatigue.h"

template <typename SolverT>
static void run_steps(SolverT& solv, std::vector<LoadStep<2>>& load) {
  int start_index = 0;
  solv.solveProblem(load, start_index);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s out.txt [static|fatigue] [n_steps]\n", argv[0]);
    return 2;
  }
  const std::string mode = argc > 2 ? argv[2] : "static";
  const int n_steps = argc > 3 ? atoi(argv[3]) : 2;
  const int n_layer = 2;
  const double radius = 0.2;
  UnitCell cell(LatticeType::Hexagon2D, radius);
  double angles[] = {0.0, 0.0, 0.0};
  Eigen::MatrixXd R_matrix = createRMatrix(0, angles);
  std::array<double, 2 * NDIM> box{0.0, 6.0, -0.4, 12.0, -0.4, 6.0};
  std::vector<std::array<double, NDIM>> xyz = createPlateHEX2D(box, cell, R_matrix);
  Assembly<n_layer> ass{xyz, box, cell, ParticleType::Elastic};
  printf("Particle number is %d\n", ass.nparticle);

  const double E0 = 69e3, mu0 = 0.3, du = 0.002;
  std::vector<Particle<n_layer>*> top, bottom;
  for (Particle<n_layer>* p : ass.pt_sys) {
    if (p->xyz[1] > box[3] - 2 * radius) {
      top.push_back(p);
      p->type = 1;
    }
    if (p->xyz[1] < box[2] + 2 * radius) {
      bottom.push_back(p);
      p->type = 2;
    }
    dynamic_cast<ParticleElastic<n_layer>*>(p)->setParticleProperty(0.0, false, E0, mu0, 1.0);
  }
  // setParticleProperty maps (C11, C12, C44) with the hexagonal table read
  // column by column, which gives a negative normal stiffness; set the bond
  // constants from the table's rows instead (plane strain):
  //   Kn = sqrt(3)/12 (C11 - C12),  Tv = sqrt(3)/48 C12 - sqrt(3)/144 C11
  const double C11 = E0 * (1.0 - mu0) / (1.0 + mu0) / (1.0 - 2.0 * mu0);
  const double C12 = E0 * mu0 / (1.0 + mu0) / (1.0 - 2.0 * mu0);
  const double Kn = sqrt(3.0) / 12.0 * (C11 - C12), Tv = sqrt(3.0) / 48.0 * C12 - sqrt(3.0) / 144.0 * C11;
  for (Particle<n_layer>* p : ass.pt_sys)
    for (int l = 0; l < n_layer; ++l)
      for (Bond<n_layer>* bd : p->bond_layers[l]) {
        bd->Kn = Kn;
        bd->Tv = Tv;
      }
  std::vector<LoadStep<n_layer>> load;
  for (int i = 0; i < n_steps; ++i) {
    LoadStep<n_layer> step;
    step.dispBCs.push_back(DispBC<n_layer>(bottom, LoadMode::Relative, 'x', 0.0));
    step.dispBCs.push_back(DispBC<n_layer>(bottom, LoadMode::Relative, 'y', 0.0));
    step.dispBCs.push_back(DispBC<n_layer>(top, LoadMode::Relative, 'x', 0.0));
    step.dispBCs.push_back(DispBC<n_layer>(top, LoadMode::Relative, 'y', du));
    load.push_back(step);
  }
  ass.updateGeometry();
  ass.updateForceState();
  const std::string dump = std::string(argv[1]) + ".dump";
  if (mode == "fatigue") {
    SolverFatigue<n_layer> solv{-1, ass, StiffnessMode::Analytical, SolverMode::CG, TimeMapMode::Linear, 1.0,
                                dump, 30, 1e-5};
    int start_index = 0;
    solv.solveProblemStatic(load, start_index);
  } else {
    SolverStatic<n_layer> solv{-1, ass, StiffnessMode::Analytical, SolverMode::CG, dump, 30, 1e-5};
    run_steps(solv, load);
  }
  FILE* f = fopen(argv[1], "w");
  if (!f) return 1;
  for (Particle<n_layer>* p : ass.pt_sys)
    fprintf(f, "%d %.17g %.17g %.17g %.17g %.17g %.17g\n", p->id, p->xyz[0], p->xyz[1], p->xyz[2], p->xyz_initial[0],
            p->xyz_initial[1], p->xyz_initial[2]);
  fclose(f);
  return 0;
}
