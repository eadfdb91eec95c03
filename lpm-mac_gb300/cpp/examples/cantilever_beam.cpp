// Cantilever beam under a transverse end force, and the relative L2 error of
// its displacement against the closed-form beam solution (Solution,
// solution.h): the setup of the reference's convergence example
// (examples/ex7_convergence_beam.cpp: a 30 x 10 hexagonal plate, E = 69 GPa,
// nu = 0.33, plane strain, the right end clamped, a force of 2 N on the left
// end), written against the LPM class interface.  Compiled against these
// headers it runs on the GPU; the same source compiles against the original
// header set.
//
//   cantilever_beam <out.txt> [static|fatigue] [radius]
//
// "static" solves with SolverStatic as the example does; "fatigue" with
// SolverFatigue::solveProblemStatic, which eliminates the displacement
// boundary conditions from the tangent.  The bond constants are set from
// the stiffness table's rows (see hex_plate_tension.cpp).  Writes
// "id x y z x0 y0 z0" per particle (17 significant digits) and prints
// "L2 error is: <value>" with 17 significant digits.
#include <climits>
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
#include "solution.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s out.txt [static|fatigue] [radius]\n", argv[0]);
    return 2;
  }
  const std::string mode = argc > 2 ? argv[2] : "fatigue";
  const double radius = argc > 3 ? atof(argv[3]) : 0.2;
  const int n_layer = 2;
  UnitCell cell(LatticeType::Hexagon2D, radius);
  double angles[] = {0.0, 0.0, 0.0};
  Eigen::MatrixXd R_matrix = createRMatrix(0, angles);
  std::array<double, 2 * NDIM> box{0.0, 30.0, -5.0, 5.0, 0.0, 1.0};
  std::vector<std::array<double, NDIM>> xyz = createPlateHEX2D(box, cell, R_matrix);
  Assembly<n_layer> ass{xyz, box, cell, ParticleType::Elastic};
  printf("Particle number is %d\n", ass.nparticle);

  double left = INT_MAX, right = INT_MIN;
  for (const auto& x : xyz) {
    left = std::min(left, x[0]);
    right = std::max(right, x[0]);
  }
  const double E0 = 69e3, mu0 = 0.33, force = 2.0;
  std::vector<Particle<n_layer>*> left_end, right_end;
  for (Particle<n_layer>* p : ass.pt_sys) {
    if (p->xyz[0] < left + EPS) {
      left_end.push_back(p);
      p->type = 2;
    }
    if (p->xyz[0] > right - EPS) {
      right_end.push_back(p);
      p->type = 1;
    }
    dynamic_cast<ParticleElastic<n_layer>*>(p)->setParticleProperty(EPS, false, E0, mu0, 1.0);
  }
  const double C11 = E0 * (1.0 - mu0) / (1.0 + mu0) / (1.0 - 2.0 * mu0);
  const double C12 = E0 * mu0 / (1.0 + mu0) / (1.0 - 2.0 * mu0);
  const double Kn = sqrt(3.0) / 12.0 * (C11 - C12), Tv = sqrt(3.0) / 48.0 * C12 - sqrt(3.0) / 144.0 * C11;
  for (Particle<n_layer>* p : ass.pt_sys)
    for (int l = 0; l < n_layer; ++l)
      for (Bond<n_layer>* bd : p->bond_layers[l]) {
        bd->Kn = Kn;
        bd->Tv = Tv;
      }
  std::vector<LoadStep<n_layer>> load(1);
  load[0].dispBCs.push_back(DispBC<n_layer>(right_end, LoadMode::Relative, 'x', 0.0));
  load[0].dispBCs.push_back(DispBC<n_layer>(right_end, LoadMode::Relative, 'y', 0.0));
  load[0].forceBCs.push_back(ForceBC<n_layer>(left_end, LoadMode::Relative, 0.0, force, 0.0));
  ass.updateGeometry();
  ass.updateForceState();
  ass.updateStateVar();
  const std::string dump = std::string(argv[1]) + ".dump";
  int start_index = 0;
  if (mode == "fatigue") {
    SolverFatigue<n_layer> solv{4, ass, StiffnessMode::Analytical, SolverMode::CG, TimeMapMode::Linear, 1.0,
                                dump, 30, 1e-5};
    solv.solveProblemStatic(load, start_index);
  } else {
    SolverStatic<n_layer> solv{4, ass, StiffnessMode::Analytical, SolverMode::CG, dump, 30, 1e-5};
    solv.solveProblem(load, start_index);
  }
  Solution<n_layer> sol{ass, ExactSolution::Beam001};
  sol.computeSolBeam001(box[1] - box[0], box[3] - box[2], force, E0, mu0);
  printf("L2 error is: %.17g\n", sol.computeL2Error());
  FILE* f = fopen(argv[1], "w");
  if (!f) return 1;
  for (Particle<n_layer>* p : ass.pt_sys)
    fprintf(f, "%d %.17g %.17g %.17g %.17g %.17g %.17g\n", p->id, p->xyz[0], p->xyz[1], p->xyz[2], p->xyz_initial[0],
            p->xyz_initial[1], p->xyz_initial[2]);
  fclose(f);
  return 0;
}
