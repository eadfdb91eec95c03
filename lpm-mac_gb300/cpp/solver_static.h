// SolverStatic (solver_static.h:19-149 of the reference).
#pragma once

#include "solver.h"

template <int nlayer>
class SolverStatic : public Solver<nlayer> {
 public:
  int undamaged_pt_type{0};

  SolverStatic(const int& p_undamaged, Assembly<nlayer>& p_ass, const StiffnessMode& p_stiff_mode,
               const SolverMode& p_sol_mode, const std::string& p_dumpFile, const int& p_niter, const double& p_tol)
      : Solver<nlayer>{p_ass, p_stiff_mode, p_sol_mode, p_dumpFile, p_niter, p_tol}, undamaged_pt_type{p_undamaged} {
    this->ass.setUndamagedType(undamaged_pt_type);
  }

  // solver_static.h:31-62 on the device
  bool updateStaticDamage() {
    int any = 0;
    lpm_check(lpm_update_damage(this->ass.device(), &any), "lpm_update_damage");
    this->ass.pullParticles();
    return any != 0;
  }

  void solveProblem(std::vector<LoadStep<nlayer>>& load, int& start_index) {
    int n_step = (int)load.size();
    double dt = 1;
    for (int i = 0; i < n_step; i++) {
    restart:
      printf("Loading step-%d, iteration starts:\n", i + start_index);
      double t1 = omp_get_wtime();
      bool is_converged = solveProblemStep(load[(size_t)i], dt);
      if (!is_converged) {
        this->ass.resetStateVar(true);
        load[(size_t)i].loadCutHalf();
        load.insert(load.begin() + i, load[(size_t)i]);
        ++n_step;
        printf("Step-%d not converging\n\n", i + start_index);
        goto restart;
      }
      this->ass.writeDump(this->dumpFile, i + start_index);
      double t2 = omp_get_wtime();
      printf("Loading step %d has finished, spent %f seconds\n\nData output ...\n\n", i + start_index, t2 - t1);
    }
    start_index += n_step;
  }

  bool solveProblemStep(LoadStep<nlayer>& load_step, double&) {
    this->updateForceBC(load_step);
    this->updateDisplacementBC(load_step);
    int n_newton{0};
    bool new_damaged{false};
    do {
      double t11 = omp_get_wtime();
      this->stiffness.calcStiffness(this->ass.pt_sys);
      this->stiffness.flush();
      double t12 = omp_get_wtime();
      printf("Stiffness matrix calculation costs %f seconds\n", t12 - t11);
      n_newton = this->NewtonIteration();
      if (n_newton >= this->max_NR_iter) break;
      this->ass.updateStateVar();
      new_damaged = updateStaticDamage();
      this->ass.storeStateVar();
      if (new_damaged) {
        printf("Updating damage\n");
        this->ass.updateGeometry();
        this->ass.updateForceState();
      }
    } while (new_damaged);
    return n_newton < this->max_NR_iter;
  }
};
