// SolverFatigue (solver_fatigue.h:19-299 of the reference): cyclic loading
// with the fatigue damage update on the device.
#pragma once

#include "load_step_fatigue.h"
#include "solver.h"

// cycle jump per simulated time unit (solver_fatigue.h:62-70)
inline int func_dNdt_linear(const double& tau) { return (int)(1 / tau); }
inline int func_dNdt_exponental(const double& tau, const double& t) { return (int)(1 / tau * exp(t / tau)); }

template <int nlayer>
class SolverFatigue : public Solver<nlayer> {
 public:
  int undamaged_pt_type{0};
  TimeMapMode t_mode;
  double tau{0};
  std::vector<double> load_spectrum;

  SolverFatigue(const int& p_undamaged, Assembly<nlayer>& p_ass, const StiffnessMode& p_stiff_mode,
                const SolverMode& p_sol_mode, const TimeMapMode& p_t_mode, const double& p_tau,
                const std::string& p_dumpFile, const int& p_niter, const double& p_tol)
      : Solver<nlayer>{p_ass, p_stiff_mode, p_sol_mode, p_dumpFile, p_niter, p_tol},
        undamaged_pt_type{p_undamaged},
        t_mode(p_t_mode),
        tau(p_tau) {
    this->ass.setUndamagedType(undamaged_pt_type);
  }

  // one number per entry: f_min, then f_max, f_min, ... (solver_fatigue.h:41-60)
  void readLoad(const std::string& loadFile) {
    FILE* f = fopen(loadFile.c_str(), "r");
    if (!f) {
      printf("'%s' does not exist!\n", loadFile.c_str());
      exit(1);
    }
    double v;
    while (fscanf(f, "%lf", &v) > 0) load_spectrum.push_back(v);
    fclose(f);
  }

  // nonlocal damage rate and the damage increment, on the device
  // (solver_fatigue.h:72-120)
  bool updateFatigueDamage(double dNdt) {
    int any = 0;
    lpm_check(lpm_fatigue_damage(this->ass.device(), dNdt, &any), "lpm_fatigue_damage");
    this->ass.pullParticles();
    return any != 0;
  }

  // the 2*n_interval load steps of cycle N (solver_fatigue.h:122-172)
  std::vector<LoadStep<nlayer>> generateLoadCycle(FatigueLoadType ltype, int N, int n_interval,
                                                  std::vector<std::vector<Particle<nlayer>*>> g) {
    const double f0 = load_spectrum[(size_t)(2 * N)], f1 = load_spectrum[(size_t)(2 * N + 1)],
                 f2 = load_spectrum[(size_t)(2 * N + 2)];
    std::vector<LoadStep<nlayer>> out;
    for (double d : {(f1 - f0) / n_interval, (f2 - f1) / n_interval})
      for (int i = 0; i < n_interval; ++i) {
        if (ltype == FatigueLoadType::LoadUniaxialDisp) out.push_back(LoadUniaxialDisp<nlayer>(d, g[0], g[1], g[2]));
        if (ltype == FatigueLoadType::LoadUniaxialForce) out.push_back(LoadUniaxialForce<nlayer>(d, g[0], g[1], g[2]));
        if (ltype == FatigueLoadType::LoadDogBoneDisp) out.push_back(LoadDogBoneDisp<nlayer>(0, d, 0, g[0], g[1]));
        if (ltype == FatigueLoadType::LoadCTForce) out.push_back(LoadCTForce<nlayer>(d, g[0], g[1], g[2]));
      }
    return out;
  }

  // solver_fatigue.h:174-210
  void solveProblemCyclic(FatigueLoadType loadType, int n_interval, std::vector<std::vector<Particle<nlayer>*>> g) {
    const double n_cycles = 0.5 * ((double)load_spectrum.size() - 1);
    double t{0}, dNdt{1};
    int N{0};
    do {
      printf("Cycle-%d starts:\n\n", N + 1);
      std::vector<LoadStep<nlayer>> load_cycle = generateLoadCycle(loadType, N, n_interval, g);
      dNdt = (t_mode == TimeMapMode::Linear) ? func_dNdt_linear(tau) : func_dNdt_exponental(tau, t++);
      solveProblemOneCycle(load_cycle, dNdt);
      double ave_u{0};
      int n_pt = 0;
      for (Particle<nlayer>* pt : this->ass.pt_sys)
        if (pt->type != undamaged_pt_type) {
          n_pt++;
          ave_u += pt->state_var.empty() ? 0.0 : pt->state_var[0];
        }
      std::cout << "Average strain energy is: " << ave_u / n_pt << std::endl;
      N += (int)dNdt;
      this->ass.writeDump(this->dumpFile, N);
    } while (N < n_cycles);
  }

  // solver_fatigue.h:212-233
  void solveProblemOneCycle(std::vector<LoadStep<nlayer>>& load, double dNdt) {
    const int n_step = (int)load.size();
    for (int i = 0; i < n_step; ++i) {
      printf("Substep-%d, iteration starts:\n", i);
      double t1 = omp_get_wtime();
      solveProblemStep(load[(size_t)i]);
      this->ass.updateStateVar();
      double t2 = omp_get_wtime();
      printf("Loading step %d has finished, spent %f seconds\n\n", i, t2 - t1);
    }
    updateFatigueDamage(dNdt);
    this->ass.storeStateVar();
    this->ass.updateGeometry();
    this->ass.updateForceState();
  }

  // solver_fatigue.h:235-270
  void solveProblemStatic(std::vector<LoadStep<nlayer>>& load, int& start_index) {
    int n_step = (int)load.size();
    for (int i = 0; i < n_step; i++) {
    restart:
      printf("Loading step-%d, iteration starts:\n", i + start_index);
      double t1 = omp_get_wtime();
      if (!solveProblemStep(load[(size_t)i])) {
        this->ass.resetStateVar(true);
        load[(size_t)i].loadCutHalf();
        load.insert(load.begin() + i, load[(size_t)i]);
        ++n_step;
        printf("Step-%d not converging\n\n", i + start_index);
        goto restart;
      }
      this->ass.updateStateVar();
      this->ass.storeStateVar();
      double t2 = omp_get_wtime();
      printf("Loading step %d has finished, spent %f seconds\n\nData output ...\n\n", i + start_index, t2 - t1);
      this->ass.writeDump(this->dumpFile, i);
    }
    start_index += n_step;
  }

  // solver_fatigue.h:272-296: tangent with the displacement BCs eliminated
  bool solveProblemStep(LoadStep<nlayer>& load_step) {
    this->updateForceBC(load_step);
    this->updateDisplacementBC(load_step);
    this->stiffness.reset(this->ass.pt_sys);
    double t11 = omp_get_wtime();
    this->stiffness.calcStiffness(this->ass.pt_sys);
    this->stiffness.updateStiffnessDispBC(this->ass.pt_sys);
    this->stiffness.flush();
    double t12 = omp_get_wtime();
    printf("Stiffness matrix calculation costs %f seconds\n", t12 - t11);
    return this->NewtonIteration() < this->max_NR_iter;
  }
};
