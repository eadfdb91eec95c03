// Solver (solver.h:16-218 of the reference): Newton iteration, boundary
// conditions and the linear solve, each step on the device.  The printed
// lines are the reference's.
#pragma once

#include "load_step.h"
#include "stiffness.h"

template <int nlayer>
class Solver {
 public:
  int problem_size, max_NR_iter;
  double tol_NR_iter;
  std::string dumpFile;
  SolverMode sol_mode;
  Eigen::VectorXd disp;
  Eigen::VectorXd reaction_force;
  Stiffness<nlayer> stiffness;
  Assembly<nlayer> ass;

  Solver(Assembly<nlayer>& p_ass, const StiffnessMode& p_stiff_mode, const SolverMode& p_sol_mode,
         const std::string& p_dumpFile, const int& p_niter, const double& p_tol)
      : problem_size((p_ass.pt_sys[0]->cell.dim) * (int)p_ass.pt_sys.size()),
        max_NR_iter(p_niter),
        tol_NR_iter(p_tol),
        dumpFile(p_dumpFile),
        sol_mode{p_sol_mode},
        disp((Eigen::Index)problem_size),
        reaction_force((Eigen::Index)0),
        stiffness(p_ass.pt_sys, p_stiff_mode),
        ass(p_ass) {
    stiffness.attach(&ass);
  }

  // solver.h:130-166 (an Absolute BC moves the particle to (step,0,0)-style
  // positions, as the reference's moveTo(dxyz) does)
  void updateDisplacementBC(LoadStep<nlayer>& load_step) {
    for (DispBC<nlayer>& bc : load_step.dispBCs) {
      const int axis = bc.flag == 'x' ? 0 : (bc.flag == 'y' ? 1 : 2);
      const int mode = bc.load_mode == LoadMode::Relative ? 0 : 1;
      lpm_check(lpm_apply_disp_bc(ass.device(), ass.groupId(bc.group), axis, mode, bc.step), "lpm_apply_disp_bc");
      for (Particle<nlayer>* pt : bc.group) {
        std::array<double, NDIM> d{0, 0, 0};
        d[(size_t)axis] = bc.step;
        if (mode == 0)
          pt->moveBy(d);
        else
          pt->moveTo(d);
        pt->disp_constraint[(size_t)axis] = 1;
      }
    }
  }
  // solver.h:168-190
  void updateForceBC(LoadStep<nlayer>& load_step) {
    for (ForceBC<nlayer>& bc : load_step.forceBCs) {
      const int mode = bc.load_mode == LoadMode::Relative ? 0 : 1;
      lpm_check(lpm_apply_force_bc(ass.device(), ass.groupId(bc.group), mode, bc.fx, bc.fy, bc.fz),
                "lpm_apply_force_bc");
      const int n = (int)bc.group.size();
      for (Particle<nlayer>* pt : bc.group) {
        if (mode == 0) {
          pt->Pex[0] += bc.fx / n;
          pt->Pex[1] += bc.fy / n;
          pt->Pex[2] += bc.fz / n;
        } else {
          pt->Pex[0] = bc.fx / n;
          pt->Pex[1] = bc.fy / n;
          pt->Pex[2] = bc.fz / n;
        }
      }
    }
  }
  // solver.h:108-128: residual on the device; the reaction list from the
  // internal forces at constrained DOFs (read from the device, since the
  // Newton loop does not copy the particles back between iterations)
  void updateRR() {
    lpm_check(lpm_residual(ass.device(), &norm_r_, &norm_R_), "lpm_residual");
    lpm_check(lpm_download(ass.device(), LPM_F_RESIDUAL, stiffness.residual.data()), "lpm_download");
    pin_.resize(3 * ass.pt_sys.size());
    lpm_check(lpm_download(ass.device(), LPM_F_PIN, pin_.data()), "lpm_download");
    std::vector<double> temp;
    for (size_t i = 0; i < ass.pt_sys.size(); ++i) {
      Particle<nlayer>* pt = ass.pt_sys[i];
      for (int k = 0; k < pt->cell.dim; k++)
        if (pt->disp_constraint[(size_t)k] == 1) temp.push_back(pin_[3 * i + (size_t)k]);
    }
    reaction_force.resize((Eigen::Index)temp.size());
    for (size_t i = 0; i < temp.size(); ++i) reaction_force((Eigen::Index)i) = temp[i];
  }
  // solver.h:192-217
  void LPM_CG() {
    int64_t it = 0;
    double err = 0;
    const LpmGpuOptions& o = lpm_gpu_options();
    stiffness.flush();
    int st = lpm_solve(ass.device(), o.precision, o.cg_tol, -1, &it, &err);
    lpm_check(st, "lpm_solve");
    lpm_check(lpm_download(ass.device(), LPM_F_DISP, disp.data()), "lpm_download");
    if (st != LPM_OK) {
      std::cout << "Solving failed." << std::endl;
      return;
    }
    if (o.verbose) {
      std::cout << "The system has been solved after " << it << " iterations." << std::endl;
      std::cout << "The estimated error is " << err << std::endl;
    }
  }
  // solver.h:91-106
  void solveLinearSystem() {
    if (sol_mode == SolverMode::CG) LPM_CG();
    lpm_check(lpm_move_by_disp(ass.device()), "lpm_move_by_disp");
  }
  // solver.h:53-89.  The force state stays on the device through the loop;
  // the particles are brought up to date once, when it returns.
  int NewtonIteration() {
    const int ni = newtonLoop();
    ass.pullParticles();
    return ni;
  }

 protected:
  double norm_r_ = 0, norm_R_ = 0;
  std::vector<double> pin_;

  int newtonLoop() {
    ass.refreshForceState();  // updateGeometry and updateForceState are one device pass
    updateRR();
    double norm_residual = norm_r_, norm_reaction_force = norm_R_;
    double tol_multiplier = std::max(norm_residual, norm_reaction_force);
    const bool v = lpm_gpu_options().verbose;
    if (v)
      printf("|  Norm of residual is %.5e, norm of reaction is %.5e, tolerance criterion is based on %s force\n",
             norm_residual, norm_reaction_force, norm_residual > norm_reaction_force ? "residual" : "reaction");
    int ni{0};
    while (norm_residual > tol_NR_iter * tol_multiplier) {
      if (++ni > max_NR_iter) return max_NR_iter;
      if (v) printf("|  |  Iteration-%d: ", ni);
      solveLinearSystem();
      ass.refreshForceState();
      updateRR();
      norm_residual = norm_r_;
      if (v)
        printf("|  |  Norm of residual is %.3e, residual ratio is %.3e\n", norm_residual,
               norm_residual / tol_multiplier);
    }
    return ni;
  }
};
