// Stiffness (stiffness.h:18-295 of the reference): the tangent lives on the
// device.  calcStiffness and updateStiffnessDispBC record what is asked for
// (the tangent, then the tangent with the constrained rows and columns
// eliminated) and flush() assembles it in one device pass; the solve and
// exportK flush first, so the pair costs one assembly, not two.  The
// assembled matrix is read back with exportK (block CSR, K not transposed).
#pragma once

#include "assembly.h"

template <int nlayer>
class Stiffness {
  StiffnessMode mode;
  Assembly<nlayer>* ass_ = nullptr;
  bool pending_ = false;
  int bc_ = LPM_BC_NONE;

 public:
  Eigen::VectorXd residual;

  Stiffness(std::vector<Particle<nlayer>*>& pt_sys, StiffnessMode p_mode)
      : mode(p_mode), residual((Eigen::Index)(pt_sys.size() * pt_sys[0]->cell.dim)) {
    // The forward-difference tangent (localStiffnessFD, stiffness.h:103-154)
    // is not built on the device.  Asking for it ends the program with an
    // argument error rather than silently assembling a different matrix.
    if (mode == StiffnessMode::FiniteDifference) {
      fprintf(stderr, "liblpmgpu: StiffnessMode::FiniteDifference is not supported on the GPU path "
                      "(use StiffnessMode::Analytical)\n");
      exit(1);
    }
  }
  void attach(Assembly<nlayer>* a) { ass_ = a; }
  void reset(std::vector<Particle<nlayer>*>&) {}
  void calcStiffness(std::vector<Particle<nlayer>*>&) {
    pending_ = true;
    bc_ = lpm_gpu_options().static_bc;
  }
  void updateStiffnessDispBC(std::vector<Particle<nlayer>*>&) {
    pending_ = true;
    bc_ = LPM_BC_ELIMINATE;
  }
  void flush() {
    if (!pending_) return;
    pending_ = false;
    lpm_check(lpm_assemble(ass_->device(), lpm_gpu_options().tangent, bc_), "lpm_assemble");
  }
  // block CSR of the assembled K: cptr (N+1), cidx, dim*dim values per block
  void exportK(std::vector<int64_t>& cptr, std::vector<int>& cidx, std::vector<double>& vals) {
    flush();
    lpm_handle* h = ass_->device();
    int64_t nblk = 0;
    lpm_num_blocks(h, &nblk);
    const int dim = ass_->pt_sys[0]->cell.dim;
    cptr.resize(ass_->pt_sys.size() + 1);
    cidx.resize((size_t)nblk);
    vals.resize((size_t)nblk * dim * dim);
    lpm_check(lpm_get_pattern(h, cptr.data(), cidx.data()), "lpm_get_pattern");
    lpm_check(lpm_get_K(h, vals.data()), "lpm_get_K");
  }
};
