/* liblpmgpu: C ABI of the GB300 (sm_103a) LPM quasi-static Newton load step.
 *
 * The LPM-MAC reference has no FFI: its interface is the header-only class
 * set (Assembly, Particle*, Stiffness, Solver, SolverStatic, SolverFatigue,
 * LoadStep/DispBC/ForceBC).  Each entry point below replaces the body of one
 * of those methods; the class it stands in for is cited next to it
 * (paths relative to the LPM-MAC project root).  The C++ mirror of the class
 * API (lpm-mac_gb300/cpp/) and the Python mirror call these functions.
 *
 * Conventions: plain pointers and sizes; host buffers unless stated; an
 * opaque handle per lattice; every call returns an int status
 * (0 ok, >0 not converged, <0 error, see LPM_* below) and never throws or
 * exits.  All device work runs on the handle's own CUDA stream on the
 * current device; calls are synchronous with respect to the host unless
 * stated.  Indices are 0-based particle ids; a particle's DOF k lives at
 * dim*id + k (solver.h:102,117).
 */
#ifndef LPM_GPU_H
#define LPM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lpm_handle lpm_handle;

/* status codes */
#define LPM_OK 0
#define LPM_NOT_CONVERGED 1    /* Newton or CG hit its iteration cap       */
#define LPM_ERR_ARG (-1)       /* bad argument, size or id                  */
#define LPM_ERR_TOPOLOGY (-2)  /* a bond has no opposite bond               */
#define LPM_ERR_CUDA (-3)      /* CUDA runtime error (see lpm_last_error)   */
#define LPM_ERR_NOMEM (-4)     /* device allocation failed                  */
#define LPM_ERR_STATE (-5)     /* call out of order (e.g. solve before K)   */
#define LPM_ERR_NONFINITE (-6) /* NaN/Inf met in a solve                    */

/* particle fields for lpm_upload / lpm_download (double unless noted) */
#define LPM_F_XYZ 0        /* N*3 current positions (Particle::xyz)          */
#define LPM_F_XYZ0 1       /* N*3 initial positions (xyz_initial)            */
#define LPM_F_PIN 2        /* N*3 internal force (Pin)                        */
#define LPM_F_PEX 3        /* N*3 external force (Pex)                        */
#define LPM_F_STRESS 4     /* N*6 xx yy zz yz xz xy (stress)                  */
#define LPM_F_DVIS 5       /* N   damage_visual                               */
#define LPM_F_DLE_TOT 6    /* N*2 per-layer sum of dLe (dLe_total)            */
#define LPM_F_TDLE_TOT 7   /* N*2 per-layer sum of Tv*dLe (TdLe_total)        */
#define LPM_F_CS_SUM 8     /* N*2*3 per-layer direction-cosine sums           */
#define LPM_F_DAMAGE 9     /* N   particle damage                             */
#define LPM_F_XYZ_LAST 10  /* N*3 last converged positions (xyz_last)         */
#define LPM_F_DISP 11      /* N*dim last Newton increment (Solver::disp)     */
#define LPM_F_RESIDUAL 12  /* N*dim residual (Stiffness::residual)           */
#define LPM_F_STATE 13     /* N*nstate state variables (state_var)           */
#define LPM_F_DDOT_LOCAL 14    /* N local damage rate (Ddot_local)           */
#define LPM_F_DDOT_NONLOCAL 15 /* N nonlocal damage rate (Ddot_nonlocal)     */
#define LPM_F_DAMAGE_LAST 16   /* N last converged damage (damage_last)      */
/* bond fields, stored order (by p1, layer, input order) */
#define LPM_B_BFORCE 100
#define LPM_B_BDAMAGE 101
#define LPM_B_DLE 102
#define LPM_B_DIS 103
#define LPM_B_BSTRAIN 104
#define LPM_B_CS 105 /* Nb*3 */
#define LPM_B_KN 106
#define LPM_B_TV 107
#define LPM_B_DIS0 108
#define LPM_B_DLP 109
#define LPM_B_SCRIT 110 /* critical stretch of the softening law (LPM_LAW_SOFTENING) */
#define LPM_B_KAPPA 111 /* largest stretch reached, softening law history             */

/* tangent variants for lpm_assemble */
#define LPM_TANGENT_AS_WRITTEN 0 /* derivative.h as written: K_ii[1][0] stays 0 (derivative.h:38) */
#define LPM_TANGENT_SYMMETRIC 1  /* K_ii[1][0] = K_ii[0][1]                                    */
/* boundary treatment of the tangent */
#define LPM_BC_NONE 0      /* SolverStatic: K unchanged (solver_static.h:113 leaves it out)  */
#define LPM_BC_ELIMINATE 1 /* Stiffness::updateStiffnessDispBC (stiffness.h:265-294)          */
/* linear-solver precision */
#define LPM_PREC_FP64 0  /* Jacobi CG in FP64, the Eigen algorithm (solver.h:192-217)       */
#define LPM_PREC_MIXED 1 /* FP32 Jacobi CG inside FP64 iterative refinement                 */
/* how the solves apply the tangent (lpm_set_operator) */
#define LPM_OPERATOR_ASSEMBLED 0   /* assembled block operator, as calcStiffness builds K (default)   */
#define LPM_OPERATOR_MATRIX_FREE 1 /* the same operator applied from bond data, never assembled       */

/* Creates the device lattice.  Replaces Assembly's constructors
 * (assembly.h:83-106), Assembly::createBonds / readBond (bond lists are given
 * here, assembly.h:212-234, 390-424), Assembly::updateConnections
 * (assembly.h:236-266, computed on the device) and the Kn/Tv assignment of
 * setParticleProperty (particle_elastic.h:70-143: per-bond constants given).
 * xyz N*3; p1/p2/layer/Kn/Tv per directed bond; particle_volume and
 * nneighbors from the UnitCell (unit_cell.h).  Every bond must have an
 * opposite bond in the same layer (LPM_ERR_TOPOLOGY otherwise). */
/* Selects the CUDA device for the calling host thread's later lpm_create
 * calls (the library links its own CUDA runtime, so a device chosen through
 * another runtime instance does not carry over).  Every later call on a
 * handle must come from a thread whose device is the handle's: the library
 * launches on the handle's stream and does not switch devices itself.
 * Library-level addition: the reference runs on the host only. */
int lpm_set_device(int device);

int lpm_create(int dim, int n, int64_t nb, const double* xyz, const int* p1, const int* p2, const int* layer,
               const double* Kn, const double* Tv, double particle_volume, int nneighbors, lpm_handle** out);
int lpm_destroy(lpm_handle* h);
/* Human-readable text of the last error on this handle (or global). */
const char* lpm_last_error(const lpm_handle* h);

int lpm_num_bonds(const lpm_handle* h, int64_t* nb);
int lpm_num_blocks(const lpm_handle* h, int64_t* nblocks);
/* The conns pattern (Particle::conns, assembly.h:236-266) as CSR:
 * cptr[N+1], cidx[nblocks]; and the stored bond order: bptr[N+1], bp2[Nb],
 * blayer[Nb], opp[Nb] (the opposite bond found by particle.h:207-209). */
int lpm_get_pattern(const lpm_handle* h, int64_t* cptr, int* cidx);
int lpm_get_bonds(const lpm_handle* h, int64_t* bptr, int* bp2, int* blayer, int64_t* opp);

/* Field transfer (host <-> device), sizes as listed with the field ids. */
int lpm_upload(lpm_handle* h, int field, const double* src);
int lpm_download(lpm_handle* h, int field, double* dst);
/* Particle::disp_constraint for all particles: N*3 ints (0/1). */
int lpm_set_mask(lpm_handle* h, const int* mask);
int lpm_get_mask(const lpm_handle* h, int* mask);

/* Material law of all particles (the particle class the reference
 * Assembly was built with) and its parameters: params holds nparams values
 * for every particle, or N*nparams values when per_particle is set.  Resets
 * the state variables to the class constructors' values.
 *   LPM_LAW_ELASTIC      ParticleElastic        {critical_bstrain}
 *   LPM_LAW_DAMAGE       ParticleElasticDamage  {k0, k1, damage_threshold}
 *   LPM_LAW_J2           ParticleJ2Plasticity   {E, mu, sigmay, xi, H, A, damage_threshold}
 *   LPM_LAW_FATIGUE_HCF  ParticleFatigueHCF     {A, B, d, damage_threshold}
 * (setParticleProperty of particle_elastic.h:70-143,
 * particle_elastic_damage.h:175-254, particle_j2plasticity.h:154-201,
 * particle_fatigue_hcf.h:162-209; ParticleJ2Plasticity never sets its
 * damage_threshold, which stays 0 in the reference). */
#define LPM_LAW_ELASTIC 0
#define LPM_LAW_DAMAGE 1
#define LPM_LAW_J2 2
#define LPM_LAW_FATIGUE_HCF 3
/* Continuous softening bond law, an extension with no reference class
 * (the brittle rule of particle_elastic.h:52-68 made gradual).  Each bond
 * keeps the largest stretch s = (dis - dis0)/dis0 it has reached, kappa, and
 *   d = 0                                                 kappa <= s_c
 *   d = 1 - (s_c/kappa) (alpha s_c - kappa)/((alpha - 1) s_c)   s_c < kappa < alpha s_c
 *   d = 1                                                 kappa >= alpha s_c
 * so that a bond's force falls linearly from its peak at s_c to zero at
 * alpha s_c.  bdamage = max(bdamage, d) after each converged solve; an
 * increase above 1e-3 on some bond asks for another solve, as the static
 * damage update does.  params {alpha, s_c}; s_c is the default critical
 * stretch of the particle's bonds, which LPM_B_SCRIT overrides per bond
 * (e.g. Weibull draws shared by the two directed copies of a bond). */
#define LPM_LAW_SOFTENING 4
int lpm_set_law(lpm_handle* h, int law, const double* params, int nparams, int per_particle);
/* Particle::type of every particle and the solver's undamaged_pt_type
 * (particles of that type skip the damage updates, solver_static.h:37,57). */
int lpm_set_types(lpm_handle* h, const int* types, int undamaged_type);
/* Assembly::searchNonlocalNeighbors (assembly.h:117-130) result as CSR
 * (ptr[N+1], idx ascending per particle) and Particle::nonlocal_L. */
int lpm_set_nonlocal(lpm_handle* h, const int64_t* ptr, const int* idx, const double* nonlocal_L);
/* Assembly::updateStateVar (assembly.h:161-166): the J2 return map
 * (particle_j2plasticity.h:78-140), strain-energy damage rate
 * (particle_elastic_damage.h:150-161), fatigue energy range
 * (particle_fatigue_hcf.h:127-145). */
int lpm_update_state(lpm_handle* h);
/* SolverFatigue::updateFatigueDamage (solver_fatigue.h:75-126): nonlocal
 * damage rate and D += Ddot * dNdt; *any_new = 1 if damage moved by > 1e-3. */
int lpm_fatigue_damage(lpm_handle* h, double dNdt, int* any_new);

/* SolverStatic::updateStaticDamage (solver_static.h:31-62): the nonlocal
 * damage rate (func_phi weights, lpm.h:45-49) and each law's
 * updateParticleStaticDamage: brittle bond breaking for the elastic law
 * (particle_elastic.h:52-68), D += Ddot_nonlocal with the threshold for the
 * damage and J2 laws; *any_new = 1 when something changed noticeably. */
int lpm_update_damage(lpm_handle* h, int* any_new);

/* Boundary groups: index lists registered once, used by the BC calls below
 * (DispBC / ForceBC groups, boundary.h:10-44). */
int lpm_add_group(lpm_handle* h, const int* ids, int count, int* group_id);
/* DispBC applied by Solver::updateDisplacementBC (solver.h:130-166):
 * axis 0/1/2 ('x','y','z'), mode 0 Relative (moveBy) / 1 Absolute (moveTo
 * of that axis' value, other axes set to 0 as the reference's moveTo(dxyz)
 * does), sets disp_constraint[axis] = 1. */
int lpm_apply_disp_bc(lpm_handle* h, int group, int axis, int mode, double value);
/* ForceBC applied by Solver::updateForceBC (solver.h:168-190): the total
 * force is split evenly over the group; mode 0 Relative (+=) / 1 Absolute. */
int lpm_apply_force_bc(lpm_handle* h, int group, int mode, double fx, double fy, double fz);

/* Assembly::updateGeometry + Assembly::updateForceState
 * (assembly.h:132-138, 178-191; bond.h:30-39; particle.h:151-240;
 * particle_elastic.h:38-50). */
int lpm_update_geometry_force(lpm_handle* h);
/* Solver::updateRR + the norms of NewtonIteration (solver.h:108-128, 62-64). */
int lpm_residual(lpm_handle* h, double* norm_residual, double* norm_reaction);

/* Stiffness::reset + calcStiffness (stiffness.h:43-48, 228-263, derivative.h)
 * and, with LPM_BC_ELIMINATE, updateStiffnessDispBC (stiffness.h:265-294).
 * Builds the FP64 tangent and, when mixed precision is requested later, its
 * FP32 copy. */
int lpm_assemble(lpm_handle* h, int tangent, int bc);
/* BSR values of K (not transposed) in pattern order, dim*dim row-major.
 * LPM_ERR_STATE under the matrix-free operator (nothing is assembled). */
int lpm_get_K(const lpm_handle* h, double* vals);
/* Chooses how lpm_assemble and the solves treat the tangent.  No counterpart
 * in the reference, which always assembles (stiffness.h:228-263).  With
 * LPM_OPERATOR_MATRIX_FREE, lpm_assemble keeps the bond data the tangent is
 * made of (direction cosines, bond constants, damage, per-particle sums)
 * and each CG product applies A = K^T from it in two passes over the bonds;
 * the solves give the assembled operator's results up to rounding, for
 * both tangent variants and BC modes, at less than half the bytes per
 * product.  The operator must be assembled again after the switch. */
int lpm_set_operator(lpm_handle* h, int kind);
/* y = A' v: one product of the operator the solves use (A = K^T of the last
 * lpm_assemble, BC-eliminated when asked, assembled or matrix-free), in
 * FP64 or (LPM_PREC_MIXED) as the FP32 product of the mixed solve, whose
 * double-float result is returned summed in FP64.  v, y: host arrays of
 * n*dim.  No counterpart in the reference (Eigen applies it inside CG). */
int lpm_apply_operator(lpm_handle* h, int precision, const double* v, double* y);

/* Solver::LPM_CG (solver.h:192-217): solves with the residual as right-hand
 * side into Solver::disp.  FP64: Eigen's ConjugateGradient with its Jacobi
 * preconditioner, applied through the transposed view of the column-major
 * matrix as Eigen does for Lower|Upper; stops when |r|^2 < tol^2 |b|^2, at
 * most maxit iterations (maxit < 0: 2*n_dof).  MIXED: FP32 CG steps on an
 * FP32 copy of the same operator inside FP64 refinement, stopped on the FP64
 * residual |b - A x| <= tol |b|.  iters/relres may be NULL. */
int lpm_solve(lpm_handle* h, int precision, double tol, int64_t maxit, int64_t* iters, double* relres);
/* Solver::solveLinearSystem's position update (solver.h:97-105). */
int lpm_move_by_disp(lpm_handle* h);

/* Solver::NewtonIteration (solver.h:53-89).  *n_iter gets the iteration
 * count, max_iter on failure (status LPM_NOT_CONVERGED). */
int lpm_newton(lpm_handle* h, int max_iter, double tol, int precision, double cg_tol, int64_t cg_maxit,
               int* n_iter);

/* One boundary condition of a LoadStep (load_step.h:12-29, boundary.h). */
#define LPM_BC_DISP 0
#define LPM_BC_FORCE 1
typedef struct {
  int kind;          /* LPM_BC_DISP or LPM_BC_FORCE                       */
  int group;         /* id from lpm_add_group                             */
  int mode;          /* 0 Relative, 1 Absolute (LoadMode, lpm.h:57-61)     */
  int axis;          /* DispBC flag: 0 'x', 1 'y', 2 'z'                  */
  double value;      /* DispBC step                                        */
  double fx, fy, fz; /* ForceBC total force                                */
} lpm_bc;

/* Load-step driver. */
#define LPM_SOLVER_STATIC 0 /* SolverStatic::solveProblemStep (solver_static.h:97-149) */
#define LPM_SOLVER_STATIC_ELIMINATE 2 /* SolverStatic::solveProblemStep with the displacement-BC
                                         elimination it leaves commented out (solver_static.h:113)
                                         applied, so that damage rounds run on a constrained tangent */
#define LPM_SOLVER_FATIGUE_STATIC 1 /* SolverFatigue::solveProblemStep + the storing of
                                       solveProblemStatic (solver_fatigue.h:243-298) */
typedef struct {
  int solver;        /* LPM_SOLVER_*                                       */
  int tangent;       /* LPM_TANGENT_*                                      */
  int precision;     /* LPM_PREC_*                                         */
  int max_iter;      /* Solver::max_NR_iter                                */
  double tol;        /* Solver::tol_NR_iter                                */
  double cg_tol;     /* CG tolerance (the reference uses machine epsilon)  */
  int64_t cg_maxit;  /* < 0: 2 * n_dof                                     */
  int max_cuts;      /* cut-backs allowed before giving up                 */
} lpm_step_opts;
typedef struct {
  int newton_iters;  /* Newton iterations of the last accepted sub-step    */
  int cuts;          /* load cut-backs taken                               */
  int damage_rounds; /* damage sub-iterations (SolverStatic)               */
  int pad;
  int64_t cg_iters;  /* CG iterations of the whole step                    */
} lpm_step_result;
/* Applies one LoadStep (force BCs, then displacement BCs, in the order
 * given, as updateForceBC / updateDisplacementBC do) and solves it, halving
 * the step and retrying on Newton failure as SolverStatic::solveProblem and
 * SolverFatigue::solveProblemStatic do (solver_static.h:79-87).  Returns
 * LPM_NOT_CONVERGED after max_cuts cut-backs. */
int lpm_load_step(lpm_handle* h, const lpm_bc* bcs, int nbc, const lpm_step_opts* opts, lpm_step_result* res);

/* Assembly::storeStateVar / resetStateVar (assembly.h:140-159). */
int lpm_store_state(lpm_handle* h);
int lpm_reset_state(lpm_handle* h, int reset_xyz);

/* Counters since the last lpm_reset_stats: total CG iterations, refinement
 * sweeps, kernel launches, and, when kernel timing is on, the summed device
 * time and launch count of the CG sparse product (the dominant kernel) in
 * FP64 and in FP32. */
typedef struct {
  int64_t cg_iters_total;
  int64_t refine_sweeps;
  int64_t spmv_launches;
  double spmv_ms;
  int64_t spmv32_launches;
  double spmv32_ms;
  int64_t kernel_launches;
  int64_t mixed_fallbacks; /* mixed solves that broke down (non-finite FP32 recurrence,
                              e.g. an indefinite softened tangent) and were re-solved in FP64 */
  int64_t tangent_cg_iters; /* CG iterations of the tangent solves (lpm_tangent_begin) */
  int64_t persistent_solves; /* solves whose loop ran as one persistent kernel (lpm_set_cg_loop) */
} lpm_stats;
int lpm_get_stats(const lpm_handle* h, lpm_stats* st);
int lpm_reset_stats(lpm_handle* h);
/* Records CUDA events around every CG sparse-product launch (on the
 * handle's stream) so that lpm_get_stats reports its device time.  While it
 * is on, the solves launch their iterations one by one from the host instead
 * of as one CUDA graph (same kernels, same results). */
int lpm_set_kernel_timing(lpm_handle* h, int on);
/* How lpm_solve runs its iteration loop.  No counterpart in the reference
 * (Eigen's loop runs on the host, solver.h:192-217).
 *   LPM_CG_LOOP_GRAPH       one CUDA graph per solve: per iteration the
 *                           product, the update and the direction kernels,
 *                           with the loop and reliable-update conditions set
 *                           on the device.
 *   LPM_CG_LOOP_PERSISTENT  one cooperative kernel per solve whose blocks
 *                           stay resident and meet at grid barriers (three
 *                           per iteration, two more per reliable update);
 *                           for systems too small to fill the GPU, where the
 *                           graph's per-kernel overheads dominate.  Same
 *                           recurrence, same stopping rule; the sums are
 *                           folded over another number of blocks, so the
 *                           last bits differ from the graph's.
 *   LPM_CG_LOOP_AUTO        (default) persistent when the rows fit one
 *                           resident wave with a thread each and, for the
 *                           mixed solve, the FP32 operator fits in half of
 *                           L2; else the graph.
 * Both precisions have both loops.  The matrix-free operator and kernel
 * timing always use the graph or host loop.  A barrier wait that gives up (a
 * bounded spin) ends the solve with LPM_ERR_STATE. */
#define LPM_CG_LOOP_AUTO 0
#define LPM_CG_LOOP_GRAPH 1
#define LPM_CG_LOOP_PERSISTENT 2
int lpm_set_cg_loop(lpm_handle* h, int mode);
/* Preconditioner of the mixed-precision solve.  The reference uses Jacobi
 * (Eigen's DiagonalPreconditioner, solver.h:195-206), the default here.
 *   LPM_PRECOND_COARSE  Jacobi plus a coarse correction, M^-1 = D^-1 +
 *                       P (P^T A P)^-1 P^T, with P the rigid-body modes of
 *                       boxes of particles of edge `box` (model length
 *                       units, by initial position; 0: an edge that gives
 *                       about 480 coarse DOFs), zero on eliminated DOFs.
 *                       The iteration count then depends on the box and no
 *                       longer grows with the lattice (the full-size notched
 *                       plate: about 260 iterations against 1,900).  At most
 *                       1,024 coarse DOFs (LPM_ERR_ARG beyond); the coarse
 *                       operator and its dense inverse are rebuilt after
 *                       each assembly.  Needs the assembled symmetric
 *                       tangent (LPM_ERR_STATE otherwise) and runs the
 *                       mixed solve as one persistent kernel whatever
 *                       lpm_set_cg_loop says.  The FP64 solve keeps Jacobi;
 *                       the tangent solves (lpm_tangent_begin) use it as
 *                       BiCGSTAB's right preconditioner.  A new box edge
 *                       rebuilds the aggregates on the next solve (the
 *                       previous arrays stay allocated until lpm_destroy).
 * The same solution to the solve tolerance; other iterates and counts. */
#define LPM_PRECOND_JACOBI 0
#define LPM_PRECOND_COARSE 1
int lpm_set_preconditioner(lpm_handle* h, int kind, double box);
/* The aggregates LPM_PRECOND_COARSE forms, without a device: boxes of edge
 * `box` (0: automatic) from the lowest corner of the particles' bounding
 * box, numbered in the order of their first particle.  xyz0: n*3 initial
 * positions; agg[n] receives each particle's aggregate, *nagg their count
 * (times 3 in 2-D, 6 in 3-D: the coarse DOFs), *edge (may be NULL) the edge
 * used. */
int lpm_coarse_boxes(int dim, int n, const double* xyz0, double box, int* agg, int* nagg, double* edge);
/* The handle's CUDA stream (cudaStream_t), for callers that time or order
 * work around the library. */
int lpm_get_stream(const lpm_handle* h, void** stream);
/* Blocks until the handle's stream is idle. */
int lpm_synchronize(lpm_handle* h);

/* One fatigue cycle: SolverFatigue::solveProblemOneCycle (solver_fatigue.h:
 * 212-233) on the load steps generateLoadCycle builds (solver_fatigue.h:
 * 128-172).  bcs_unit are the boundary conditions of a unit load increment
 * (the LoadUniaxialDisp / LoadUniaxialForce / LoadDogBoneDisp / LoadCTForce
 * templates of load_step_fatigue.h with their load set to 1); the cycle
 * applies them scaled by (f1 - f0)/n_interval in n_interval steps, then by
 * (f2 - f1)/n_interval in n_interval steps.  Each step assembles the
 * BC-eliminated tangent, runs Newton (opts: tangent, precision, max_iter,
 * tol, cg_tol, cg_maxit; no cut-back, as in the reference) and updates the
 * state variables; then the nonlocal fatigue damage rate and damage are
 * updated with dNdt, the state is stored and the force state refreshed.
 * res (may be NULL) sums the Newton and CG iterations of the cycle and
 * reports whether new damage appeared. */
typedef struct {
  int newton_iters;      /* Newton iterations, all steps of the cycle    */
  int unconverged_steps; /* steps that hit max_iter (kept, as the reference does) */
  int new_damage;        /* updateFatigueDamage found a damage change   */
  int pad;
  int64_t cg_iters;      /* CG iterations of the cycle                  */
} lpm_cycle_result;
int lpm_fatigue_cycle(lpm_handle* h, const lpm_bc* bcs_unit, int nbc, double f0, double f1, double f2,
                      int n_interval, double dNdt, const lpm_step_opts* opts, lpm_cycle_result* res);

/* Cyclic loading: SolverFatigue::solveProblemCyclic (solver_fatigue.h:
 * 174-210) with generateLoadCycle (:128-172), run inside the library.  The
 * load spectrum (readLoad's format, solver_fatigue.h:41-60: f_min, then
 * f_max, f_min pairs; an odd count of values) is copied to the device once
 * per call; cycle N's increments (f1 - f0)/n_interval and (f2 - f1)/n_interval
 * with f0, f1, f2 = spectrum[2N..2N+2] are formed there and scale the unit
 * boundary conditions bcs_unit on the device.  Each simulated cycle is
 * lpm_fatigue_cycle's work with dNdt from the time map (LPM_TIME_LINEAR:
 * (int)(1/tau); LPM_TIME_EXPONENTIAL: (int)(exp(t/tau)/tau), t counting
 * simulated cycles), after which N += dNdt; the run ends when N reaches
 * (count-1)/2, after max_cycles simulated cycles (if > 0), or after a cycle
 * with dNdt = 0 (where the reference would loop for ever).  One record per
 * simulated cycle goes to records (up to capacity): N after the cycle,
 * dNdt, the cycle's iteration counts, whether new damage appeared, and the
 * mean strain energy the reference prints (first state variable over the
 * particles that damage).  *ncycles = simulated cycles run.  Returns
 * LPM_NOT_CONVERGED if any step of any cycle hit max_iter (kept, as the
 * reference keeps it). */
#define LPM_TIME_LINEAR 0
#define LPM_TIME_EXPONENTIAL 1
typedef struct {
  int64_t N;             /* real cycle count after this simulated cycle  */
  int dNdt;              /* real cycles this simulated cycle stood for   */
  int newton_iters;
  int unconverged_steps;
  int new_damage;
  int64_t cg_iters;
  double mean_energy;    /* "Average strain energy" of solveProblemCyclic */
} lpm_fatigue_record;
int lpm_fatigue_run(lpm_handle* h, const lpm_bc* bcs_unit, int nbc, const double* spectrum, int64_t nvalues,
                    int n_interval, int time_mode, double tau, int64_t max_cycles, const lpm_step_opts* opts,
                    lpm_fatigue_record* records, int64_t capacity, int64_t* ncycles);

/* ---- Adjoint (backward) of a converged load step ----
 * No counterpart in the reference, whose only derivative of the internal
 * force is the forward-difference tangent (Stiffness::localStiffnessFD,
 * stiffness.h:103-154).  lpm_load_step is the forward half of the pair.
 *
 * Response J = sum dJdx . x + sum dJdpin . Pin over the N*dim particle DOFs
 * (x the current positions, Pin the internal forces; either array may be
 * NULL).  A reaction over a constrained group is dJdpin = 1 on the group's
 * DOFs along the axis; a gauge displacement is dJdx.  At the converged
 * state (free DOFs in equilibrium) lpm_backward_step solves the adjoint
 * system H_ff lambda = (dJdx + H dJdpin)_f with H = dPin/dx, the exact
 * Jacobian applied matrix-free (not the analytical tangent, which leaves out
 * the change of bond directions), by Jacobi-PCG at cg_tol (cg_maxit < 0:
 * 2*n_dof), and returns dJ/dKn and dJ/dTv for every directed bond in stored
 * bond order (lpm_get_bonds).  accumulate = 1 adds to the gradients of the
 * previous calls (a response summed over load steps); 0 starts afresh.
 * Every bond must be intact or broken on both sides (the energy-conserving
 * case, H symmetric); partially damaged bonds give LPM_ERR_STATE.  The
 * device gradients persist between calls; dJdKn/dJdTv may be NULL. */
typedef struct {
  int64_t cg_iters;  /* adjoint CG iterations */
  double relres;     /* final relative residual of the adjoint solve */
} lpm_adjoint_result;
int lpm_backward_step(lpm_handle* h, const double* dJdx, const double* dJdpin, double cg_tol, int64_t cg_maxit,
                      int accumulate, double* dJdKn, double* dJdTv, lpm_adjoint_result* res);
/* y = H v with H = dPin/dx at the current state (all DOFs, N*dim each):
 * the exact Jacobian-vector product the adjoint uses. */
int lpm_apply_jacobian(lpm_handle* h, const double* v, double* y);

/* Forward-mode (tangent-linear) sensitivity of a J2 load history with respect
 * to the law's parameters, for responses of the stress-strain curve.
 * Between lpm_tangent_begin and lpm_tangent_end every converged load step
 * (lpm_load_step) also carries ndir tangent states along: dparams
 * (ndir x n x np, host, np the law's parameters per particle) gives each
 * direction's change of the parameters, e.g. 1 in the yield-stress column
 * for d/d(sigma_y).  At each state update (lpm_update_state, or the one
 * inside lpm_load_step: solver_fatigue.h:266, solver_static.h:122), first,
 * at the converged equilibrium: the change of the
 * equilibrium, H_ff dx_f = -(dPin/d dLp . d dLp)_f with dx = 0 on
 * constrained DOFs (CG on the exact Jacobian to `tol`); the change of the
 * internal forces (LPM_T_PIN) and positions (LPM_T_XYZ) of that equilibrium;
 * then the radial return (particle_j2plasticity.h:78-140) differentiated,
 * which advances the tangents of the state variables and of dLp.  A
 * response R(Pin, x) summed over steps has dR/dtheta = sum over steps of
 * its partial derivatives times these tangents.  E and nu also set the
 * bond constants (per-bond inputs): a direction that changes them gives the
 * constants' changes with lpm_tangent_bond_constants (dKn, dTv: nb each,
 * stored bond order; e.g. from the UnitCell map's derivative) after
 * lpm_tangent_begin.  Damage is held fixed
 * (bonds intact or broken on both sides; LPM_ERR_STATE otherwise); a
 * load step that cuts back fails with LPM_ERR_STATE. */
#define LPM_T_PIN 1 /* n x dim: d Pin / d theta at the step's equilibrium */
#define LPM_T_XYZ 2 /* n x dim: d x / d theta at the step's equilibrium */
#define LPM_T_DAMAGE 3 /* n: d damage / d theta of each particle (HCF law) */
int lpm_tangent_begin(lpm_handle* h, int ndir, const double* dparams, double tol);
int lpm_tangent_bond_constants(lpm_handle* h, int dir, const double* dKn, const double* dTv);
/* Softening law (LPM_LAW_SOFTENING, configuration 3's damage): the same
 * forward-mode tangents follow the damage history instead of holding it
 * fixed.  dparams may be NULL (the law's alpha is not a direction); a
 * direction changes the bond constants (lpm_tangent_bond_constants, e.g.
 * dKn = Kn/E, dTv = Tv/E for d/dE) and/or the per-bond critical stretch
 * (lpm_tangent_bond_scrit: d s_c per directed bond, stored order, e.g.
 * s_c/lambda for the scale lambda of the Weibull draws).  Each damage round
 * of lpm_load_step (LPM_SOLVER_STATIC_ELIMINATE; solver_static.h:107-136)
 * then solves the equilibrium's change on the exact Jacobian of the
 * partially damaged state, which is not symmetric (BiCGSTAB with its exact
 * diagonal), and differentiates the damage update that follows: the
 * largest stretch kappa = max(kappa, s) where s sets it, and
 * d = D(kappa, s_c) where d rises.  LPM_T_PIN after a step is the change of
 * the internal forces at the step's final equilibrium, so a reaction's
 * derivative is their sum over the constrained group; the peak reaction's
 * is that of the step where it peaks.  The derivative is that of the
 * discrete algorithm (rounds, thresholds) at fixed round counts. */
int lpm_tangent_bond_scrit(lpm_handle* h, int dir, const double* dscrit);
/* HCF fatigue law (LPM_LAW_FATIGUE_HCF, configuration 5): dparams gives
 * each direction's change of the per-particle {A, B, d, threshold} (e.g. A
 * in column 0 for d/d(log A) scaling, 1 in column 1 for d/dB).  Through the
 * cycles of lpm_fatigue_cycle / lpm_fatigue_run the tangents follow each
 * step's equilibrium (the partially damaged Jacobian, BiCGSTAB), the strain
 * energy's history (U_min, U_max, U_hist of particle_fatigue_hcf.h:127-145,
 * with the branch each takes), the local rate A U_hist^B (U_max - U_min)^d,
 * its nonlocal average with position-dependent weights
 * (solver_fatigue.h:79-116), the damage update with the cycle jump
 * (particle_fatigue_hcf.h:147-160) and the bond damage the force pass raises
 * to the larger particle damage.  LPM_T_DAMAGE gives d damage / d theta per
 * particle, so a crack-length measure sum_i w_i D_i (e.g. the damage along
 * the ligament times the spacing) has the derivative sum_i w_i dD_i.  The
 * tangents ride along with the forward run: no checkpoint or recompute is
 * needed for a few parameters. */
int lpm_tangent_get(const lpm_handle* h, int dir, int field, double* dst);
int lpm_tangent_end(lpm_handle* h);

/* Device-resident snapshots of a step's state: positions, last converged
 * positions, external loads, constraints, particle damage and state
 * variables, bond damage, plastic stretch and their last converged copies.
 * Restore reloads one and recomputes the force state.  They extend
 * Assembly::storeStateVar/resetStateVar (assembly.h:140-166), which keep a
 * single copy, to the many an adjoint over a load history replays from
 * (checkpoint every k steps, recompute the steps between).  About
 * 1 GB per snapshot at a million particles (18M bonds). */
int lpm_checkpoint_save(lpm_handle* h, int* id);
int lpm_checkpoint_restore(lpm_handle* h, int id);
int lpm_checkpoint_drop(lpm_handle* h, int id);

/* ---- Neighbour search on the device (set-up) ----
 * Assembly::createBonds (assembly.h:212-234): directed bonds i -> j for
 * every j != i with distance < 1.01*cutoff1, layer 0 when also below
 * 1.01*cutoff0, sorted by (i, j), the order createBonds pushes them.  The
 * distance arithmetic is the reference's, so the result is bit-for-bit its
 * O(N^2) search, found through a uniform cell grid.  xyz: N*3 host array.
 * With p2 == NULL only *nb is returned; otherwise p1/p2/layer must hold
 * capacity entries (LPM_ERR_ARG with *nb set when they do not).  p1 may be
 * NULL.  Runs on the calling thread's current device. */
int lpm_find_bonds(int n, const double* xyz, double cutoff0, double cutoff1, int64_t capacity, int* p1, int* p2,
                   int* layer, int64_t* nb);
/* Assembly::searchNonlocalNeighbors (assembly.h:117-130): for every
 * particle i the ids j (ascending, i itself included) with distance <
 * radius[i] (= cutoff_ratio * nonlocal_L of particle i), as CSR ptr[N+1] /
 * idx[total].  With idx == NULL only *total is returned. */
int lpm_find_neighbors(int n, const double* xyz, const double* radius, int64_t capacity, int64_t* ptr, int* idx,
                       int64_t* total);

/* Allocation-free Jacobi-CG solve.  No counterpart in the reference: it is
 * for callers that cannot allocate device memory while they solve (a
 * real-time loop that reserved its memory up front, a host framework whose
 * allocator owns the device).  The caller passes device buffers: the
 * operator in block CSR (ptr[n+1] int64, col[nnz] int32, vals[nnz*dim*dim]
 * row-major blocks, applied as y = A x), the right-hand side b and the
 * solution x (n*dim doubles each).  The iteration is lpm_solve's FP64 one
 * (Jacobi preconditioner from the diagonal blocks, zero start,
 * |r|^2 < tol^2 |b|^2, maxit < 0: 2*n*dim); its product reads the block CSR
 * row by row, so an iteration is slower than one of lpm_solve.
 * Work vectors live in one fixed device array inside the library, sized for
 * n*dim <= LPM_NOALLOC_MAX_DOF (about 33.6 MB, created on each GPU when the
 * library's device code is loaded there, held until the process exits);
 * larger systems are refused with LPM_ERR_ARG.  The first call on a device
 * looks up that array's address and caches it: make it before any stream
 * capture, and do not use the library across a device reset, which
 * invalidates the cached address.  All calls share the array, so calls that
 * overlap on the same GPU race.  Runs on `stream` (NULL: the default stream)
 * and returns when the solve is done (it synchronises with `stream` to read
 * the counts back); iters/relres may be NULL. */
#define LPM_NOALLOC_MAX_DOF 1048576
int lpm_cg_solve_noalloc(int dim, int n, const int64_t* ptr, const int* col, const double* vals, const double* b,
                         double* x, double tol, int64_t maxit, void* stream, int64_t* iters, double* relres);

#ifdef __cplusplus
}
#endif
#endif
