/* CPU oracle for the LPM quasi-static Newton load step (TEST INFRASTRUCTURE).
 *
 * A plain C++ restatement of the reference's algorithm, used only by tests/,
 * the smoke check and the CPU-baseline leg of bench.py.  The product never
 * links, loads or calls it.  Each function cites the reference lines it
 * follows (paths are relative to the LPM-MAC project root).
 *
 * Pinning: tests/golden/ holds vectors produced by the reference headers
 * themselves (compiled unmodified against a documented Eigen stand-in, see
 * oracle/ref_driver.cpp); tests check this restatement against them.
 */
#ifndef LPM_ORACLE_H
#define LPM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lo_sys lo_sys;

/* particle fields (lo_get_particle / lo_set_particle) */
enum lo_pfield {
  LO_XYZ = 0,        /* N*3 current positions                        */
  LO_XYZ0 = 1,       /* N*3 initial positions                        */
  LO_PIN = 2,        /* N*3 internal force                           */
  LO_PEX = 3,        /* N*3 external force                           */
  LO_STRESS = 4,     /* N*6 xx yy zz yz xz xy                        */
  LO_DVIS = 5,       /* N   damage_visual                            */
  LO_DLE_TOT = 6,    /* N*2 per-layer sum of dLe                     */
  LO_TDLE_TOT = 7,   /* N*2 per-layer sum of Tv*dLe                  */
  LO_CS_SUM = 8,     /* N*2*3 per-layer sum of direction cosines     */
  LO_DAMAGE = 9,     /* N   particle damage                          */
  LO_XYZ_LAST = 10,  /* N*3 last converged positions                 */
  LO_STATE = 11,     /* N*nstate state variables                     */
  LO_DDOT_LOCAL = 12 /* N   local damage rate                        */
};
/* bond fields (bond CSR order: by p1, then layer, then input order) */
enum lo_bfield {
  LO_BFORCE = 0, LO_BDAMAGE = 1, LO_DLE = 2, LO_DIS = 3, LO_BSTRAIN = 4,
  LO_CS = 5, /* Nb*3 */
  LO_KN = 6, LO_TV = 7, LO_DIS0 = 8, LO_DLP = 9,
  LO_SCRIT = 10, /* softening law: critical stretch per bond      */
  LO_KAPPA = 11  /* softening law: largest stretch reached        */
};

/* Creates a system.  Bonds are directed (p1 -> p2) with layer 0 or 1; the
 * library orders them by (p1, layer) keeping input order inside each group,
 * which is the order Particle::bond_layers holds them (assembly.h:212-234,
 * assembly.h:390-424).  Returns NULL and sets *err on invalid input
 * (-1 bad sizes/ids, -2 a bond without its opposite bond). */
lo_sys* lo_create(int dim, int n, long nb, const double* xyz, const int* p1, const int* p2, const int* layer,
                  const double* Kn, const double* Tv, double particle_volume, int nneighbors, int* err);
void lo_destroy(lo_sys* s);
void lo_set_threads(int nthreads);

long lo_num_bonds(const lo_sys* s);
long lo_num_blocks(const lo_sys* s);
/* bptr[N+1], bp2[Nb], blayer[Nb], bsrc[Nb] (input index of each stored bond),
 * opp[Nb], cptr[N+1], cidx[num_blocks] (conns pattern, assembly.h:236-266) */
void lo_get_topology(const lo_sys* s, long* bptr, int* bp2, int* blayer, long* bsrc, long* opp, long* cptr,
                     int* cidx);

void lo_get_particle(const lo_sys* s, int field, double* out);
void lo_set_particle(lo_sys* s, int field, const double* in);
void lo_get_bond(const lo_sys* s, int field, double* out);
void lo_set_bond(lo_sys* s, int field, const double* in);
void lo_set_mask(lo_sys* s, const int* mask); /* N*3 disp_constraint */

/* Material law of all particles and its parameters (uniform, or N*nparams
 * when per_particle is set):
 *   0 ParticleElastic        {critical_bstrain}
 *   1 ParticleElasticDamage  {k0, k1, damage_threshold}
 *   2 ParticleJ2Plasticity   {E, mu, sigmay, xi, H, A, damage_threshold}
 *   3 ParticleFatigueHCF     {A, B, d, damage_threshold}
 *   4 softening bond law     {alpha, s_c}: no reference class; d(kappa)
 *     falls from 0 at kappa = s_c to 1 at alpha*s_c with a linearly
 *     softening bond force, kappa the largest stretch (dis-dis0)/dis0
 * Resets the state variables to the constructors' values. */
void lo_set_law(lo_sys* s, int law, const double* params, int nparams, int per_particle);
void lo_set_types(lo_sys* s, const int* types, int undamaged_type);
/* Assembly::searchNonlocalNeighbors result (CSR, ascending ids) and each
 * particle's nonlocal length scale. */
void lo_set_nonlocal(lo_sys* s, const long* ptr, const int* idx, const double* L);
void lo_update_state(lo_sys* s);               /* Assembly::updateStateVar */
int lo_static_damage(lo_sys* s);               /* SolverStatic::updateStaticDamage */
int lo_fatigue_damage(lo_sys* s, double dNdt); /* SolverFatigue::updateFatigueDamage */
void lo_get_ddot(const lo_sys* s, double* local, double* nonlocal);
int lo_num_state(const lo_sys* s);

/* Assembly::updateGeometry + updateForceState (assembly.h:132-138,178-191) */
void lo_update_geometry_force(lo_sys* s);
/* Solver::updateRR (solver.h:108-128): r (N*dim) and norms */
void lo_residual(lo_sys* s, double* r, double* norm_r, double* norm_R);

/* Stiffness::calcStiffness (stiffness.h:228-263, derivative.h).
 * sym = 0: as written (K_ii[1][0] stays 0, derivative.h:38);
 * sym = 1: K_ii[1][0] = K_ii[0][1].
 * bc  = 1: then Stiffness::updateStiffnessDispBC (stiffness.h:265-294). */
void lo_assemble(lo_sys* s, int sym, int bc);
/* BSR values of K (not transposed): blocks in conns order, dim*dim row-major */
void lo_get_K(const lo_sys* s, double* vals);

/* Jacobi PCG on the operator K^T, as Eigen::ConjugateGradient<.., Lower|Upper>
 * applies a column-major matrix (solver.h:192-217).  Returns 0 on success
 * (error <= tol), 1 when not converged. */
int lo_cg(lo_sys* s, const double* b, double* x, double tol, long maxit, long* iters, double* err);

/* Solver::NewtonIteration (solver.h:53-106): returns the iteration count,
 * max_iter on failure.  cg_* give the linear solve; iteration records
 * (cg iterations, cg error, residual norm) go to an internal log. */
int lo_newton(lo_sys* s, int max_iter, double tol, double cg_tol, long cg_maxit);
long lo_log_size(const lo_sys* s);
void lo_get_log(const lo_sys* s, double* out); /* 3 doubles per record */
void lo_clear_log(lo_sys* s);

/* Relative displacement increment on masked DOFs (DispBC Relative,
 * solver.h:130-166): x[i][k] += d[i*3+k] where apply[i*3+k] != 0, and sets
 * the mask there.  Force BC Relative: Pex += f (solver.h:168-190). */
void lo_apply_disp_bc(lo_sys* s, const int* apply, const double* d);
void lo_add_pex(lo_sys* s, const double* f);

/* One static load step with the step cut-back of solver_static.h:64-95 and
 * solver_fatigue.h:243-275.  bc_elim selects the tangent BC treatment
 * (0: SolverStatic, 1: SolverFatigue, 2: SolverStatic's damage rounds on
 * the BC-eliminated tangent).  Returns the number of Newton
 * iterations of the accepted step, or -1 after max_cuts cut-backs. */
int lo_load_step(lo_sys* s, const int* apply, const double* d, const double* f, int sym, int bc_elim, int max_iter,
                 double tol, double cg_tol, long cg_maxit, int max_cuts);

void lo_store_state(lo_sys* s);            /* Assembly::storeStateVar (assembly.h:140-148) */
void lo_reset_state(lo_sys* s, int reset_xyz); /* Assembly::resetStateVar (assembly.h:150-159) */

#ifdef __cplusplus
}
#endif
#endif
