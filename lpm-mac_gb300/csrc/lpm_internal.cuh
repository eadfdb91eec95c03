// Internal declarations shared by the liblpmgpu translation units.
//
// Device layout (all arrays live in HBM for the life of the handle):
//   particles  SoA, positions interleaved xyz (3 doubles per particle even in
//              2-D, z = 0), per-layer sums [i][layer], stress [i][6]
//   bonds      CSR by owner particle (bptr), layer 0 then layer 1 inside a
//              particle (lptr = first layer-1 bond), each group in input
//              order, as Particle::bond_layers holds them; SoA per field
//   pattern    conns CSR (cptr, cidx), ascending ids, self included
//   operator   A = K^T over the same pattern: block (j, i) of A is K_ij
//              transposed.  Sliced block-ELL storage in groups of four
//              with a one-block tail: rows are grouped in slices of 32
//              consecutive rows, each slice holds 32 x w slots with w its
//              longest row, g4 = w rounded down to a multiple of 4.  Block k
//              of row j sits in slot
//                sell_ptr[j/32] + 128*(k/4) + 4*(j%32) + k%4     (k < g4),
//                sell_ptr[j/32] + 32*g4 + 32*(k-g4) + j%32       (k >= g4),
//              so a thread reads four consecutive blocks of its row with one
//              vector load, the 32 rows of a slice read 512 contiguous bytes,
//              and the last w - g4 blocks (at most three) are read one per
//              row, 128 contiguous bytes per slice: no slot is padding in a
//              slice of equal rows.  Values are stored one array per block
//              element ("element-major"): A[e * nslots + slot], e = r*dim + s.
//              Padding slots of a row's last group of four hold zeros and
//              point at the row itself
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "lpm_gpu.h"

namespace lpm {

constexpr int NL = 2;            // neighbour layers
constexpr double EPS = 1e-6;     // lpm.h:37
constexpr int kRedThreads = 256; // threads per block of the reduction kernels

// Scalars of one CG run, resident on the device.
struct CgScalars {
  double rhs_norm2;   // |b|^2
  double threshold;   // max(tol^2 |b|^2, DBL_MIN)
  double abs_new;     // r . z
  double alpha, beta;
  double rr;          // |r|^2 of the last update
  long long it;       // completed iterations (Eigen's count)
  long long maxit;
  int done;           // 0 running, 1 converged, 2 iteration cap, 3 non-finite
  int ru;             // mixed solve: a reliable update is pending
  int pfault;         // persistent solve: a grid-barrier wait gave up
  double rmax;        // mixed solve: largest |r| since the last reliable update
  long long ru_count; // mixed solve: reliable updates taken
  long long graph_passes;  // mixed solve: loop passes run by the solve graph
  double zcoef;       // mixed solve: p = zcoef z + beta p (1 except right after an update)
  unsigned long long bmax_bits;  // mixed solve: bits of max |b| (non-negative doubles order as integers)
  double bscale;      // mixed solve: power of two that brings max |b| to [1, 2)
  float alpha32, beta32, zcoef32;  // mixed solve: FP32 copies, so that the vector kernels convert nothing
  float alpha32lo, beta32lo;       // mixed solve: alpha - alpha32 and beta - beta32 rounded (double-float pairs)
};

// Deterministic grid reductions: each block writes a partial, the last block
// to finish (atomic ticket) folds the partials in index order.
struct RedBuf {
  double* partials;       // [kMaxRedBlocks * 4]
  unsigned int* ticket;   // one counter per reduction slot
};
constexpr int kMaxRedBlocks = 2048;
constexpr int kSlice = 32;  // rows per slice of the sliced operator
constexpr int kVec = 4;     // consecutive blocks of a row stored together

// Row j of the sliced operator: blocks k < g4 in groups of four from base
// (slot base + 128*(k/4) + k%4), the others one per slot from tail (slot
// tail + 32*(k - g4)).
struct SellRow {
  int64_t base, tail;
  int g4;
};
__host__ __device__ __forceinline__ SellRow sell_row(const int64_t* sell_ptr, int j) {
  const int64_t s0 = sell_ptr[j / kSlice];
  const int w = (int)((sell_ptr[j / kSlice + 1] - s0) / kSlice);  // the slice's longest row
  const int g4 = w / kVec * kVec;
  return SellRow{s0 + (int64_t)(j % kSlice) * kVec, s0 + (int64_t)g4 * kSlice + j % kSlice, g4};
}
__host__ __device__ __forceinline__ int64_t sell_slot(const SellRow& r, int k) {
  return k < r.g4 ? r.base + (int64_t)(k / kVec) * (kSlice * kVec) + (k % kVec) : r.tail + (int64_t)(k - r.g4) * kSlice;
}
// Slots of row j the products read: its blocks, and in the group region the
// padding of its last group of four.
__host__ __device__ __forceinline__ int sell_read_len(const SellRow& r, int len) {
  return len <= r.g4 ? (len + kVec - 1) / kVec * kVec : len;
}

struct Group {
  int* ids;
  int count;
};

struct Dev {
  // particles
  double *x, *x0, *xlast, *pin, *pex, *stress, *dvis, *dle_tot, *tdle_tot, *cs_sum, *damage, *damage_last;
  int *mask, *nbonds;
  // per particle and layer, for the tangent: T = sum w Tv n, M = sum w (2Kn+Tv) n n^T
  // (upper triangle xx xy xz yy yz zz)
  double *tsum, *msum;
  // bonds
  int64_t *bptr, *lptr;
  int *bp2, *blayer, *opp;
  int *sbond, *sp2;  // per (particle, layer) segment: bond ids and partners sorted by partner id
  double *Kn, *Tv, *dis0, *dis, *dis_last, *dLe, *dLp, *dLp_last, *bstrain, *cs, *bforce, *bforce_last, *bdamage,
      *bdamage_last;
  // pattern (CSR) and its sliced layout
  int64_t* cptr;
  int *cidx, *diag_slot;  // diag_slot: slot of the diagonal block (sliced)
  int64_t* sell_ptr;      // [nslice + 1] first slot of each slice
  int* scol;              // [nslots] column (particle id) of each slot
  int* rowlen;            // [n] blocks in each row
  // operator values
  double* A64;
  float* A32;
  float* S32;  // [n * dim * dim] block row sums of A64, rounded (difference-form FP32 product)
  short* soff16;  // [nslots] column - row of each slot read by the FP32 product, valid when soff16_ok
  // solver vectors (n_dof each)
  double *rhs, *disp, *x64, *r64, *p64, *q64, *invd64;
  float *b32, *x32, *r32, *p32, *q32, *invd32;
  // mixed solve: low words of the residual, the product and the solution
  // increment (each a double-float pair with the FP32 vector above)
  float *r32lo, *q32lo, *x32lo;
  // matrix-free operator (lpm_set_operator): the bonds in slices of 32
  // particles (bond k of particle i at slot mbase[i/32] + 32 k + i%32), each
  // slot holding its partner (layer in the top bit) and, in FP64 and FP32,
  // the opposite bond's direction cosines, a' - t' and t' (t = w Tv,
  // a = w (2 Kn + Tv)) as five arrays of mslots; per particle and layer the
  // direction-cosine sums S and the sums U = S + sum n', V = T + sum t' n'
  // ([n][2][3]); per particle the block row sums of A ([n][9]); the
  // diagonal of K per DOF; the first pass's two sums per particle and layer
  int64_t* mbase;
  unsigned* mp2;
  double *m64, *mS64, *mU64, *mV64, *mR64, *mdiag, *mHF64;
  float *m32, *mS32, *mU32, *mV32, *mR32, *mHF32;
  // cyclic driver: the load spectrum, and the cycle's two load increments
  // and mean strain energy
  double *spectrum, *cycle;
  // reductions
  RedBuf red;
  CgScalars* cg;   // device scalars
  unsigned long long* gbar;  // persistent solve: grid-barrier arrivals (zeroed before each launch)
  // coarse-space preconditioner (lpm_coarse.cu): aggregate of each particle,
  // members of each aggregate, coupled aggregate pairs, offsets from the
  // aggregate centroids; the coarse operator and its inverse (dense, nc x nc),
  // the modes kept, the restriction and coarse solution, the preconditioned
  // residual
  int *cagg, *cmem_ptr, *cmem, *cpair, *cprow_ptr, *cprow, *cact, *cfault;
  float* coff;
  double *cA, *cA2, *cAinv, *cyc, *cec;  // cAinv: cA or cA2, wherever the inversion ended
  float* cz;
  double* norms;   // device results of small reductions [8]
  // per-particle flags for the BC elimination
  unsigned char* fixed;
  // critical bond strain per particle (elastic law)
  double* crit;
  // material laws: type, parameters, state variables, damage rates
  int* ptype;
  double *pp, *state, *state_last, *ddot_local, *ddot_nl, *nonlocal_L;
  int64_t* nl_ptr;  // nonlocal neighbours (CSR, ascending ids)
  int* nl_idx;
  // softening law: critical stretch and largest stretch reached, per bond
  double *bcrit, *bkappa, *bkappa_last;
  // adjoint: response weights a, c; CG vectors; mu = c - lambda; d f per
  // bond; parameter gradients per bond; a device flag
  double *adj_a, *adj_c, *adj_g, *adj_lam, *adj_r, *adj_p, *adj_q, *adj_invd, *adj_mu;
  double *adj_gkn, *adj_gtv;
  int* adj_flag;
  // adjoint: sliced bond data of the exact Jacobian (32 particles per slice)
  int64_t* jbase;
  int *jslot_of, *jp2, *jopp, *jlayer;
  double *jc, *jk, *jt, *jf, *jd;
  // tangent-linear sensitivity (lpm_tangent_begin): per direction the
  // tangents of dLp [nb], of the state variables [n * nstate], of the
  // equilibrium positions and internal forces [n * dim], and the parameter
  // direction [n * np]; the stress tangent and the tangent of dLp in the
  // sliced bond layout are scratch
  double *tg_dlp, *tg_sv, *tg_x, *tg_pin, *tg_dp, *tg_stress, *tg_jdl;
  double *tg_dkn, *tg_dtv, *tg_jdk;  // per direction d Kn, d Tv [nb]; the force change in sliced layout
  // softening law: per direction the tangents of the bond damage and of the
  // largest stretch, and the direction's change of the critical stretch
  // [nb each]; BiCGSTAB work vectors (the partially damaged Jacobian is not
  // symmetric)
  double *tg_dd, *tg_dkappa, *tg_dsc, *tg_bicg;
  // HCF law: per direction the tangents of the particle damage, of the
  // local and of the nonlocal damage rate [n each]
  double *tg_dD, *tg_ddot, *tg_dnl;
};

// One device-resident copy of a step's state (lpm_checkpoint_save).
struct Checkpoint {
  void* buf = nullptr;
  size_t bytes = 0;
};

}  // namespace lpm

struct lpm_handle {
  int dim = 3, n = 0;
  int64_t nb = 0, nblk = 0;
  int64_t nslots = 0;  // sliced slots (nblk plus padding)
  int nslice = 0;
  double particle_volume = 0;
  int nneighbors = 1;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  lpm::Dev d{};
  std::vector<lpm::Group> groups;
  int law = 0;
  int law_np = 1;      // parameters per particle
  int nstate = 1;      // state variables per particle
  int undamaged = -1;  // particle type that skips damage updates
  bool have_K = false;
  bool a32_valid = false;  // FP32 copy of the operator matches A64
  bool soff16_ok = false;  // every column offset of the pattern fits 16 bits
  int sms = 0;             // multiprocessors of the device (looked up on the first mixed solve)
  int tangent = LPM_TANGENT_AS_WRITTEN;
  bool mf = false;        // the CG applies the tangent matrix-free (lpm_set_operator)
  int64_t mslots = 0;     // slots of the matrix-free bond layout
  int mnsl = 0;           // 32-particle slices of that layout
  int64_t spectrum_cap = 0;  // values the device spectrum buffer holds
  // host mirrors
  lpm::CgScalars* h_cg = nullptr;  // pinned
  double* h_norms = nullptr;       // pinned [8]
  lpm_stats stats{};
  bool timing = false;
  int cg_loop = LPM_CG_LOOP_AUTO;  // how the solves run their iteration loop (lpm_set_cg_loop)
  int precond = LPM_PRECOND_JACOBI;  // preconditioner of the mixed solve (lpm_set_preconditioner)
  double cbox = 0;                   // requested aggregate edge (0: chosen from the coarse target)
  double cedge = 0;                  // edge in use
  int cnagg = 0, cnc = 0, cnpair = 0;
  bool coarse_valid = false;         // the coarse inverse matches the operator
  int last_bc = -1;                  // BC mode of the last assembly
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<void*> allocations;
  std::vector<lpm::Checkpoint> checkpoints;
  int64_t jslots = 0;  // adjoint: slots of the sliced bond data
  int tg_ndir = 0;      // tangent directions carried by the load steps (0: off)
  int tg_cap = 0;       // directions the tangent buffers hold
  double tg_tol = 1e-12;
  bool tg_bond = false;  // some direction changes the bond constants
  // the FP64 solve's iteration loop as a graph (for the solution vector fp_graph_x)
  cudaGraph_t fp_graph = nullptr;
  cudaGraphExec_t fp_exec = nullptr;
  const void* fp_graph_x = nullptr;
  // the mixed solve's iteration loop as a graph with device-side conditions
  cudaGraph_t mx_graph = nullptr;
  cudaGraphExec_t mx_exec = nullptr;
  const void* mx_graph_spmv = nullptr;  // the FP32 product kernel the graph launches
  bool fp_graph_mf = false, mx_graph_mf = false;  // the operator form each graph was built for
};

namespace lpm {

// ---- kernels launched by the C ABI layer (definitions in the .cu files) ----
// geometry / force / residual (lpm_force.cu)
int launch_geometry_force(lpm_handle* h);
int launch_residual(lpm_handle* h, double* norm_r, double* norm_R);
int launch_move_by_disp(lpm_handle* h);
int launch_disp_bc(lpm_handle* h, const Group& g, int axis, int mode, double value);
int launch_force_bc(lpm_handle* h, const Group& g, int mode, double fx, double fy, double fz);
// the cyclic driver (lpm_fatigue_run): increments of cycle N from a device
// spectrum, BCs scaled by a device factor, mean strain energy (device out)
int launch_cycle_increments(lpm_handle* h, const double* spectrum, long long N, int n_interval, double* inc);
int launch_disp_bc_scaled(lpm_handle* h, const Group& g, int axis, int mode, double unit, const double* scale);
int launch_force_bc_scaled(lpm_handle* h, const Group& g, int mode, double fx, double fy, double fz,
                           const double* scale);
int launch_mean_state0(lpm_handle* h, double* out_dev);
// material laws (lpm_laws.cu)
int launch_update_state(lpm_handle* h);
int launch_static_damage(lpm_handle* h, int* any_new);
int launch_fatigue_damage(lpm_handle* h, double dt, int* any_new);
// pattern / tangent (lpm_tangent.cu)
int build_pattern(lpm_handle* h);
int launch_assemble(lpm_handle* h, int tangent, int bc);
int convert_A32(lpm_handle* h);
// matrix-free operator (lpm_mfree.cu): the per-assembly data, the Jacobi
// diagonal, the product q = A p with p.q and alpha (FP32 with q as a
// double-float pair, or FP64), and the mixed solve's FP64 true residual,
// launched on the handle's stream or appended to a graph after `dep`
int mf_assemble(lpm_handle* h, int tangent, int bc);
int mf_prepare_invd(lpm_handle* h, bool want32);
// (mask: the input may be nonzero on eliminated DOFs; the solves' inputs are not)
int mf_launch_product(lpm_handle* h, bool fp32, const void* p, void* q, float* qlo, bool mask = false);
int mf_launch_residual(lpm_handle* h);
int mf_graph_product(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, bool fp32, const void* p, void* q,
                     float* qlo, cudaGraphNode_t* last);
int mf_graph_residual(lpm_handle* h, cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphNode_t* last);
// coarse-space preconditioner (lpm_coarse.cu): aggregates once per handle,
// the coarse operator's inverse once per assembly
int coarse_boxes(int dim, int n, const double* x0, double box, int* agg, double* edge_out);
int coarse_setup(lpm_handle* h);
int coarse_assemble(lpm_handle* h);
// z = invd r + P A_c^-1 P^T r for FP64 device vectors (the tangent solves),
// when coarse_usable
bool coarse_usable(const lpm_handle* h);
int coarse_apply64(lpm_handle* h, const double* r, const double* invd, double* z);
// solvers (lpm_cg.cu)
int solve_fp64(lpm_handle* h, double tol, long long maxit, long long* iters, double* relres);
int solve_mixed(lpm_handle* h, double tol, long long maxit, long long* iters, double* relres);
int prepare_invd(lpm_handle* h, bool want32);
int apply_operator(lpm_handle* h, int precision, const double* v_host, double* y_host);
// adjoint and checkpoints (lpm_adjoint.cu); vectors are device pointers
int adjoint_buffers(lpm_handle* h);
int adjoint_apply(lpm_handle* h, const double* v, double* y);
int adjoint_step(lpm_handle* h, const double* a, const double* c, double tol, long long maxit, int accumulate,
                 double* gKn, double* gTv, long long* iters, double* relres);
int tangent_begin(lpm_handle* h, int ndir, const double* dparams_host, double tol);
int tangent_step(lpm_handle* h);
int tangent_bond_constants(lpm_handle* h, int dir, const double* dkn_host, const double* dtv_host);
int tangent_bond_scrit(lpm_handle* h, int dir, const double* dsc_host);
int tangent_soft_damage(lpm_handle* h);
int tangent_hcf_state(lpm_handle* h);
int tangent_hcf_bdamage(lpm_handle* h);
int checkpoint_save(lpm_handle* h, int* id);
int checkpoint_restore(lpm_handle* h, int id);
int checkpoint_drop(lpm_handle* h, int id);

// helpers (lpm_capi.cu)
int cuda_fail(lpm_handle* h, cudaError_t e, const char* what);
void set_global_error(const std::string& msg);  // text of lpm_last_error(NULL)
void* dev_alloc(lpm_handle* h, size_t bytes);
void* zeros_dev(lpm_handle* h, size_t bytes);  // dev_alloc + zero fill
inline int grid_for(long long work, int threads, int cap = 1 << 20) {
  long long g = (work + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

}  // namespace lpm

#define LPM_CUDA(h, call)                                  \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return lpm::cuda_fail(h, e_, #call); \
  } while (0)

#define LPM_LAUNCHED(h, what)                             \
  do {                                                    \
    cudaError_t e_ = cudaGetLastError();                  \
    if (e_ != cudaSuccess) return lpm::cuda_fail(h, e_, what); \
    (h)->stats.kernel_launches++;                         \
  } while (0)
