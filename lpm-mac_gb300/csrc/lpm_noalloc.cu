// lpm_cg_solve_noalloc: the Jacobi-CG solve for callers that must not
// allocate device memory.
//
// Who needs it: code that runs inside a region where allocation is not
// allowed, e.g. a real-time loop that has reserved all its memory up front,
// or a host framework whose own allocator owns the device and forbids
// cudaMalloc from libraries.  Such a caller allocates its inputs and outputs
// itself and passes them in; the solver's work vectors and reduction scratch
// live in one file-scope device array of fixed size (LPM_NOALLOC_MAX_DOF),
// so no call allocates or frees.  The call waits for its stream at the end
// to read the iteration count back.
//
// The array belongs to the library: it is created when the library's device
// code is loaded on a GPU (about 33.6 MB), whether or not this entry point
// is ever called, and stays until the process exits; all calls on a device
// share it.  Two calls whose work overlaps on the same GPU (different
// streams, or different host threads) therefore race; serialise them.  Each
// call clears the parts that must start at zero (the reduction tickets)
// before use.
//
// Device address: in host code the array's name is a host-side stand-in, not
// a device address, so the first call on each device looks the address up
// with cudaGetSymbolAddress (with that device current) and caches it.  Make
// that first call before any stream capture begins.  The cached address
// belongs to the device's context: after a device reset (cudaDeviceReset) it
// is stale, so do not use the library across one.
//
// The product walks the caller's block CSR one row per thread (plain loads,
// no sliced layout), so an iteration costs more than one of lpm_solve.
#include <cfloat>
#include <cmath>
#include <mutex>

#include "lpm_device.cuh"

namespace lpm {
namespace {

// scratch layout (doubles): r, p, q, invd (LPM_NOALLOC_MAX_DOF each), then
// reduction partials (2 * kMaxRedBlocks), then the CG scalars and the tickets
constexpr long long kMaxDof = LPM_NOALLOC_MAX_DOF;
constexpr long long kPartials = 2LL * kMaxRedBlocks;
constexpr long long kScalarDoubles = (sizeof(CgScalars) + sizeof(double) - 1) / sizeof(double);
constexpr long long kTicketDoubles = 4;  // 8 unsigned counters
constexpr long long kScratchDoubles = 4 * kMaxDof + kPartials + kScalarDoubles + kTicketDoubles;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// One thread per row of the block-CSR operator: y_j = sum_k A_jk p_k, and the
// p.q partial for alpha.
template <int DIM>
__global__ void __launch_bounds__(256) k_bsr_spmv(int n, const int64_t* __restrict__ ptr, const int* __restrict__ col,
                                                  const double* __restrict__ vals, const double* __restrict__ p,
                                                  double* __restrict__ q, CgScalars* cg, double* partials,
                                                  unsigned int* ticket) {
  if (cg->done) return;
  double acc = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
    double y[DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r) y[r] = 0.0;
    for (int64_t k = ptr[row]; k < ptr[row + 1]; ++k) {
      const int c = col[k];
      const double* a = vals + k * DIM * DIM;
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int t = 0; t < DIM; ++t) y[r] = fma(a[r * DIM + t], p[(int64_t)c * DIM + t], y[r]);
    }
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
      q[(int64_t)row * DIM + r] = y[r];
      acc += p[(int64_t)row * DIM + r] * y[r];
    }
  }
  double w[1] = {acc}, tot[1];
  if (grid_sum<1>(w, partials, ticket, tot) && threadIdx.x == 0) cg->alpha = cg->abs_new / tot[0];
}

// Jacobi preconditioner: 1 / diagonal entry, 1 where it is zero or missing.
template <int DIM>
__global__ void k_bsr_invd(int n, const int64_t* __restrict__ ptr, const int* __restrict__ col,
                           const double* __restrict__ vals, double* __restrict__ invd) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  double dg[DIM];
#pragma unroll
  for (int r = 0; r < DIM; ++r) dg[r] = 0.0;
  for (int64_t k = ptr[row]; k < ptr[row + 1]; ++k)
    if (col[k] == row) {
#pragma unroll
      for (int r = 0; r < DIM; ++r) dg[r] = vals[k * DIM * DIM + r * DIM + r];
      break;
    }
#pragma unroll
  for (int r = 0; r < DIM; ++r) invd[(int64_t)row * DIM + r] = dg[r] != 0.0 ? 1.0 / dg[r] : 1.0;
}

// The CG steps shared with the handle solver, restated for the scratch
// vectors (same recurrence and stopping rule as lpm_solve's FP64 path).
__global__ void k_nc_init(int64_t m, const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r,
                          double* __restrict__ p, const double* __restrict__ invd, CgScalars* cg, double tol,
                          long long maxit, double* partials, unsigned int* ticket) {
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const double bi = b[i], pi = invd[i] * bi;
    x[i] = 0.0;
    r[i] = bi;
    p[i] = pi;
    v[0] += bi * bi;
    v[1] += bi * pi;
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rhs_norm2 = tot[0];
    cg->rr = tot[0];
    cg->threshold = fmax(tol * tol * tot[0], DBL_MIN);
    cg->abs_new = tot[1];
    cg->alpha = cg->beta = 0.0;
    cg->it = 0;
    cg->maxit = maxit;
    cg->ru = 0;
    cg->rmax = 0.0;
    cg->ru_count = 0;
    if (!isfinite(tot[0]) || !isfinite(tot[1]))
      cg->done = 3;
    else if (tot[0] == 0.0 || tot[0] < cg->threshold)
      cg->done = 1;
    else if (maxit <= 0)
      cg->done = 2;
    else
      cg->done = 0;
  }
}

__global__ void k_nc_update(int64_t m, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                            const double* __restrict__ q, const double* __restrict__ invd, CgScalars* cg,
                            double* partials, unsigned int* ticket) {
  if (cg->done) return;
  const double alpha = cg->alpha;
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = r[i] - alpha * q[i];
    x[i] = x[i] + alpha * p[i];
    r[i] = ri;
    v[0] += ri * ri;
    v[1] += ri * (invd[i] * ri);
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rr = tot[0];
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      cg->done = 3;
    } else if (tot[0] < cg->threshold) {
      cg->done = 1;
    } else {
      const double old = cg->abs_new;
      cg->abs_new = tot[1];
      cg->beta = tot[1] / old;
      cg->it += 1;
      if (cg->it >= cg->maxit) cg->done = 2;
    }
  }
}

__global__ void k_nc_pupdate(int64_t m, const double* __restrict__ r, const double* __restrict__ invd,
                             double* __restrict__ p, const CgScalars* cg) {
  if (cg->done) return;
  const double beta = cg->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = invd[i] * r[i] + beta * p[i];
}

std::mutex g_scratch_mu;
double* g_scratch_addr[64] = {nullptr};

// Errors are reported through the return code; the text goes to the text
// lpm_last_error(NULL) returns.
int nc_fail(const char* what, cudaError_t e, int code) {
  set_global_error(std::string(what) + (e == cudaSuccess ? "" : std::string(": ") + cudaGetErrorString(e)));
  return code;
}

}  // namespace
}  // namespace lpm

using namespace lpm;

extern "C" int lpm_cg_solve_noalloc(int dim, int n, const int64_t* ptr, const int* col, const double* vals,
                                    const double* b, double* x, double tol, int64_t maxit, void* stream,
                                    int64_t* iters, double* relres) {
  if (dim != 2 && dim != 3) return nc_fail("dim must be 2 or 3", cudaSuccess, LPM_ERR_ARG);
  if (n <= 0 || !ptr || !col || !vals || !b || !x) return nc_fail("bad size or NULL device pointer", cudaSuccess, LPM_ERR_ARG);
  const long long ndof = (long long)n * dim;
  if (ndof > kMaxDof) return nc_fail("n * dim exceeds LPM_NOALLOC_MAX_DOF (1048576): use lpm_solve", cudaSuccess, LPM_ERR_ARG);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nc_fail("cudaGetDevice", e, LPM_ERR_CUDA);
  if (dev < 0 || dev >= 64) return nc_fail("device ordinal above 63", cudaSuccess, LPM_ERR_ARG);
  double* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      // once per device, with that device current (the caller's current device)
      e = cudaGetSymbolAddress((void**)&g_scratch_addr[dev], g_noalloc_scratch);
      if (e != cudaSuccess) {
        g_scratch_addr[dev] = nullptr;
        return nc_fail("cudaGetSymbolAddress", e, LPM_ERR_CUDA);
      }
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* r = base;
  double* p = base + kMaxDof;
  double* q = base + 2 * kMaxDof;
  double* invd = base + 3 * kMaxDof;
  double* partials = base + 4 * kMaxDof;
  CgScalars* cg = (CgScalars*)(partials + kPartials);
  unsigned int* tickets = (unsigned int*)(base + 4 * kMaxDof + kPartials + kScalarDoubles);
  if (maxit < 0) maxit = 2 * ndof;
  e = cudaMemsetAsync(tickets, 0, kTicketDoubles * sizeof(double), s);
  if (e != cudaSuccess) return nc_fail("cudaMemsetAsync", e, LPM_ERR_CUDA);
  const int GV = grid_for(ndof, 256, kMaxRedBlocks), GR = grid_for(n, 256, kMaxRedBlocks);
  if (dim == 3)
    k_bsr_invd<3><<<grid_for(n, 256), 256, 0, s>>>(n, ptr, col, vals, invd);
  else
    k_bsr_invd<2><<<grid_for(n, 256), 256, 0, s>>>(n, ptr, col, vals, invd);
  k_nc_init<<<GV, 256, 0, s>>>(ndof, b, x, r, p, invd, cg, tol, maxit, partials, tickets + 0);
  e = cudaGetLastError();
  if (e != cudaSuccess) return nc_fail("kernel launch", e, LPM_ERR_CUDA);
  CgScalars hc;
  long long batch = 8;
  for (;;) {
    for (long long k = 0; k < batch; ++k) {
      if (dim == 3)
        k_bsr_spmv<3><<<GR, 256, 0, s>>>(n, ptr, col, vals, p, q, cg, partials, tickets + 1);
      else
        k_bsr_spmv<2><<<GR, 256, 0, s>>>(n, ptr, col, vals, p, q, cg, partials, tickets + 1);
      k_nc_update<<<GV, 256, 0, s>>>(ndof, x, r, p, q, invd, cg, partials, tickets + 2);
      k_nc_pupdate<<<GV, 256, 0, s>>>(ndof, r, invd, p, cg);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return nc_fail("kernel launch", e, LPM_ERR_CUDA);
    e = cudaMemcpyAsync(&hc, cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return nc_fail("reading the CG state", e, LPM_ERR_CUDA);
    if (hc.done) break;
    if (batch < 64) batch *= 2;
  }
  const double err = hc.rhs_norm2 > 0 ? std::sqrt(hc.rr / hc.rhs_norm2) : 0.0;
  if (iters) *iters = hc.it;
  if (relres) *relres = err;
  if (hc.done == 3) return nc_fail("non-finite value in the CG iteration", cudaSuccess, LPM_ERR_NONFINITE);
  return err <= tol ? LPM_OK : LPM_NOT_CONVERGED;
}
