// Jacobi-preconditioned conjugate gradients on A = K^T.
//
// The iteration is the one Eigen's ConjugateGradient runs for
// Solver::LPM_CG (solver.h:192-217): zero start, p = M^-1 r,
//   q = A p; alpha = (r.z)/(p.q); x += alpha p; r -= alpha q;
//   stop if |r|^2 < max(tol^2 |b|^2, DBL_MIN); z = M^-1 r; beta = (r.z)_new/(r.z)_old;
//   p = z + beta p; it++   (at most maxit iterations)
// with M the diagonal of the matrix (1 where it is zero or missing).
//
// Each iteration is three kernels on the handle's stream:
//   k_cg_spmv    q = A p and p.q; the last block sets alpha
//   k_cg_update  x, r, |r|^2, r.z; the last block tests convergence, sets beta
//   k_cg_pupdate p = z + beta p
// Kernels return at once when the device flag `done` is set, so the host
// enqueues iterations in batches and reads the flag once per batch.
//
// Mixed precision: FP32 CG (same kernels, float storage, FP64 dot
// accumulation) on an FP32 copy of A, inside an FP64 refinement loop
// x += CG32(b - A64 x) that stops on the FP64 residual.
#include <cfloat>
#include <cmath>

#include "lpm_device.cuh"

namespace lpm {
namespace {

template <typename T, int DIM>
__device__ __forceinline__ void row_product(const int64_t* __restrict__ cptr, const int* __restrict__ cidx,
                                            const T* __restrict__ A, int64_t nblk, const T* __restrict__ p,
                                            long long row, int lane, T (&y)[DIM]) {
#pragma unroll
  for (int r = 0; r < DIM; ++r) y[r] = T(0);
  const int64_t q1 = cptr[row + 1];
  for (int64_t s = cptr[row] + lane; s < q1; s += 32) {
    const int c = __ldg(&cidx[s]);
    T pc[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) pc[k] = __ldg(&p[(int64_t)c * DIM + k]);
    T a[DIM * DIM];
#pragma unroll
    for (int e = 0; e < DIM * DIM; ++e) a[e] = __ldcs(&A[e * nblk + s]);
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int k = 0; k < DIM; ++k) y[r] = fma(a[r * DIM + k], pc[k], y[r]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int r = 0; r < DIM; ++r) y[r] += __shfl_xor_sync(0xffffffffu, y[r], o);
}

template <typename T, int DIM>
__device__ __forceinline__ T pick(const T (&y)[DIM], int lane) {
  T v = y[0];
#pragma unroll
  for (int r = 1; r < DIM; ++r) v = lane == r ? y[r] : v;
  return v;
}

template <typename T, int DIM>
__global__ void __launch_bounds__(256) k_cg_spmv(const int64_t* __restrict__ cptr, const int* __restrict__ cidx,
                                                 const T* __restrict__ A, int64_t nblk, int n,
                                                 const T* __restrict__ p, T* __restrict__ q, CgScalars* cg,
                                                 double* partials, unsigned int* ticket) {
  if (cg->done) return;
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (long long row = w0; row < n; row += nw) {
    T y[DIM];
    row_product<T, DIM>(cptr, cidx, A, nblk, p, row, lane, y);
    if (lane < DIM) {
      const T yv = pick<T, DIM>(y, lane);
      q[row * DIM + lane] = yv;
      acc += (double)p[row * DIM + lane] * (double)yv;
    }
  }
  double v[1] = {acc}, tot[1];
  if (grid_sum<1>(v, partials, ticket, tot) && threadIdx.x == 0) cg->alpha = cg->abs_new / tot[0];
}

template <typename T>
__global__ void __launch_bounds__(256) k_cg_update(int64_t ndof, T* __restrict__ x, T* __restrict__ r,
                                                   const T* __restrict__ p, const T* __restrict__ q,
                                                   const T* __restrict__ invd, CgScalars* cg, double* partials,
                                                   unsigned int* ticket) {
  if (cg->done) return;
  const T alpha = (T)cg->alpha;
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = r[i] - alpha * q[i];
    x[i] = x[i] + alpha * p[i];
    r[i] = ri;
    const T zi = invd[i] * ri;
    v[0] += (double)ri * (double)ri;
    v[1] += (double)ri * (double)zi;
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

template <typename T>
__global__ void __launch_bounds__(256) k_cg_pupdate(int64_t ndof, const T* __restrict__ r, const T* __restrict__ invd,
                                                    T* __restrict__ p, const CgScalars* cg) {
  if (cg->done) return;
  const T beta = (T)cg->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = invd[i] * r[i] + beta * p[i];
}

template <typename T>
__global__ void k_cg_init(int64_t ndof, const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                          T* __restrict__ p, const T* __restrict__ invd, CgScalars* cg, double tol, long long maxit,
                          double* partials, unsigned int* ticket) {
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const T bi = b[i];
    const T pi = invd[i] * bi;
    x[i] = T(0);
    r[i] = bi;
    p[i] = pi;
    v[0] += (double)bi * (double)bi;
    v[1] += (double)bi * (double)pi;
  }
  double tot[2];
  if (grid_sum<2>(v, partials, ticket, tot) && threadIdx.x == 0) {
    cg->rhs_norm2 = tot[0];
    cg->rr = tot[0];
    cg->threshold = fmax(tol * tol * tot[0], DBL_MIN);
    cg->abs_new = tot[1];
    cg->alpha = 0.0;
    cg->beta = 0.0;
    cg->it = 0;
    cg->maxit = maxit;
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

// Jacobi preconditioner from the diagonal blocks of A (= diagonal of K).
template <int DIM>
__global__ void k_invd(int n, const int* __restrict__ diag_slot, const double* __restrict__ A, int64_t nblk,
                       double* __restrict__ invd64, float* __restrict__ invd32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = diag_slot[i];
#pragma unroll
  for (int r = 0; r < DIM; ++r) {
    const double a = s >= 0 ? A[(r * DIM + r) * nblk + s] : 0.0;
    const double v = a != 0.0 ? 1.0 / a : 1.0;
    invd64[DIM * i + r] = v;
    if (invd32) invd32[DIM * i + r] = (float)v;
  }
}

// r = b - A x (FP64) and |r|^2 into norms[3].
template <int DIM>
__global__ void __launch_bounds__(256) k_true_residual(const int64_t* __restrict__ cptr, const int* __restrict__ cidx,
                                                       const double* __restrict__ A, int64_t nblk, int n,
                                                       const double* __restrict__ x, const double* __restrict__ b,
                                                       double* __restrict__ r, double* partials,
                                                       unsigned int* ticket, double* norms) {
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (long long row = w0; row < n; row += nw) {
    double y[DIM];
    row_product<double, DIM>(cptr, cidx, A, nblk, x, row, lane, y);
    if (lane < DIM) {
      const double ri = b[row * DIM + lane] - pick<double, DIM>(y, lane);
      r[row * DIM + lane] = ri;
      acc += ri * ri;
    }
  }
  double v[1] = {acc}, tot[1];
  if (grid_sum<1>(v, partials, ticket, tot) && threadIdx.x == 0) norms[3] = tot[0];
}

// r32 = s * r64, with s = 1/|r64| (keeps the FP32 system near unit scale).
__global__ void k_to_scaled32(int64_t m, const double* __restrict__ a, const double* norms, float* __restrict__ b) {
  const double nr2 = norms[3];
  const double s = nr2 > 0.0 ? 1.0 / sqrt(nr2) : 1.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)(a[t] * s);
}

// x64 += |r64| * x32
__global__ void k_accumulate(int64_t m, const float* __restrict__ d, const double* norms, double* __restrict__ x) {
  const double nr2 = norms[3];
  const double s = nr2 > 0.0 ? sqrt(nr2) : 1.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
    x[t] += s * (double)d[t];
}

__global__ void k_sqnorm(int64_t m, const double* __restrict__ a, double* partials, unsigned int* ticket,
                         double* norms, int slot) {
  double v[1] = {0.0};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
    v[0] += a[t] * a[t];
  double tot[1];
  if (grid_sum<1>(v, partials, ticket, tot) && threadIdx.x == 0) norms[slot] = tot[0];
}

// Grid of the row kernels: whole warps per row, a fixed grid so that the
// reduction partials (and the result bits) do not depend on the row count.
int row_grid(lpm_handle* h) { return grid_for((long long)h->n * 32, 256, kMaxRedBlocks); }
int vec_grid(long long m) { return grid_for(m, 256, kMaxRedBlocks); }

cudaEvent_t next_event(lpm_handle* h) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_used++];
}

// Runs the CG iteration on the given operator/vectors.  Returns the device
// `done` code through h->h_cg.
template <typename T>
int run_cg(lpm_handle* h, const T* A, const T* b, T* x, T* r, T* p, T* q, const T* invd, double tol, long long maxit) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t ndof = (int64_t)h->n * dim;
  const int GV = vec_grid(ndof), GR = row_grid(h);
  k_cg_init<T><<<GV, 256, 0, h->stream>>>(ndof, b, x, r, p, invd, d.cg, tol, maxit, d.red.partials,
                                          d.red.ticket + 2);
  LPM_LAUNCHED(h, "k_cg_init");
  const bool timing = h->timing;
  const size_t ev0 = h->ev_used;
  long long batch = 8;
  for (;;) {
    for (long long k = 0; k < batch; ++k) {
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (timing) {
        e0 = next_event(h);
        e1 = next_event(h);
        if (e0) cudaEventRecord(e0, h->stream);
      }
      if (dim == 3)
        k_cg_spmv<T, 3><<<GR, 256, 0, h->stream>>>(d.cptr, d.cidx, A, h->nblk, h->n, p, q, d.cg, d.red.partials,
                                                   d.red.ticket + 3);
      else
        k_cg_spmv<T, 2><<<GR, 256, 0, h->stream>>>(d.cptr, d.cidx, A, h->nblk, h->n, p, q, d.cg, d.red.partials,
                                                   d.red.ticket + 3);
      LPM_LAUNCHED(h, "k_cg_spmv");
      if (timing && e1) cudaEventRecord(e1, h->stream);
      k_cg_update<T><<<GV, 256, 0, h->stream>>>(ndof, x, r, p, q, invd, d.cg, d.red.partials, d.red.ticket + 4);
      LPM_LAUNCHED(h, "k_cg_update");
      k_cg_pupdate<T><<<GV, 256, 0, h->stream>>>(ndof, r, invd, p, d.cg);
      LPM_LAUNCHED(h, "k_cg_pupdate");
    }
    LPM_CUDA(h, cudaMemcpyAsync(h->h_cg, d.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->h_cg->done) break;
    if (batch < 64) batch *= 2;
  }
  if (timing) {
    // sparse products that did work: one per completed iteration, plus the
    // one of the final iteration when it stopped on the tolerance
    long long real = h->h_cg->it + (h->h_cg->done == 1 && h->h_cg->rhs_norm2 > 0 && h->h_cg->maxit > 0 ? 1 : 0);
    double ms_sum = 0.0;
    long long used = 0;
    for (size_t k = ev0; k + 1 < h->ev_used && used < real; k += 2, ++used) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, h->ev_pool[k], h->ev_pool[k + 1]) == cudaSuccess) ms_sum += ms;
    }
    if (sizeof(T) == 8) {
      h->stats.spmv_launches += used;
      h->stats.spmv_ms += ms_sum;
    } else {
      h->stats.spmv32_launches += used;
      h->stats.spmv32_ms += ms_sum;
    }
    h->ev_used = ev0;
  }
  return LPM_OK;
}

int prepare_invd(lpm_handle* h, bool want32) {
  Dev& d = h->d;
  if (h->dim == 3)
    k_invd<3><<<grid_for(h->n, 256), 256, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nblk, d.invd64,
                                                          want32 ? d.invd32 : nullptr);
  else
    k_invd<2><<<grid_for(h->n, 256), 256, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nblk, d.invd64,
                                                          want32 ? d.invd32 : nullptr);
  LPM_LAUNCHED(h, "k_invd");
  return LPM_OK;
}

}  // namespace

int solve_fp64(lpm_handle* h, double tol, long long maxit, long long* iters, double* relres) {
  Dev& d = h->d;
  if (!d.A64 || !d.rhs || !d.disp || !d.r64 || !d.p64 || !d.q64 || !d.invd64 || !d.diag_slot) {
    h->err = "FP64 solve: work buffers missing";
    return LPM_ERR_STATE;
  }
  if (maxit < 0) maxit = 2LL * h->n * h->dim;  // Eigen's default: twice the number of columns
  int st = prepare_invd(h, false);
  if (st) return st;
  st = run_cg<double>(h, d.A64, d.rhs, d.disp, d.r64, d.p64, d.q64, d.invd64, tol, maxit);
  if (st) return st;
  const CgScalars& c = *h->h_cg;
  const double err = c.rhs_norm2 > 0 ? sqrt(c.rr / c.rhs_norm2) : 0.0;
  if (iters) *iters = c.it;
  if (relres) *relres = err;
  h->stats.cg_iters_total += c.it;
  if (c.done == 3) {
    h->err = "non-finite value in the CG iteration";
    return LPM_ERR_NONFINITE;
  }
  return err <= tol ? LPM_OK : LPM_NOT_CONVERGED;
}

// Inner FP32 tolerance of each refinement sweep: FP32 CG reliably reaches
// about this relative residual on the LPM tangent.
static const double kInnerTol = 1e-5;
static const int kMaxSweeps = 40;

int solve_mixed(lpm_handle* h, double tol, long long maxit, long long* iters, double* relres) {
  Dev& d = h->d;
  const int dim = h->dim;
  const int64_t ndof = (int64_t)h->n * dim;
  if (!d.b32) {  // FP32 work vectors, allocated on the first mixed solve
    float** vecs[6] = {&d.b32, &d.x32, &d.r32, &d.p32, &d.q32, &d.invd32};
    for (float** v : vecs) {
      *v = (float*)dev_alloc(h, sizeof(float) * (size_t)ndof);
      if (!*v) return LPM_ERR_NOMEM;
    }
  }
  if (!h->a32_valid) {
    const int st0 = convert_A32(h);
    if (st0) return st0;
  }
  if (!d.A32 || !d.b32 || !d.x32 || !d.r32 || !d.p32 || !d.q32 || !d.invd32 || !d.x64 || !d.r64 || !d.rhs) {
    h->err = "mixed solve: work buffers missing";
    return LPM_ERR_STATE;
  }
  const int GV = vec_grid(ndof), GR = row_grid(h);
  int st = prepare_invd(h, true);
  if (st) return st;
  // |b|^2 and r64 = b (x64 = 0)
  LPM_CUDA(h, cudaMemsetAsync(d.x64, 0, sizeof(double) * ndof, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.r64, d.rhs, sizeof(double) * ndof, cudaMemcpyDeviceToDevice, h->stream));
  k_sqnorm<<<GV, 256, 0, h->stream>>>(ndof, d.rhs, d.red.partials, d.red.ticket + 5, d.norms, 4);
  LPM_LAUNCHED(h, "k_sqnorm");
  k_sqnorm<<<GV, 256, 0, h->stream>>>(ndof, d.rhs, d.red.partials, d.red.ticket + 5, d.norms, 3);
  LPM_LAUNCHED(h, "k_sqnorm");
  LPM_CUDA(h, cudaMemcpyAsync(h->h_norms, d.norms, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  const double bb = h->h_norms[4];
  long long total = 0;
  double rel = bb > 0 ? 1.0 : 0.0;
  int sweeps = 0;
  if (!std::isfinite(bb)) {
    h->err = "non-finite right-hand side";
    return LPM_ERR_NONFINITE;
  }
  while (bb > 0 && rel > tol && sweeps < kMaxSweeps && (maxit < 0 || total < maxit)) {
    k_to_scaled32<<<GV, 256, 0, h->stream>>>(ndof, d.r64, d.norms, d.b32);
    LPM_LAUNCHED(h, "k_to_scaled32");
    const double want = std::max(kInnerTol, 0.5 * tol / rel);
    const long long cap = maxit < 0 ? 2 * ndof : std::max<long long>(1, maxit - total);
    st = run_cg<float>(h, d.A32, d.b32, d.x32, d.r32, d.p32, d.q32, d.invd32, want, cap);
    if (st) return st;
    total += h->h_cg->it;
    if (h->h_cg->done == 3) {
      h->err = "non-finite value in the FP32 CG iteration";
      return LPM_ERR_NONFINITE;
    }
    k_accumulate<<<GV, 256, 0, h->stream>>>(ndof, d.x32, d.norms, d.x64);
    LPM_LAUNCHED(h, "k_accumulate");
    if (dim == 3)
      k_true_residual<3><<<GR, 256, 0, h->stream>>>(d.cptr, d.cidx, d.A64, h->nblk, h->n, d.x64, d.rhs, d.r64,
                                                    d.red.partials, d.red.ticket + 6, d.norms);
    else
      k_true_residual<2><<<GR, 256, 0, h->stream>>>(d.cptr, d.cidx, d.A64, h->nblk, h->n, d.x64, d.rhs, d.r64,
                                                    d.red.partials, d.red.ticket + 6, d.norms);
    LPM_LAUNCHED(h, "k_true_residual");
    LPM_CUDA(h, cudaMemcpyAsync(h->h_norms, d.norms, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    const double rr = h->h_norms[3];
    if (!std::isfinite(rr)) {
      h->err = "non-finite residual in the refinement loop";
      return LPM_ERR_NONFINITE;
    }
    rel = sqrt(rr / bb);
    ++sweeps;
  }
  LPM_CUDA(h, cudaMemcpyAsync(d.disp, d.x64, sizeof(double) * ndof, cudaMemcpyDeviceToDevice, h->stream));
  h->stats.cg_iters_total += total;
  h->stats.refine_sweeps += sweeps;
  if (iters) *iters = total;
  if (relres) *relres = rel;
  return rel <= tol ? LPM_OK : LPM_NOT_CONVERGED;
}

}  // namespace lpm
