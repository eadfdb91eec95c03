// Sparsity pattern (Particle::conns) and the analytical tangent.
//
// Pattern (assembly.h:236-266): conns(i) = sorted unique {k, m : k a layer-l
// bond partner of i, m a layer-l bond partner of k}.  Built on the device in
// three passes (count candidates, fill + sort + unique per particle,
// compact); integer work, identical to the reference's lists.
//
// Tangent (stiffness.h:67-101, 228-263; derivative.h): block K_ij for every
// j in conns(i).  The stored operator is A = K^T (see lpm_internal.cuh); a
// warp owns one row j of A and its lanes compute the blocks K_ij, i in
// conns(j), each by walking the bond lists exactly as derivative.h does, so
// the terms of a block are added in the reference's order.
#include <algorithm>
#include <numeric>

#include "lpm_device.cuh"

namespace lpm {
namespace {

__device__ __forceinline__ void layer_range(const int64_t* bptr, const int64_t* lptr, int i, int l, int64_t& b,
                                            int64_t& e) {
  b = l == 0 ? bptr[i] : lptr[i];
  e = l == 0 ? lptr[i] : bptr[i + 1];
}

__global__ void k_count_candidates(int n, const int64_t* __restrict__ bptr, const int64_t* __restrict__ lptr,
                                   const int* __restrict__ bp2, const int* __restrict__ blayer,
                                   int64_t* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t c = 0;
  for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
    int64_t kb, ke;
    layer_range(bptr, lptr, bp2[b], blayer[b], kb, ke);
    c += 1 + (ke - kb);
  }
  cnt[i] = c;
}

// Candidates of particle i in the reference's push order, then an insertion
// sort and unique in place.  Writes the unique count.
__global__ void k_fill_candidates(int n, const int64_t* __restrict__ bptr, const int64_t* __restrict__ lptr,
                                  const int* __restrict__ bp2, const int64_t* __restrict__ cand_ptr,
                                  int* __restrict__ cand, int64_t* __restrict__ ucnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int* c = cand + cand_ptr[i];
  int64_t m = 0;
  for (int l = 0; l < NL; ++l) {
    int64_t lb, le;
    layer_range(bptr, lptr, i, l, lb, le);
    for (int64_t b = lb; b < le; ++b) {
      const int k = bp2[b];
      c[m++] = k;
      int64_t kb, ke;
      layer_range(bptr, lptr, k, l, kb, ke);
      for (int64_t b2 = kb; b2 < ke; ++b2) c[m++] = bp2[b2];
    }
  }
  for (int64_t a = 1; a < m; ++a) {
    const int v = c[a];
    int64_t t = a - 1;
    while (t >= 0 && c[t] > v) {
      c[t + 1] = c[t];
      --t;
    }
    c[t + 1] = v;
  }
  int64_t u = 0;
  for (int64_t a = 0; a < m; ++a)
    if (u == 0 || c[a] != c[u - 1]) c[u++] = c[a];
  ucnt[i] = u;
}

__global__ void k_compact_pattern(int n, const int64_t* __restrict__ cand_ptr, const int* __restrict__ cand,
                                  const int64_t* __restrict__ cptr, int* __restrict__ cidx, int* __restrict__ diag_slot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* c = cand + cand_ptr[i];
  const int64_t q0 = cptr[i], len = cptr[i + 1] - q0;
  int ds = -1;
  for (int64_t a = 0; a < len; ++a) {
    cidx[q0 + a] = c[a];
    if (c[a] == i) ds = (int)(q0 + a);
  }
  diag_slot[i] = ds;
}

struct AsmView {
  const int64_t *bptr, *lptr, *cptr;
  const int *bp2, *cidx;
  const double *cs, *cs_sum, *Kn, *Tv, *bdamage;
  double* A;
  int64_t nblk;
  int n, sym;
};

// derivative.h:8-45
template <int DIM>
__device__ __forceinline__ void diag_block(const AsmView& v, int i, double (&K)[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) K[r][c] = 0.0;
  for (int l = 0; l < NL; ++l) {
    const double* S = v.cs_sum + (NL * i + l) * 3;
    const double S0 = S[0], S1 = S[1], S2 = S[2];
    const double Sv[3] = {S0, S1, S2};
    int64_t lb, le;
    layer_range(v.bptr, v.lptr, i, l, lb, le);
    for (int64_t b = lb; b < le; ++b) {
      const double nv[3] = {v.cs[3 * b], v.cs[3 * b + 1], v.cs[3 * b + 2]};
      const double w = 1 - v.bdamage[b], kn = v.Kn[b], tv = v.Tv[b], kt = kn + tv;
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int c = r; c < DIM; ++c) K[r][c] += w * ((kn * nv[c] + tv * Sv[c]) * nv[r] + kt * nv[r] * nv[c]);
    }
  }
  K[1][0] = v.sym ? K[0][1] : K[1][0];
  K[2][0] = K[0][2];
  K[2][1] = K[1][2];
}

// derivative.h:47-142 (layer 0) and 144-239 (layer 1), summed as
// stiffness.h:72-98 does.
template <int DIM>
__device__ __forceinline__ void off_block(const AsmView& v, int i, int j, double (&K)[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) K[r][c] = 0.0;
  for (int l = 0; l < NL; ++l) {
    double B[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) B[r][c] = 0.0;
    int64_t lb, le;
    layer_range(v.bptr, v.lptr, i, l, lb, le);
    int64_t b1 = -1;
    for (int64_t b = lb; b < le; ++b)
      if (v.bp2[b] == j) {
        b1 = b;
        break;
      }
    if (b1 >= 0) {
      const double n1[3] = {v.cs[3 * b1], v.cs[3 * b1 + 1], v.cs[3 * b1 + 2]};
      const double w1t = (1 - v.bdamage[b1]) * v.Tv[b1];
      for (int64_t b2 = lb; b2 < le; ++b2) {
        const int k = v.bp2[b2];
        const double n2[3] = {v.cs[3 * b2], v.cs[3 * b2 + 1], v.cs[3 * b2 + 2]};
        const double w2 = 1 - v.bdamage[b2];
        if (k == j) {
          const double* S = v.cs_sum + (NL * j + l) * 3;
          const double Sj[3] = {S[0], S[1], S[2]};
          const double kn = v.Kn[b2], tv = v.Tv[b2], kt = kn + tv;
#pragma unroll
          for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int c = 0; c < DIM; ++c) B[r][c] += w2 * ((-kn * n2[c] + tv * Sj[c]) * n2[r] - kt * n2[r] * n2[c]);
        } else {
          const double w2t = w2 * v.Tv[b2];
          const double hh = 0.5 * (w1t + w2t);
#pragma unroll
          for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int c = 0; c < DIM; ++c) B[r][c] -= hh * n2[r] * n1[c];
          int64_t kb, ke;
          layer_range(v.bptr, v.lptr, k, l, kb, ke);
          for (int64_t b3 = kb; b3 < ke; ++b3) {
            if (v.bp2[b3] != j) continue;
            const double n3[3] = {v.cs[3 * b3], v.cs[3 * b3 + 1], v.cs[3 * b3 + 2]};
            const double h3 = 0.5 * ((1 - v.bdamage[b3]) * v.Tv[b3] + w2t);
#pragma unroll
            for (int r = 0; r < DIM; ++r)
#pragma unroll
              for (int c = 0; c < DIM; ++c) B[r][c] -= h3 * n2[r] * n3[c];
          }
        }
      }
    } else {
      for (int64_t ba = lb; ba < le; ++ba) {
        const int k = v.bp2[ba];
        int64_t kb, ke;
        layer_range(v.bptr, v.lptr, k, l, kb, ke);
        double n1[3];
        bool loaded = false;
        double w1t = 0.0;
        for (int64_t bb = kb; bb < ke; ++bb) {
          if (v.bp2[bb] != j) continue;
          if (!loaded) {
            n1[0] = v.cs[3 * ba];
            n1[1] = v.cs[3 * ba + 1];
            n1[2] = v.cs[3 * ba + 2];
            w1t = (1 - v.bdamage[ba]) * v.Tv[ba];
            loaded = true;
          }
          const double n2[3] = {v.cs[3 * bb], v.cs[3 * bb + 1], v.cs[3 * bb + 2]};
          const double hh = 0.5 * ((1 - v.bdamage[bb]) * v.Tv[bb] + w1t);
#pragma unroll
          for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int c = 0; c < DIM; ++c) B[r][c] -= hh * n1[r] * n2[c];
        }
      }
    }
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int c = 0; c < DIM; ++c) K[r][c] += B[r][c];
  }
}

// One warp per row j of A = K^T; lane t takes the row's blocks t, t+32, ...
template <int DIM>
__global__ void __launch_bounds__(256) k_assemble(AsmView v) {
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long j = w0; j < v.n; j += nw) {
    const int64_t q0 = v.cptr[j], q1 = v.cptr[j + 1];
    for (int64_t q = q0 + lane; q < q1; q += 32) {
      const int i = v.cidx[q];
      double K[3][3];
      if (i == (int)j)
        diag_block<DIM>(v, i, K);
      else
        off_block<DIM>(v, i, (int)j, K);
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int s = 0; s < DIM; ++s) v.A[(r * DIM + s) * v.nblk + q] = K[s][r];
    }
  }
}

// |diag(K)|_2 (stiffness.h:269-270) and the DOFs to eliminate
// (stiffness.h:277: disp_constraint or damage_visual == 1).
template <int DIM>
__global__ void k_diag_norm_fixed(int n, const int* __restrict__ diag_slot, const double* __restrict__ A,
                                  int64_t nblk, const int* __restrict__ mask, const double* __restrict__ dvis,
                                  unsigned char* __restrict__ fixed, double* partials, unsigned int* ticket,
                                  double* norms) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = diag_slot[i];
    const bool dead = fabs(dvis[i] - 1.0) < EPS;
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
      if (s >= 0) {
        const double a = A[(r * DIM + r) * nblk + s];
        v[0] += a * a;
      }
      fixed[DIM * i + r] = (mask[3 * i + r] == 1 || dead) ? 1 : 0;
    }
  }
  double tot[1];
  if (grid_sum<1>(v, partials, ticket, tot) && threadIdx.x == 0) norms[2] = sqrt(tot[0]);
}

// Zero the rows and columns of fixed DOFs, norm on their diagonal
// (stiffness.h:273-291).  Entry (r, s) of block (j, i) of A is K(i s, j r).
template <int DIM>
__global__ void __launch_bounds__(256) k_apply_bc(int n, const int64_t* __restrict__ cptr, const int* __restrict__ cidx,
                                                  const unsigned char* __restrict__ fixed, const double* norms,
                                                  double* __restrict__ A, int64_t nblk) {
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const double nd = norms[2];
  for (long long j = w0; j < n; j += nw) {
    unsigned char fj[DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r) fj[r] = fixed[DIM * j + r];
    for (int64_t q = cptr[j] + lane; q < cptr[j + 1]; q += 32) {
      const int i = cidx[q];
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int s = 0; s < DIM; ++s)
          if (fj[r] || fixed[DIM * i + s]) A[(r * DIM + s) * nblk + q] = (i == (int)j && r == s) ? nd : 0.0;
    }
  }
}

__global__ void k_to_fp32(int64_t m, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

}  // namespace

int build_pattern(lpm_handle* h) {
  Dev& d = h->d;
  const int n = h->n, T = 128;
  int64_t* cnt = (int64_t*)dev_alloc(h, sizeof(int64_t) * (size_t)n);
  int64_t* cand_ptr = (int64_t*)dev_alloc(h, sizeof(int64_t) * ((size_t)n + 1));
  if (!cnt || !cand_ptr) return LPM_ERR_NOMEM;
  k_count_candidates<<<grid_for(n, T), T, 0, h->stream>>>(n, d.bptr, d.lptr, d.bp2, d.blayer, cnt);
  LPM_LAUNCHED(h, "k_count_candidates");
  std::vector<int64_t> hc((size_t)n), hp((size_t)n + 1, 0);
  LPM_CUDA(h, cudaMemcpyAsync(hc.data(), cnt, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int i = 0; i < n; ++i) hp[(size_t)i + 1] = hp[(size_t)i] + hc[(size_t)i];
  LPM_CUDA(h, cudaMemcpyAsync(cand_ptr, hp.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, h->stream));
  int* cand = nullptr;
  LPM_CUDA(h, cudaMallocAsync((void**)&cand, sizeof(int) * (size_t)std::max<int64_t>(hp[(size_t)n], 1), h->stream));
  k_fill_candidates<<<grid_for(n, T), T, 0, h->stream>>>(n, d.bptr, d.lptr, d.bp2, cand_ptr, cand, cnt);
  LPM_LAUNCHED(h, "k_fill_candidates");
  LPM_CUDA(h, cudaMemcpyAsync(hc.data(), cnt, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<int64_t> cp((size_t)n + 1, 0);
  for (int i = 0; i < n; ++i) cp[(size_t)i + 1] = cp[(size_t)i] + hc[(size_t)i];
  h->nblk = cp[(size_t)n];
  if (h->nblk >= (int64_t)1 << 31) {
    cudaFreeAsync(cand, h->stream);
    h->err = "pattern has 2^31 or more blocks";
    return LPM_ERR_ARG;
  }
  d.cptr = (int64_t*)dev_alloc(h, sizeof(int64_t) * ((size_t)n + 1));
  d.cidx = (int*)dev_alloc(h, sizeof(int) * (size_t)std::max<int64_t>(h->nblk, 1));
  d.diag_slot = (int*)dev_alloc(h, sizeof(int) * (size_t)n);
  if (!d.cptr || !d.cidx || !d.diag_slot) {
    cudaFreeAsync(cand, h->stream);
    return LPM_ERR_NOMEM;
  }
  LPM_CUDA(h, cudaMemcpyAsync(d.cptr, cp.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, h->stream));
  k_compact_pattern<<<grid_for(n, T), T, 0, h->stream>>>(n, cand_ptr, cand, d.cptr, d.cidx, d.diag_slot);
  LPM_LAUNCHED(h, "k_compact_pattern");
  LPM_CUDA(h, cudaFreeAsync(cand, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int launch_assemble(lpm_handle* h, int tangent, int bc) {
  Dev& d = h->d;
  const int dim = h->dim;
  const size_t vals = (size_t)h->nblk * dim * dim;
  if (!d.A64) {
    d.A64 = (double*)dev_alloc(h, sizeof(double) * std::max<size_t>(vals, 1));
    if (!d.A64) return LPM_ERR_NOMEM;
  }
  AsmView v{d.bptr, d.lptr, d.cptr, d.bp2, d.cidx, d.cs, d.cs_sum, d.Kn, d.Tv, d.bdamage, d.A64, h->nblk, h->n,
            tangent == LPM_TANGENT_SYMMETRIC ? 1 : 0};
  const int T = 256;
  const int G = grid_for((long long)h->n * 32, T, 152 * 64);
  if (dim == 3)
    k_assemble<3><<<G, T, 0, h->stream>>>(v);
  else
    k_assemble<2><<<G, T, 0, h->stream>>>(v);
  LPM_LAUNCHED(h, "k_assemble");
  if (bc == LPM_BC_ELIMINATE) {
    const int GR = grid_for(h->n, kRedThreads, kMaxRedBlocks);
    if (dim == 3)
      k_diag_norm_fixed<3><<<GR, kRedThreads, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nblk, d.mask, d.dvis,
                                                              d.fixed, d.red.partials, d.red.ticket + 1, d.norms);
    else
      k_diag_norm_fixed<2><<<GR, kRedThreads, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nblk, d.mask, d.dvis,
                                                              d.fixed, d.red.partials, d.red.ticket + 1, d.norms);
    LPM_LAUNCHED(h, "k_diag_norm_fixed");
    if (dim == 3)
      k_apply_bc<3><<<G, T, 0, h->stream>>>(h->n, d.cptr, d.cidx, d.fixed, d.norms, d.A64, h->nblk);
    else
      k_apply_bc<2><<<G, T, 0, h->stream>>>(h->n, d.cptr, d.cidx, d.fixed, d.norms, d.A64, h->nblk);
    LPM_LAUNCHED(h, "k_apply_bc");
  }
  h->have_K = true;
  h->a32_valid = false;
  h->tangent = tangent;
  return LPM_OK;
}

// FP32 copy of the operator for the mixed-precision solve.
int convert_A32(lpm_handle* h) {
  Dev& d = h->d;
  const size_t vals = (size_t)h->nblk * h->dim * h->dim;
  if (!d.A32) {
    d.A32 = (float*)dev_alloc(h, sizeof(float) * std::max<size_t>(vals, 1));
    if (!d.A32) return LPM_ERR_NOMEM;
  }
  k_to_fp32<<<grid_for((long long)vals, 256, 152 * 32), 256, 0, h->stream>>>((int64_t)vals, d.A64, d.A32);
  LPM_LAUNCHED(h, "k_to_fp32");
  h->a32_valid = true;
  return LPM_OK;
}

}  // namespace lpm
