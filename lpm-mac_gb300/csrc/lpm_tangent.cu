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
                                  const int64_t* __restrict__ cptr, int* __restrict__ cidx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* c = cand + cand_ptr[i];
  const int64_t q0 = cptr[i], len = cptr[i + 1] - q0;
  for (int64_t a = 0; a < len; ++a) cidx[q0 + a] = c[a];
}

// Sliced layout: slot columns, row lengths and the diagonal slot.
__global__ void k_fill_sell(int n, const int64_t* __restrict__ cptr, const int* __restrict__ cidx,
                            const int64_t* __restrict__ sell_ptr, int* __restrict__ scol, int* __restrict__ rowlen,
                            int* __restrict__ diag_slot) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t q0 = cptr[j];
  const int len = (int)(cptr[j + 1] - q0);
  const SellRow row = sell_row(sell_ptr, j);
  int ds = -1;
  for (int k = 0; k < len; ++k) {
    const int c = cidx[q0 + k];
    scol[sell_slot(row, k)] = c;
    if (c == j) ds = (int)sell_slot(row, k);
  }
  // padding of the row's last group of four points at the row itself
  for (int k = len; k < sell_read_len(row, len); ++k) scol[sell_slot(row, k)] = j;
  rowlen[j] = len;
  diag_slot[j] = ds;
}

struct AsmView {
  const int64_t *bptr, *lptr, *sell_ptr;
  const int *scol, *rowlen, *sbond, *sp2, *opp;
  const double *cs, *cs_sum, *tsum, *msum, *Kn, *Tv, *bdamage;
  double* A;
  int64_t nslots;
  int n, nslice, sym;
};

// The analytical tangent (derivative.h) restated per block K_ij, i != j, as
// a sum over layers l of
//   own    (i->j a layer-l bond b):   w_b[(-Kn n_b[s] + Tv S_j[s]) n_b[r] - (Kn+Tv) n_b[r] n_b[s]]
//   other  (same b, derivative.h:91-99 summed over the other bonds of i):
//          -1/2 [w_b Tv_b (S_i - n_b) + (T_i - w_b Tv_b n_b)][r] n_b[s]
//   paths  (bonds i->k, k->j of layer l, derivative.h:101-115 and 122-139):
//          -1/2 (w_kj Tv_kj + w_ik Tv_ik) n_ik[r] n_kj[s]
// with S_i = sum of i's layer-l direction cosines, T_i = sum w Tv n over i's
// layer-l bonds.  The diagonal block (derivative.h:8-45) is
//   K_ii[r][s] = sum_l M_i[r][s] + T_i[r] S_i[s]   (r <= s),  M_i = sum w (2Kn+Tv) n n^T,
// then mirrored as derivative.h:37-42 does ([1][0] stays 0 in the as-written
// variant).  Common neighbours k of i and j come from a merge of the two
// particles' partner-sorted layer-l bond lists.
__device__ __forceinline__ void seg(const int64_t* bptr, const int64_t* lptr, int i, int l, int64_t& b, int64_t& e) {
  b = l == 0 ? bptr[i] : lptr[i];
  e = l == 0 ? lptr[i] : bptr[i + 1];
}

template <int DIM>
__device__ __forceinline__ void diag_block(const AsmView& v, int i, double (&K)[3][3]) {
  double k00 = 0, k01 = 0, k02 = 0, k11 = 0, k12 = 0, k22 = 0;
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    const double* M = v.msum + (NL * i + l) * 6;
    const double* T = v.tsum + (NL * i + l) * 3;
    const double* S = v.cs_sum + (NL * i + l) * 3;
    k00 += M[0] + T[0] * S[0];
    k01 += M[1] + T[0] * S[1];
    k02 += M[2] + T[0] * S[2];
    k11 += M[3] + T[1] * S[1];
    k12 += M[4] + T[1] * S[2];
    k22 += M[5] + T[2] * S[2];
  }
  K[0][0] = k00;
  K[0][1] = k01;
  K[0][2] = k02;
  K[1][0] = v.sym ? k01 : 0.0;
  K[1][1] = k11;
  K[1][2] = k12;
  K[2][0] = k02;
  K[2][1] = k12;
  K[2][2] = k22;
}

constexpr int kMatch = 8;  // common neighbours collected per merge chunk

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
    int64_t ia, ea, ib, eb;
    seg(v.bptr, v.lptr, i, l, ia, ea);
    seg(v.bptr, v.lptr, j, l, ib, eb);
    int direct = -1;
    // merge of the partner-sorted lists; the direct bond i->j shows up as
    // partner j in i's list.  The common neighbours are collected kMatch at
    // a time and their FP64 terms added after the (integer) merge, in merge
    // order: the lanes of a warp then run the FP64 work together instead of
    // each at its own point of the merge.
    while (ia < ea) {
      int m1[kMatch], m3[kMatch];
      int nm = 0;
      while (ia < ea && nm < kMatch) {
        const int pa = v.sp2[ia];
        if (pa == j) direct = v.sbond[ia];
        while (ib < eb && v.sp2[ib] < pa) ++ib;
        if (ib < eb && v.sp2[ib] == pa) {
          m1[nm] = v.sbond[ia];          // i -> k
          m3[nm] = v.opp[v.sbond[ib]];   // k -> j, opposite of j -> k
          ++nm;
        }
        ++ia;
      }
      for (int t = 0; t < nm; ++t) {
        const int b1 = m1[t], b3 = m3[t];
        const double h = 0.5 * ((1 - v.bdamage[b3]) * v.Tv[b3] + (1 - v.bdamage[b1]) * v.Tv[b1]);
        const double n1[3] = {v.cs[3 * (int64_t)b1], v.cs[3 * (int64_t)b1 + 1], v.cs[3 * (int64_t)b1 + 2]};
        const double n3[3] = {v.cs[3 * (int64_t)b3], v.cs[3 * (int64_t)b3 + 1], v.cs[3 * (int64_t)b3 + 2]};
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
          const double hr = h * n1[r];
#pragma unroll
          for (int c = 0; c < DIM; ++c) B[r][c] -= hr * n3[c];
        }
      }
    }
    if (direct >= 0) {
      const int64_t b = direct;
      const double n[3] = {v.cs[3 * b], v.cs[3 * b + 1], v.cs[3 * b + 2]};
      const double w = 1 - v.bdamage[b], kn = v.Kn[b], tv = v.Tv[b], kt = kn + tv, wt = w * tv;
      const double* Sj = v.cs_sum + (NL * j + l) * 3;
      const double* Si = v.cs_sum + (NL * i + l) * 3;
      const double* Ti = v.tsum + (NL * i + l) * 3;
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        const double o = 0.5 * (wt * (Si[r] - n[r]) + (Ti[r] - wt * n[r]));
#pragma unroll
        for (int c = 0; c < DIM; ++c)
          B[r][c] += w * ((-kn * n[c] + tv * Sj[c]) * n[r] - kt * n[r] * n[c]) - o * n[c];
      }
    }
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int c = 0; c < DIM; ++c) K[r][c] += B[r][c];
  }
}

// One warp per slice of A = K^T: lane t owns row j = 32*slice + t and,
// column by column (k), computes block K_ij with i the k-th entry of conns(j)
// and stores its transpose in the row's k-th slot.
template <int DIM>
__global__ void __launch_bounds__(256) k_assemble(AsmView v) {
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long sl = w0; sl < v.nslice; sl += nw) {
    const int j = (int)(sl * kSlice) + lane;
    const int len = j < v.n ? v.rowlen[j] : 0;
    const SellRow row = j < v.n ? sell_row(v.sell_ptr, j) : SellRow{0, 0, 0};
    for (int k = 0; k < len; ++k) {
      const int64_t slot = sell_slot(row, k);
      const int i = v.scol[slot];
      double K[3][3];
      if (i == j)
        diag_block<DIM>(v, i, K);
      else
        off_block<DIM>(v, i, j, K);
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int s = 0; s < DIM; ++s) v.A[(r * DIM + s) * v.nslots + slot] = K[s][r];
    }
  }
}

// |diag(K)|_2 (stiffness.h:269-270) and the DOFs to eliminate
// (stiffness.h:277: disp_constraint or damage_visual == 1).
template <int DIM>
__global__ void k_diag_norm_fixed(int n, const int* __restrict__ diag_slot, const double* __restrict__ A,
                                  int64_t nslots, const int* __restrict__ mask, const double* __restrict__ dvis,
                                  unsigned char* __restrict__ fixed, double* partials, unsigned int* ticket,
                                  double* norms) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = diag_slot[i];
    const bool dead = fabs(dvis[i] - 1.0) < EPS;
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
      if (s >= 0) {
        const double a = A[(r * DIM + r) * nslots + s];
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
__global__ void __launch_bounds__(256) k_apply_bc(int n, int nslice, const int64_t* __restrict__ sell_ptr,
                                                  const int* __restrict__ scol, const int* __restrict__ rowlen,
                                                  const unsigned char* __restrict__ fixed, const double* norms,
                                                  double* __restrict__ A, int64_t nslots) {
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const double nd = norms[2];
  for (long long sl = w0; sl < nslice; sl += nw) {
    const int j = (int)(sl * kSlice) + lane;
    if (j >= n) continue;
    unsigned char fj[DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r) fj[r] = fixed[DIM * j + r];
    const int len = rowlen[j];
    const SellRow row = sell_row(sell_ptr, j);
    for (int k = 0; k < len; ++k) {
      const int64_t slot = sell_slot(row, k);
      const int i = scol[slot];
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int s = 0; s < DIM; ++s)
          if (fj[r] || fixed[DIM * i + s]) A[(r * DIM + s) * nslots + slot] = (i == j && r == s) ? nd : 0.0;
    }
  }
}

__global__ void k_to_fp32(int64_t m, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

// 16-bit column offsets (column - row) of the slots the product reads for
// row j (sell_read_len).  The flag is set when one does not fit; the other
// slots are never read.
__global__ void k_col_offsets(int n, const int64_t* __restrict__ sell_ptr, const int* __restrict__ scol,
                              const int* __restrict__ rowlen, short* __restrict__ soff, int* flag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const SellRow row = sell_row(sell_ptr, j);
  const int len = sell_read_len(row, rowlen[j]);
  bool bad = false;
  for (int k = 0; k < len; ++k) {
    const int64_t s = sell_slot(row, k);
    const int o = scol[s] - j;
    bad |= (o < -32768 || o > 32767);
    soff[s] = (short)o;
  }
  if (bad) atomicOr(flag, 1);
}

// S_i = sum_j A_ij over the blocks of row i, summed in FP64 and rounded once.
template <int DIM>
__global__ void k_block_rowsum(int n, const int64_t* __restrict__ sell_ptr, const int* __restrict__ rowlen,
                               const double* __restrict__ A, int64_t nslots, float* __restrict__ S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SellRow row = sell_row(sell_ptr, i);
  double acc[DIM * DIM];
#pragma unroll
  for (int e = 0; e < DIM * DIM; ++e) acc[e] = 0.0;
  for (int k = 0; k < rowlen[i]; ++k) {
    const int64_t s = sell_slot(row, k);
#pragma unroll
    for (int e = 0; e < DIM * DIM; ++e) acc[e] += A[e * nslots + s];
  }
#pragma unroll
  for (int e = 0; e < DIM * DIM; ++e) S[(int64_t)i * DIM * DIM + e] = (float)acc[e];
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
  // sliced layout: each slice is as long as its longest row (groups of four,
  // then a tail of at most three single blocks)
  h->nslice = (n + kSlice - 1) / kSlice;
  std::vector<int64_t> sp((size_t)h->nslice + 1, 0);
  for (int sl = 0; sl < h->nslice; ++sl) {
    int64_t mx = 0;
    for (int j = sl * kSlice; j < std::min(n, (sl + 1) * kSlice); ++j) mx = std::max(mx, hc[(size_t)j]);
    sp[(size_t)sl + 1] = sp[(size_t)sl] + mx * kSlice;
  }
  h->nslots = sp[(size_t)h->nslice];
  if (h->nslots >= (int64_t)1 << 31) {
    cudaFreeAsync(cand, h->stream);
    h->err = "sliced operator has 2^31 or more slots";
    return LPM_ERR_ARG;
  }
  d.cptr = (int64_t*)dev_alloc(h, sizeof(int64_t) * ((size_t)n + 1));
  d.cidx = (int*)dev_alloc(h, sizeof(int) * (size_t)std::max<int64_t>(h->nblk, 1));
  d.diag_slot = (int*)dev_alloc(h, sizeof(int) * (size_t)n);
  d.sell_ptr = (int64_t*)dev_alloc(h, sizeof(int64_t) * ((size_t)h->nslice + 1));
  d.scol = (int*)dev_alloc(h, sizeof(int) * (size_t)std::max<int64_t>(h->nslots, 1));
  d.rowlen = (int*)dev_alloc(h, sizeof(int) * (size_t)n);
  if (!d.cptr || !d.cidx || !d.diag_slot || !d.sell_ptr || !d.scol || !d.rowlen) {
    cudaFreeAsync(cand, h->stream);
    return LPM_ERR_NOMEM;
  }
  LPM_CUDA(h, cudaMemcpyAsync(d.cptr, cp.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.sell_ptr, sp.data(), sizeof(int64_t) * (h->nslice + 1), cudaMemcpyHostToDevice,
                              h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.scol, 0, sizeof(int) * (size_t)std::max<int64_t>(h->nslots, 1), h->stream));
  k_compact_pattern<<<grid_for(n, T), T, 0, h->stream>>>(n, cand_ptr, cand, d.cptr, d.cidx);
  LPM_LAUNCHED(h, "k_compact_pattern");
  k_fill_sell<<<grid_for(n, T), T, 0, h->stream>>>(n, d.cptr, d.cidx, d.sell_ptr, d.scol, d.rowlen, d.diag_slot);
  LPM_LAUNCHED(h, "k_fill_sell");
  LPM_CUDA(h, cudaFreeAsync(cand, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int launch_assemble(lpm_handle* h, int tangent, int bc) {
  if (h->mf) return mf_assemble(h, tangent, bc);
  Dev& d = h->d;
  const int dim = h->dim;
  const size_t vals = (size_t)h->nslots * dim * dim;
  if (!d.A64) {
    d.A64 = (double*)dev_alloc(h, sizeof(double) * std::max<size_t>(vals, 1));
    if (!d.A64) return LPM_ERR_NOMEM;
    // padding slots stay zero for the life of the handle
    LPM_CUDA(h, cudaMemsetAsync(d.A64, 0, sizeof(double) * std::max<size_t>(vals, 1), h->stream));
  }
  AsmView v{d.bptr, d.lptr, d.sell_ptr, d.scol, d.rowlen, d.sbond, d.sp2, d.opp, d.cs, d.cs_sum, d.tsum, d.msum,
            d.Kn, d.Tv, d.bdamage, d.A64, h->nslots, h->n, h->nslice, tangent == LPM_TANGENT_SYMMETRIC ? 1 : 0};
  const int T = 256;
  const int G = grid_for((long long)h->nslice * 32, T, 152 * 64);
  if (dim == 3)
    k_assemble<3><<<G, T, 0, h->stream>>>(v);
  else
    k_assemble<2><<<G, T, 0, h->stream>>>(v);
  LPM_LAUNCHED(h, "k_assemble");
  if (bc == LPM_BC_ELIMINATE) {
    const int GR = grid_for(h->n, kRedThreads, kMaxRedBlocks);
    if (dim == 3)
      k_diag_norm_fixed<3><<<GR, kRedThreads, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nslots, d.mask, d.dvis,
                                                              d.fixed, d.red.partials, d.red.ticket + 1, d.norms);
    else
      k_diag_norm_fixed<2><<<GR, kRedThreads, 0, h->stream>>>(h->n, d.diag_slot, d.A64, h->nslots, d.mask, d.dvis,
                                                              d.fixed, d.red.partials, d.red.ticket + 1, d.norms);
    LPM_LAUNCHED(h, "k_diag_norm_fixed");
    if (dim == 3)
      k_apply_bc<3><<<G, T, 0, h->stream>>>(h->n, h->nslice, d.sell_ptr, d.scol, d.rowlen, d.fixed, d.norms, d.A64,
                                            h->nslots);
    else
      k_apply_bc<2><<<G, T, 0, h->stream>>>(h->n, h->nslice, d.sell_ptr, d.scol, d.rowlen, d.fixed, d.norms, d.A64,
                                            h->nslots);
    LPM_LAUNCHED(h, "k_apply_bc");
  }
  h->have_K = true;
  h->a32_valid = false;
  h->coarse_valid = false;
  h->last_bc = bc;
  h->tangent = tangent;
  return LPM_OK;
}

// FP32 copy of the operator for the mixed-precision solve, with the block
// row sums the difference-form product needs.
int convert_A32(lpm_handle* h) {
  Dev& d = h->d;
  const int dim = h->dim;
  const size_t vals = (size_t)h->nslots * dim * dim;
  if (!d.A32) {
    d.A32 = (float*)dev_alloc(h, sizeof(float) * std::max<size_t>(vals, 1));
    if (!d.A32) return LPM_ERR_NOMEM;
  }
  if (!d.S32) {
    d.S32 = (float*)dev_alloc(h, sizeof(float) * std::max<size_t>((size_t)h->n * dim * dim, 1));
    if (!d.S32) return LPM_ERR_NOMEM;
  }
  if (!d.soff16) {  // the pattern is fixed for the handle: offsets once
    d.soff16 = (short*)dev_alloc(h, sizeof(short) * std::max<size_t>((size_t)h->nslots, 1));
    int* flag = (int*)dev_alloc(h, sizeof(int));
    if (!d.soff16 || !flag) return LPM_ERR_NOMEM;
    LPM_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
    LPM_CUDA(h, cudaMemsetAsync(d.soff16, 0, sizeof(short) * std::max<size_t>((size_t)h->nslots, 1), h->stream));
    k_col_offsets<<<(h->n + 127) / 128, 128, 0, h->stream>>>(h->n, d.sell_ptr, d.scol, d.rowlen, d.soff16, flag);
    LPM_LAUNCHED(h, "k_col_offsets");
    int bad = 0;
    LPM_CUDA(h, cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    h->soff16_ok = bad == 0;
  }
  k_to_fp32<<<grid_for((long long)vals, 256, 152 * 32), 256, 0, h->stream>>>((int64_t)vals, d.A64, d.A32);
  LPM_LAUNCHED(h, "k_to_fp32");
  if (dim == 3)
    k_block_rowsum<3><<<(h->n + 127) / 128, 128, 0, h->stream>>>(h->n, d.sell_ptr, d.rowlen, d.A64, h->nslots, d.S32);
  else
    k_block_rowsum<2><<<(h->n + 127) / 128, 128, 0, h->stream>>>(h->n, d.sell_ptr, d.rowlen, d.A64, h->nslots, d.S32);
  LPM_LAUNCHED(h, "k_block_rowsum");
  h->a32_valid = true;
  return LPM_OK;
}

}  // namespace lpm
