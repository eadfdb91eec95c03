// Coarse-space preconditioner of the mixed solve (lpm_set_preconditioner):
//   M^-1 = D^-1 + P A_c^-1 P^T,   A_c = P^T A P,
// additive two-level Schwarz with Jacobi as its one-level part.  The columns
// of P are the rigid-body modes (2-D: two translations and the rotation;
// 3-D: three translations and three rotations) of boxes of particles
// (aggregates), zero on eliminated DOFs.  Jacobi leaves the smooth,
// long-wavelength error of the lattice to the CG iterations; the coarse
// correction takes it out, so the iteration count stops growing with the
// lattice's size and depends on the box's instead.
//
// Set-up once per handle (host): the aggregates from the initial positions
// (boxes of an edge `box`, numbered in the order of their first particle),
// their members, each particle's offset from its aggregate's centroid, and
// the aggregate pairs the operator's pattern couples.  Once per assembly
// (device): A_c in FP64, one warp per aggregate pair summing over the pair's
// blocks in a fixed order; modes without stiffness (an aggregate whose DOFs
// are all eliminated, the rotation of a lone particle) set aside; then the
// inverse by Gauss-Jordan elimination without pivoting (A_c is symmetric
// positive definite on the remaining modes), one cooperative launch with a
// grid barrier per column.  The solve applies it in k_mx_persistent.
#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

#include "lpm_device.cuh"
#include "lpm_coarse.cuh"
#include "lpm_grid.cuh"

namespace lpm {

// Most coarse DOFs: the dense inverse (8 MB in FP64 at 1,024) stays in L2,
// and its Gauss-Jordan elimination takes one grid barrier per column.
constexpr int kCoarseMax = 1024;
// Coarse DOFs aimed at when the box edge is chosen automatically.
constexpr int kCoarseTarget = 480;

namespace {

// A_c block (a, b) = sum over i in a, blocks (i, j) with j in b, of
// P_i^T A_ij P_j.  One warp per pair: the lanes take the pair's rows (the
// members of a with a block in b) in turn and walk each row's slots in
// order; the lane sums are then folded by a fixed shuffle tree.
template <int DIM>
__global__ void __launch_bounds__(128) k_coarse_pairs(int npair, const int* __restrict__ pairs,
                                                      const int* __restrict__ prow_ptr, const int* __restrict__ prow,
                                                      const int* __restrict__ agg, const float* __restrict__ off,
                                                      const unsigned char* __restrict__ fixed,
                                                      const int64_t* __restrict__ sell_ptr,
                                                      const int* __restrict__ scol, const int* __restrict__ rowlen,
                                                      const double* __restrict__ A, int64_t nslots, int nc,
                                                      double* __restrict__ Ac) {
  constexpr int NM = kModes<DIM>;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= npair) return;
  const int a = pairs[2 * warp], b = pairs[2 * warp + 1];
  double c[NM][NM];
#pragma unroll
  for (int m = 0; m < NM; ++m)
#pragma unroll
    for (int q = 0; q < NM; ++q) c[m][q] = 0.0;
  for (int t = prow_ptr[warp] + lane; t < prow_ptr[warp + 1]; t += 32) {
    const int i = prow[t];
    double wi[DIM][NM];
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
      mode_row<DIM, double>(r, off[3 * i], off[3 * i + 1], off[3 * i + 2], wi[r]);
      if (fixed && fixed[(int64_t)DIM * i + r])
#pragma unroll
        for (int m = 0; m < NM; ++m) wi[r][m] = 0.0;
    }
    const int len = rowlen[i];
    const SellRow sr = sell_row(sell_ptr, i);
    for (int k = 0; k < len; ++k) {
      const int64_t s = k < sr.g4 ? sr.base + (int64_t)(k / kVec) * (kSlice * kVec) + (k % kVec)
                                  : sr.tail + (int64_t)(k - sr.g4) * kSlice;
      const int j = scol[s];
      if (agg[j] != b) continue;
      double wj[DIM][NM];
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        mode_row<DIM, double>(r, off[3 * j], off[3 * j + 1], off[3 * j + 2], wj[r]);
        if (fixed && fixed[(int64_t)DIM * j + r])
#pragma unroll
          for (int m = 0; m < NM; ++m) wj[r][m] = 0.0;
      }
      // (A_ij P_j)[r][q], then P_i^T times it
#pragma unroll
      for (int r = 0; r < DIM; ++r) {
        double ap[NM];
#pragma unroll
        for (int q = 0; q < NM; ++q) ap[q] = 0.0;
#pragma unroll
        for (int s2 = 0; s2 < DIM; ++s2) {
          const double v = A[(int64_t)(r * DIM + s2) * nslots + s];
#pragma unroll
          for (int q = 0; q < NM; ++q) ap[q] += v * wj[s2][q];
        }
#pragma unroll
        for (int m = 0; m < NM; ++m)
#pragma unroll
          for (int q = 0; q < NM; ++q) c[m][q] += wi[r][m] * ap[q];
      }
    }
  }
#pragma unroll
  for (int m = 0; m < NM; ++m)
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      double v = c[m][q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) Ac[(int64_t)(a * NM + m) * nc + b * NM + q] = v;
    }
}

// Modes without stiffness: a diagonal entry at most 1e-12 of the largest.
// Their rows and columns become those of the identity for the elimination
// (the inverse's are cleared afterwards); `active` records which are kept.
__global__ void k_coarse_guard(int nc, double* __restrict__ Ac, int* __restrict__ active) {
  __shared__ double smax[32];
  double m = 0.0;
  for (int q = threadIdx.x; q < nc; q += blockDim.x) m = fmax(m, fabs(Ac[(int64_t)q * nc + q]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = m;
  __syncthreads();
  m = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, smax[w]);
  for (int q = threadIdx.x; q < nc; q += blockDim.x) active[q] = fabs(Ac[(int64_t)q * nc + q]) > 1e-12 * m ? 1 : 0;
  __syncthreads();
  for (int64_t e = threadIdx.x; e < (int64_t)nc * nc; e += blockDim.x) {
    const int r = (int)(e / nc), c = (int)(e % nc);
    if (!active[r] || !active[c]) Ac[e] = r == c ? 1.0 : 0.0;
  }
}

// In-place Gauss-Jordan inversion without pivoting, ping-ponged between two
// buffers (step k reads one and writes the other), one grid barrier per
// step.  The result is then symmetrized, (B + B^T)/2, with the rows and
// columns of inactive modes cleared, into the other buffer (X when nc is
// odd, else Y): elimination leaves the computed inverse of an
// ill-conditioned A_c slightly unsymmetric, and CG needs a symmetric
// preconditioner.
__global__ void k_coarse_invert(int nc, double* X, double* Y, const int* __restrict__ active,
                                unsigned long long* gbar, long long spin_limit, int* fault) {
  const int64_t nn = (int64_t)nc * nc;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long target = 0;
  for (int k = 0; k < nc; ++k) {
    const double* src = (k & 1) ? Y : X;
    double* dst = (k & 1) ? X : Y;
    const double rp = 1.0 / __ldcg(&src[(int64_t)k * nc + k]);
    for (int64_t e = t0; e < nn; e += stride) {
      const int i = (int)(e / nc), j = (int)(e % nc);
      double v;
      if (i == k)
        v = j == k ? rp : __ldcg(&src[e]) * rp;
      else if (j == k)
        v = -__ldcg(&src[e]) * rp;
      else
        v = __ldcg(&src[e]) - __ldcg(&src[(int64_t)i * nc + k]) * rp * __ldcg(&src[(int64_t)k * nc + j]);
      dst[e] = v;
    }
    target += gridDim.x;
    if (!grid_barrier(gbar, target, spin_limit)) {
      if (threadIdx.x == 0) atomicExch(fault, 1);
      return;
    }
  }
  const double* res = (nc & 1) ? Y : X;
  double* out = (nc & 1) ? X : Y;
  for (int64_t e = t0; e < nn; e += stride) {
    const int i = (int)(e / nc), j = (int)(e % nc);
    out[e] = (!active[i] || !active[j]) ? 0.0 : 0.5 * (__ldcg(&res[e]) + __ldcg(&res[(int64_t)j * nc + i]));
  }
}

// The same coarse correction for FP64 vectors, as three launches (the
// tangent solves' BiCGSTAB, whose loop runs from the host): y = P^T r with a
// block per aggregate, e = A_c^-1 y with a block per aggregate, then
// z = invd r + P e per row.
template <int DIM>
__global__ void __launch_bounds__(256) k_coarse_restrict64(int nagg, const int* __restrict__ mem_ptr,
                                                           const int* __restrict__ mem, const float* __restrict__ off,
                                                           const unsigned char* __restrict__ fixed,
                                                           const double* __restrict__ r, double* __restrict__ y) {
  constexpr int NM = kModes<DIM>;
  for (int ag = blockIdx.x; ag < nagg; ag += gridDim.x) {
    double acc[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) acc[m] = 0.0;
    for (int t = mem_ptr[ag] + threadIdx.x; t < mem_ptr[ag + 1]; t += blockDim.x) {
      const int i = mem[t];
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const int64_t q = (int64_t)DIM * i + k;
        if (fixed[q]) continue;
        double w[NM];
        mode_row<DIM, double>(k, off[3 * i], off[3 * i + 1], off[3 * i + 2], w);
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m] += w[m] * r[q];
      }
    }
    block_sum<NM>(acc);
    if (threadIdx.x == 0)
#pragma unroll
      for (int m = 0; m < NM; ++m) y[ag * NM + m] = acc[m];
  }
}

template <int DIM>
__global__ void __launch_bounds__(256) k_coarse_solve64(int nagg, const double* __restrict__ Ainv,
                                                        const double* __restrict__ y, double* __restrict__ e) {
  constexpr int NM = kModes<DIM>;
  const int nc = nagg * NM;
  for (int ag = blockIdx.x; ag < nagg; ag += gridDim.x) {
    double acc[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) acc[m] = 0.0;
    for (int c = threadIdx.x; c < nc; c += blockDim.x)
#pragma unroll
      for (int m = 0; m < NM; ++m) acc[m] += Ainv[(int64_t)(ag * NM + m) * nc + c] * y[c];
    block_sum<NM>(acc);
    if (threadIdx.x == 0)
#pragma unroll
      for (int m = 0; m < NM; ++m) e[ag * NM + m] = acc[m];
  }
}

template <int DIM>
__global__ void k_coarse_prolong64(int n, const int* __restrict__ agg, const float* __restrict__ off,
                                   const unsigned char* __restrict__ fixed, const double* __restrict__ invd,
                                   const double* __restrict__ r, const double* __restrict__ e,
                                   double* __restrict__ z) {
  constexpr int NM = kModes<DIM>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ag = agg[i];
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    const int64_t q = (int64_t)DIM * i + k;
    double zi = invd[q] * r[q];
    if (!fixed[q]) {
      double w[NM];
      mode_row<DIM, double>(k, off[3 * i], off[3 * i + 1], off[3 * i + 2], w);
#pragma unroll
      for (int m = 0; m < NM; ++m) zi += w[m] * e[ag * NM + m];
    }
    z[q] = zi;
  }
}

}  // namespace

// The aggregates: boxes of edge `box` from the lowest corner of the
// particles' bounding box (box <= 0: the edge that gives about
// kCoarseTarget coarse DOFs for the box volume), numbered in the order of
// their first particle.  Writes agg[n] and the edge used; returns the count.
int coarse_boxes(int dim, int n, const double* x0, double box, int* agg, double* edge_out) {
  const int nm = dim == 3 ? 6 : 3;
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = hi[k] = n ? x0[k] : 0.0;
    for (int i = 0; i < n; ++i) {
      lo[k] = std::min(lo[k], x0[3 * i + k]);
      hi[k] = std::max(hi[k], x0[3 * i + k]);
    }
  }
  double edge = box;
  if (!(edge > 0.0)) {
    double vol = 1.0;
    for (int k = 0; k < dim; ++k) vol *= std::max(hi[k] - lo[k], 1e-300);
    edge = std::pow(vol / std::max(1, kCoarseTarget / nm), 1.0 / dim);
    if (!(edge > 0.0) || !std::isfinite(edge)) edge = 1.0;  // no extent (one particle): one box
  }
  std::unordered_map<int64_t, int> box_id;
  for (int i = 0; i < n; ++i) {
    int64_t key = 0;
    for (int k = 0; k < dim; ++k) key = key * 2000003 + (int64_t)std::floor((x0[3 * i + k] - lo[k]) / edge);
    auto it = box_id.emplace(key, (int)box_id.size()).first;
    agg[i] = it->second;
  }
  if (edge_out) *edge_out = edge;
  return (int)box_id.size();
}

int coarse_setup(lpm_handle* h) {
  Dev& d = h->d;
  const int n = h->n, dim = h->dim, nm = dim == 3 ? 6 : 3;
  std::vector<double> x0((size_t)3 * n);
  LPM_CUDA(h, cudaMemcpyAsync(x0.data(), d.x0, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
  std::vector<int64_t> cptr((size_t)n + 1);
  std::vector<int> cidx((size_t)h->nblk);
  LPM_CUDA(h, cudaMemcpyAsync(cptr.data(), d.cptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(cidx.data(), d.cidx, sizeof(int) * h->nblk, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<int> agg((size_t)n);
  double edge = 0.0;
  const int nagg = coarse_boxes(dim, n, x0.data(), h->cbox, agg.data(), &edge);
  if ((long long)nagg * nm > kCoarseMax) {
    h->err = "coarse preconditioner: " + std::to_string(nagg) + " aggregates exceed " +
             std::to_string(kCoarseMax / nm) + "; give a larger box";
    return LPM_ERR_ARG;
  }
  std::vector<int> mem_ptr((size_t)nagg + 1, 0), mem((size_t)n);
  for (int i = 0; i < n; ++i) mem_ptr[(size_t)agg[(size_t)i] + 1]++;
  for (int a = 0; a < nagg; ++a) mem_ptr[(size_t)a + 1] += mem_ptr[(size_t)a];
  std::vector<int> fill(mem_ptr.begin(), mem_ptr.end() - 1);
  std::vector<double> cen((size_t)3 * nagg, 0.0);
  for (int i = 0; i < n; ++i) {
    const int a = agg[(size_t)i];
    mem[(size_t)fill[(size_t)a]++] = i;
    for (int k = 0; k < 3; ++k) cen[(size_t)3 * a + k] += x0[(size_t)3 * i + k];
  }
  std::vector<float> off((size_t)3 * n);
  for (int a = 0; a < nagg; ++a)
    for (int k = 0; k < 3; ++k) cen[(size_t)3 * a + k] /= std::max(1, mem_ptr[(size_t)a + 1] - mem_ptr[(size_t)a]);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k)
      off[(size_t)3 * i + k] = (float)(x0[(size_t)3 * i + k] - cen[(size_t)3 * agg[(size_t)i] + k]);
  // aggregate pairs coupled by the pattern, in order, each with its rows
  // (the members of a with a block in b, ascending)
  std::vector<int> pairs, prow_ptr(1, 0), prow;
  std::vector<int> seen_row((size_t)nagg, -1);
  std::vector<std::vector<int>> rows_of((size_t)nagg);
  std::vector<int> nbr;
  for (int a = 0; a < nagg; ++a) {
    nbr.clear();
    for (int t = mem_ptr[(size_t)a]; t < mem_ptr[(size_t)a + 1]; ++t) {
      const int i = mem[(size_t)t];
      for (int64_t q = cptr[(size_t)i]; q < cptr[(size_t)i + 1]; ++q) {
        const int b = agg[(size_t)cidx[(size_t)q]];
        if (seen_row[(size_t)b] == i) continue;
        if (rows_of[(size_t)b].empty()) nbr.push_back(b);
        seen_row[(size_t)b] = i;
        rows_of[(size_t)b].push_back(i);
      }
    }
    std::sort(nbr.begin(), nbr.end());
    for (int b : nbr) {
      pairs.push_back(a);
      pairs.push_back(b);
      prow.insert(prow.end(), rows_of[(size_t)b].begin(), rows_of[(size_t)b].end());
      prow_ptr.push_back((int)prow.size());
      rows_of[(size_t)b].clear();
    }
  }
  const int nc = nagg * nm;
  const int64_t ndof = (int64_t)n * dim;
  d.cagg = (int*)dev_alloc(h, sizeof(int) * n);
  d.cmem_ptr = (int*)dev_alloc(h, sizeof(int) * (nagg + 1));
  d.cmem = (int*)dev_alloc(h, sizeof(int) * n);
  d.cpair = (int*)dev_alloc(h, sizeof(int) * std::max<size_t>(pairs.size(), 1));
  d.cprow_ptr = (int*)dev_alloc(h, sizeof(int) * prow_ptr.size());
  d.cprow = (int*)dev_alloc(h, sizeof(int) * std::max<size_t>(prow.size(), 1));
  d.coff = (float*)dev_alloc(h, sizeof(float) * 3 * n);
  d.cA = (double*)dev_alloc(h, sizeof(double) * (size_t)nc * nc);
  d.cA2 = (double*)dev_alloc(h, sizeof(double) * (size_t)nc * nc);
  d.cact = (int*)dev_alloc(h, sizeof(int) * nc);
  d.cyc = (double*)dev_alloc(h, sizeof(double) * nc);
  d.cec = (double*)dev_alloc(h, sizeof(double) * nc);
  d.cz = (float*)dev_alloc(h, sizeof(float) * ndof);
  d.cfault = (int*)dev_alloc(h, sizeof(int));
  if (!d.cagg || !d.cmem_ptr || !d.cmem || !d.cpair || !d.cprow_ptr || !d.cprow || !d.coff || !d.cA || !d.cA2 ||
      !d.cact || !d.cyc || !d.cec || !d.cz || !d.cfault)
    return LPM_ERR_NOMEM;
  LPM_CUDA(h, cudaMemcpyAsync(d.cagg, agg.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.cmem_ptr, mem_ptr.data(), sizeof(int) * (nagg + 1), cudaMemcpyHostToDevice,
                              h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.cmem, mem.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  if (!pairs.empty())
    LPM_CUDA(h, cudaMemcpyAsync(d.cpair, pairs.data(), sizeof(int) * pairs.size(), cudaMemcpyHostToDevice,
                                h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.coff, off.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.cprow_ptr, prow_ptr.data(), sizeof(int) * prow_ptr.size(), cudaMemcpyHostToDevice,
                              h->stream));
  if (!prow.empty())
    LPM_CUDA(h, cudaMemcpyAsync(d.cprow, prow.data(), sizeof(int) * prow.size(), cudaMemcpyHostToDevice, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->cnagg = nagg;
  h->cnc = nc;
  h->cnpair = (int)(pairs.size() / 2);
  h->cedge = edge;
  h->coarse_valid = false;
  return LPM_OK;
}

// A_c of the current operator and its symmetrized inverse (in d.cAinv).
int coarse_assemble(lpm_handle* h) {
  Dev& d = h->d;
  if (!d.cagg) {
    const int st = coarse_setup(h);
    if (st) return st;
  }
  const int nc = h->cnc;
  const unsigned char* fixed = h->last_bc == LPM_BC_ELIMINATE ? d.fixed : nullptr;
  LPM_CUDA(h, cudaMemsetAsync(d.cA, 0, sizeof(double) * (size_t)nc * nc, h->stream));
  const int warps_per_block = 4;
  const int G = (h->cnpair + warps_per_block - 1) / warps_per_block;
  if (G > 0) {
    if (h->dim == 3)
      k_coarse_pairs<3><<<G, 32 * warps_per_block, 0, h->stream>>>(h->cnpair, d.cpair, d.cprow_ptr, d.cprow, d.cagg,
                                                                  d.coff, fixed, d.sell_ptr, d.scol, d.rowlen,
                                                                  d.A64, h->nslots, nc, d.cA);
    else
      k_coarse_pairs<2><<<G, 32 * warps_per_block, 0, h->stream>>>(h->cnpair, d.cpair, d.cprow_ptr, d.cprow, d.cagg,
                                                                  d.coff, fixed, d.sell_ptr, d.scol, d.rowlen,
                                                                  d.A64, h->nslots, nc, d.cA);
    LPM_LAUNCHED(h, "k_coarse_pairs");
  }
  k_coarse_guard<<<1, 1024, 0, h->stream>>>(nc, d.cA, d.cact);
  LPM_LAUNCHED(h, "k_coarse_guard");
  if (!h->sms && cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess)
    h->sms = 1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_coarse_invert, 256, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long long want = ((long long)nc * nc + 255) / 256;
  const int grid = (int)std::max<long long>(1, std::min<long long>((long long)h->sms * per_sm, want));
  LPM_CUDA(h, cudaMemsetAsync(d.gbar, 0, sizeof(unsigned long long), h->stream));
  LPM_CUDA(h, cudaMemsetAsync(d.cfault, 0, sizeof(int), h->stream));
  long long spin = kPcgSpinLimit;
  int ncv = nc;
  void* args[] = {&ncv, &d.cA, &d.cA2, &d.cact, &d.gbar, &spin, &d.cfault};
  LPM_CUDA(h, cudaLaunchCooperativeKernel((const void*)k_coarse_invert, dim3(grid), dim3(256), args, 0, h->stream));
  LPM_LAUNCHED(h, "k_coarse_invert");
  int fault = 0;
  LPM_CUDA(h, cudaMemcpyAsync(&fault, d.cfault, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (fault) {
    h->err = "coarse preconditioner: a grid-barrier wait gave up in the inversion";
    return LPM_ERR_STATE;
  }
  d.cAinv = (nc & 1) ? d.cA : d.cA2;
  h->coarse_valid = true;
  return LPM_OK;
}

}  // namespace lpm

namespace lpm {

// The coarse correction applies to the tangent solves when the user chose it
// and the last assembly is the symmetric tangent with the displacement BCs
// eliminated (its eliminated DOFs contain the constrained ones, on which the
// correction is zero).
bool coarse_usable(const lpm_handle* h) {
  return h->precond == LPM_PRECOND_COARSE && h->have_K && !h->mf && h->tangent == LPM_TANGENT_SYMMETRIC &&
         h->last_bc == LPM_BC_ELIMINATE;
}

int coarse_apply64(lpm_handle* h, const double* r, const double* invd, double* z) {
  Dev& d = h->d;
  if (!h->coarse_valid) {
    const int st = coarse_assemble(h);
    if (st) return st;
  }
  const int nagg = h->cnagg;
  if (h->dim == 3) {
    k_coarse_restrict64<3><<<nagg, 256, 0, h->stream>>>(nagg, d.cmem_ptr, d.cmem, d.coff, d.fixed, r, d.cyc);
    k_coarse_solve64<3><<<nagg, 256, 0, h->stream>>>(nagg, d.cAinv, d.cyc, d.cec);
    k_coarse_prolong64<3><<<grid_for(h->n, 256), 256, 0, h->stream>>>(h->n, d.cagg, d.coff, d.fixed, invd, r, d.cec, z);
  } else {
    k_coarse_restrict64<2><<<nagg, 256, 0, h->stream>>>(nagg, d.cmem_ptr, d.cmem, d.coff, d.fixed, r, d.cyc);
    k_coarse_solve64<2><<<nagg, 256, 0, h->stream>>>(nagg, d.cAinv, d.cyc, d.cec);
    k_coarse_prolong64<2><<<grid_for(h->n, 256), 256, 0, h->stream>>>(h->n, d.cagg, d.coff, d.fixed, invd, r, d.cec, z);
  }
  LPM_LAUNCHED(h, "k_coarse_apply64");
  h->stats.kernel_launches += 2;
  return LPM_OK;
}

}  // namespace lpm
