// Neighbour search on the device: the bond rule of Assembly::createBonds
// (assembly.h:212-234) and the nonlocal neighbour lists of
// Assembly::searchNonlocalNeighbors (assembly.h:117-130), over a uniform cell
// grid instead of the all-pairs loop.
//
// Particles are binned into cubic cells at least as wide as the largest
// search radius, so every pair within range lies in the 27 cells around a
// particle.  A first pass counts each particle's partners, a host prefix sum
// places them, a second pass writes them and sorts each particle's list by
// partner id: the order createBonds pushes bonds in.  Distances use the
// reference's arithmetic, sqrt((x1-x2)^2 + (y1-y2)^2 + (z1-z2)^2) summed in
// that order, with the _rn intrinsics so that no FMA contraction changes a
// rounding: the accepted pairs and layers are bit-for-bit the reference's.
#include <algorithm>
#include <cmath>
#include <vector>

#include "lpm_device.cuh"

namespace lpm {
namespace {

struct Grid {
  double lo[3];
  double h;
  int dims[3];
};

__device__ __forceinline__ double ref_distance(const double* a, const double* b) {
  return bond_length(__dsub_rn(a[0], b[0]), __dsub_rn(a[1], b[1]), __dsub_rn(a[2], b[2]));
}

__device__ __forceinline__ void cell_of(const Grid& g, const double* x, int (&c)[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int v = (int)floor((x[k] - g.lo[k]) / g.h);
    c[k] = min(max(v, 0), g.dims[k] - 1);
  }
}

__global__ void k_bin_count(int n, const double* __restrict__ xyz, Grid g, int* __restrict__ cell,
                            int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  cell_of(g, xyz + 3 * (int64_t)i, c);
  const int id = (c[2] * g.dims[1] + c[1]) * g.dims[0] + c[0];
  cell[i] = id;
  atomicAdd(&count[id], 1);
}

__global__ void k_bin_fill(int n, const int* __restrict__ cell, const int* __restrict__ start, int* __restrict__ fill,
                           int* __restrict__ sorted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int id = cell[i];
  sorted[start[id] + atomicAdd(&fill[id], 1)] = i;
}

// Partners of particle i: distance below its radius (bonds: r1, layer 0
// below r0), itself included only for the nonlocal lists.  With out == null
// it counts; otherwise it writes (partner, layer) and sorts them by partner.
__global__ void k_pairs(int n, const double* __restrict__ xyz, Grid g, const int* __restrict__ start,
                        const int* __restrict__ sorted, const double* __restrict__ radius, double r_all, double r0,
                        int self, const int64_t* __restrict__ ptr, int64_t* __restrict__ count, int* __restrict__ out,
                        int* __restrict__ out_layer) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* xi = xyz + 3 * (int64_t)i;
  const double ri = radius ? radius[i] : r_all;
  int c[3];
  cell_of(g, xi, c);
  int64_t m = 0;
  const int64_t base = out ? ptr[i] : 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
        if (x < 0 || y < 0 || z < 0 || x >= g.dims[0] || y >= g.dims[1] || z >= g.dims[2]) continue;
        const int id = (z * g.dims[1] + y) * g.dims[0] + x;
        for (int q = start[id]; q < start[id + 1]; ++q) {
          const int j = sorted[q];
          if (j == i && !self) continue;
          const double d = ref_distance(xi, xyz + 3 * (int64_t)j);
          if (!(d < ri)) continue;
          if (out) {
            out[base + m] = j;
            if (out_layer) out_layer[base + m] = d < r0 ? 0 : 1;
          }
          ++m;
        }
      }
  if (!out) {
    count[i] = m;
    return;
  }
  // insertion sort by partner id (a few dozen entries)
  for (int64_t a = 1; a < m; ++a) {
    const int v = out[base + a];
    const int lv = out_layer ? out_layer[base + a] : 0;
    int64_t b = a - 1;
    while (b >= 0 && out[base + b] > v) {
      out[base + b + 1] = out[base + b];
      if (out_layer) out_layer[base + b + 1] = out_layer[base + b];
      --b;
    }
    out[base + b + 1] = v;
    if (out_layer) out_layer[base + b + 1] = lv;
  }
}

struct Scratch {
  std::vector<void*> p;
  ~Scratch() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T>
  T* get(size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) return nullptr;
    p.push_back(q);
    return (T*)q;
  }
};

int fail(cudaError_t e, const char* what) {
  set_global_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? LPM_ERR_NOMEM : LPM_ERR_CUDA;
}

#define SEARCH_CUDA(call)                        \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return fail(e_, #call); \
  } while (0)

// Shared driver: binning, counting and (when out is given) filling.
int search(int n, const double* xyz_h, const double* radius_h, double r_all, double r0, int self, int64_t capacity,
           int64_t* ptr_h, int* idx_h, int* layer_h, int64_t* total) {
  if (n <= 0 || !xyz_h || !total) {
    set_global_error("neighbour search: bad arguments");
    return LPM_ERR_ARG;
  }
  double rmax = r_all;
  if (radius_h) {
    rmax = 0.0;
    for (int i = 0; i < n; ++i) rmax = std::max(rmax, radius_h[i]);
  }
  if (!(rmax > 0.0) || !std::isfinite(rmax)) {
    set_global_error("neighbour search: the radius must be positive and finite");
    return LPM_ERR_ARG;
  }
  Grid g;
  double hi[3];
  for (int k = 0; k < 3; ++k) {
    g.lo[k] = hi[k] = xyz_h[k];
  }
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      g.lo[k] = std::min(g.lo[k], xyz_h[3 * (size_t)i + k]);
      hi[k] = std::max(hi[k], xyz_h[3 * (size_t)i + k]);
    }
  g.h = rmax * (1.0 + 1e-9);
  long long ncell = 1;
  for (int k = 0; k < 3; ++k) {
    g.dims[k] = (int)std::min<double>(std::floor((hi[k] - g.lo[k]) / g.h) + 1.0, 1 << 20);
    ncell *= g.dims[k];
  }
  // keep the grid at most a few cells per particle
  while (ncell > 4LL * n + 64) {
    g.h *= 1.5;
    ncell = 1;
    for (int k = 0; k < 3; ++k) {
      g.dims[k] = (int)std::floor((hi[k] - g.lo[k]) / g.h) + 1;
      ncell *= g.dims[k];
    }
  }
  Scratch s;
  double* xyz = s.get<double>(3 * (size_t)n);
  double* rad = radius_h ? s.get<double>((size_t)n) : nullptr;
  int* cell = s.get<int>((size_t)n);
  int* cnt = s.get<int>((size_t)ncell);
  int* start = s.get<int>((size_t)ncell + 1);
  int* fill = s.get<int>((size_t)ncell);
  int* sorted = s.get<int>((size_t)n);
  int64_t* count = s.get<int64_t>((size_t)n);
  int64_t* ptr = s.get<int64_t>((size_t)n + 1);
  if (!xyz || (radius_h && !rad) || !cell || !cnt || !start || !fill || !sorted || !count || !ptr)
    return fail(cudaErrorMemoryAllocation, "neighbour search scratch");
  SEARCH_CUDA(cudaMemcpy(xyz, xyz_h, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice));
  if (rad) SEARCH_CUDA(cudaMemcpy(rad, radius_h, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
  SEARCH_CUDA(cudaMemset(cnt, 0, sizeof(int) * (size_t)ncell));
  SEARCH_CUDA(cudaMemset(fill, 0, sizeof(int) * (size_t)ncell));
  const int T = 128;
  k_bin_count<<<grid_for(n, T), T>>>(n, xyz, g, cell, cnt);
  SEARCH_CUDA(cudaGetLastError());
  std::vector<int> hc((size_t)ncell), hs((size_t)ncell + 1, 0);
  SEARCH_CUDA(cudaMemcpy(hc.data(), cnt, sizeof(int) * (size_t)ncell, cudaMemcpyDeviceToHost));
  for (long long c = 0; c < ncell; ++c) hs[(size_t)c + 1] = hs[(size_t)c] + hc[(size_t)c];
  SEARCH_CUDA(cudaMemcpy(start, hs.data(), sizeof(int) * ((size_t)ncell + 1), cudaMemcpyHostToDevice));
  k_bin_fill<<<grid_for(n, T), T>>>(n, cell, start, fill, sorted);
  SEARCH_CUDA(cudaGetLastError());
  k_pairs<<<grid_for(n, T), T>>>(n, xyz, g, start, sorted, rad, r_all, r0, self, nullptr, count, nullptr, nullptr);
  SEARCH_CUDA(cudaGetLastError());
  std::vector<int64_t> hcount((size_t)n), hp((size_t)n + 1, 0);
  SEARCH_CUDA(cudaMemcpy(hcount.data(), count, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) hp[(size_t)i + 1] = hp[(size_t)i] + hcount[(size_t)i];
  *total = hp[(size_t)n];
  if (!idx_h) return LPM_OK;  // count only
  if (*total > capacity) {
    set_global_error("neighbour search: capacity too small (total returned)");
    return LPM_ERR_ARG;
  }
  int* idx = s.get<int>((size_t)*total);
  int* lay = layer_h ? s.get<int>((size_t)*total) : nullptr;
  if (!idx || (layer_h && !lay)) return fail(cudaErrorMemoryAllocation, "neighbour search output");
  SEARCH_CUDA(cudaMemcpy(ptr, hp.data(), sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice));
  k_pairs<<<grid_for(n, T), T>>>(n, xyz, g, start, sorted, rad, r_all, r0, self, ptr, count, idx, lay);
  SEARCH_CUDA(cudaGetLastError());
  SEARCH_CUDA(cudaMemcpy(idx_h, idx, sizeof(int) * (size_t)*total, cudaMemcpyDeviceToHost));
  if (layer_h) SEARCH_CUDA(cudaMemcpy(layer_h, lay, sizeof(int) * (size_t)*total, cudaMemcpyDeviceToHost));
  if (ptr_h) std::copy(hp.begin(), hp.end(), ptr_h);
  return LPM_OK;
}

}  // namespace
}  // namespace lpm

using namespace lpm;

extern "C" {

int lpm_find_bonds(int n, const double* xyz, double cutoff0, double cutoff1, int64_t capacity, int* p1, int* p2,
                   int* layer, int64_t* nb) {
  const double r0 = 1.01 * cutoff0, r1 = 1.01 * cutoff1;  // assembly.h:221-225
  std::vector<int64_t> ptr(p2 ? (size_t)n + 1 : 0);
  const int st = search(n, xyz, nullptr, r1, r0, 0, capacity, p2 ? ptr.data() : nullptr, p2, layer, nb);
  if (st || !p2) return st;
  if (p1)
    for (int i = 0; i < n; ++i)
      for (int64_t b = ptr[(size_t)i]; b < ptr[(size_t)i + 1]; ++b) p1[b] = i;
  return LPM_OK;
}

int lpm_find_neighbors(int n, const double* xyz, const double* radius, int64_t capacity, int64_t* ptr, int* idx,
                       int64_t* total) {
  if (!radius) {
    set_global_error("neighbour search: radius array required");
    return LPM_ERR_ARG;
  }
  return search(n, xyz, radius, 0.0, 0.0, 1, capacity, ptr, idx, nullptr, total);
}

}  // extern "C"
