// C ABI of liblpmgpu (declared in include/lpm_gpu.h): handle life cycle,
// host <-> device transfers and the Newton driver.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lpm_internal.cuh"

namespace lpm {

static thread_local std::string g_err;

void set_global_error(const std::string& msg) { g_err = msg; }

int cuda_fail(lpm_handle* h, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (h) h->err = m;
  g_err = m;
  return e == cudaErrorMemoryAllocation ? LPM_ERR_NOMEM : LPM_ERR_CUDA;
}

void* dev_alloc(lpm_handle* h, size_t bytes) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) {
    cuda_fail(h, e, "cudaMalloc");
    return nullptr;
  }
  h->allocations.push_back(p);
  return p;
}

void* zeros_dev(lpm_handle* h, size_t bytes) {
  void* p = dev_alloc(h, bytes);
  if (p && cudaMemset(p, 0, std::max<size_t>(bytes, 16)) != cudaSuccess) {
    cuda_fail(h, cudaErrorUnknown, "cudaMemset");
    return nullptr;
  }
  return p;
}

}  // namespace lpm

using namespace lpm;

namespace {

int arg_error(lpm_handle* h, const char* msg) {
  if (h) h->err = msg;
  g_err = msg;
  return LPM_ERR_ARG;
}

template <typename T>
T* upload_new(lpm_handle* h, const T* src, size_t count) {
  T* p = (T*)dev_alloc(h, sizeof(T) * count);
  if (!p) return nullptr;
  if (count && cudaMemcpy(p, src, sizeof(T) * count, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
  return p;
}

template <typename T>
T* zeros_new(lpm_handle* h, size_t count) {
  T* p = (T*)dev_alloc(h, sizeof(T) * count);
  if (!p) return nullptr;
  if (cudaMemset(p, 0, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) return nullptr;
  return p;
}

struct FieldRef {
  double* ptr;
  size_t count;
};

FieldRef field_ref(lpm_handle* h, int f) {
  const size_t N = (size_t)h->n, B = (size_t)h->nb, D = (size_t)h->dim;
  Dev& d = h->d;
  switch (f) {
    case LPM_F_XYZ: return {d.x, 3 * N};
    case LPM_F_XYZ0: return {d.x0, 3 * N};
    case LPM_F_PIN: return {d.pin, 3 * N};
    case LPM_F_PEX: return {d.pex, 3 * N};
    case LPM_F_STRESS: return {d.stress, 6 * N};
    case LPM_F_DVIS: return {d.dvis, N};
    case LPM_F_DLE_TOT: return {d.dle_tot, NL * N};
    case LPM_F_TDLE_TOT: return {d.tdle_tot, NL * N};
    case LPM_F_CS_SUM: return {d.cs_sum, NL * 3 * N};
    case LPM_F_DAMAGE: return {d.damage, N};
    case LPM_F_XYZ_LAST: return {d.xlast, 3 * N};
    case LPM_F_DISP: return {d.disp, D * N};
    case LPM_F_RESIDUAL: return {d.rhs, D * N};
    case LPM_F_STATE: return {d.state, (size_t)h->nstate * N};
    case LPM_F_DDOT_LOCAL: return {d.ddot_local, N};
    case LPM_F_DDOT_NONLOCAL: return {d.ddot_nl, N};
    case LPM_F_DAMAGE_LAST: return {d.damage_last, N};
    case LPM_B_BFORCE: return {d.bforce, B};
    case LPM_B_BDAMAGE: return {d.bdamage, B};
    case LPM_B_DLE: return {d.dLe, B};
    case LPM_B_DIS: return {d.dis, B};
    case LPM_B_BSTRAIN: return {d.bstrain, B};
    case LPM_B_CS: return {d.cs, 3 * B};
    case LPM_B_KN: return {d.Kn, B};
    case LPM_B_TV: return {d.Tv, B};
    case LPM_B_DIS0: return {d.dis0, B};
    case LPM_B_DLP: return {d.dLp, B};
    case LPM_B_SCRIT: return {d.bcrit, d.bcrit ? B : 0};
    case LPM_B_KAPPA: return {d.bkappa, d.bkappa ? B : 0};
  }
  return {nullptr, 0};
}

}  // namespace

extern "C" {

const char* lpm_last_error(const lpm_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

int lpm_set_device(int device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  return LPM_OK;
}

int lpm_create(int dim, int n, int64_t nb, const double* xyz, const int* p1, const int* p2, const int* layer,
               const double* Kn, const double* Tv, double particle_volume, int nneighbors, lpm_handle** out) {
  if (!out) return arg_error(nullptr, "out is NULL");
  *out = nullptr;
  if ((dim != 2 && dim != 3) || n <= 0 || nb < 0 || nneighbors <= 0 || !xyz || (nb > 0 && (!p1 || !p2 || !layer ||
                                                                                            !Kn || !Tv)))
    return arg_error(nullptr, "bad sizes or NULL arrays");
  if (nb >= ((int64_t)1 << 31) || (int64_t)n * 3 >= ((int64_t)1 << 31))
    return arg_error(nullptr, "lattice too large for 32-bit bond/particle indices");
  for (int64_t b = 0; b < nb; ++b)
    if (p1[b] < 0 || p1[b] >= n || p2[b] < 0 || p2[b] >= n || layer[b] < 0 || layer[b] >= NL)
      return arg_error(nullptr, "bond with particle id or layer out of range");
  const size_t N = (size_t)n, B = (size_t)nb;
  // bond CSR by (p1, layer), stable (bond_layers order)
  std::vector<int64_t> cnt(N * NL + 1, 0);
  for (int64_t b = 0; b < nb; ++b) cnt[(size_t)p1[b] * NL + layer[b] + 1]++;
  for (size_t k = 1; k < cnt.size(); ++k) cnt[k] += cnt[k - 1];
  std::vector<int64_t> src(B);
  {
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int64_t b = 0; b < nb; ++b) src[(size_t)pos[(size_t)p1[b] * NL + layer[b]]++] = b;
  }
  std::vector<int64_t> bptr(N + 1), lptr(N);
  for (size_t i = 0; i <= N; ++i) bptr[i] = cnt[i * NL];
  for (size_t i = 0; i < N; ++i) lptr[i] = cnt[i * NL + 1];
  std::vector<int> bp2(B), bl(B), nbonds(N), opp(B, -1);
  std::vector<double> kn(B), tv(B), dis0(B);
  for (size_t b = 0; b < B; ++b) {
    bp2[b] = p2[src[b]];
    bl[b] = layer[src[b]];
    kn[b] = Kn[src[b]];
    tv[b] = Tv[src[b]];
  }
  for (size_t i = 0; i < N; ++i) {
    nbonds[i] = (int)(bptr[i + 1] - bptr[i]);
    for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) {
      const double* xi = xyz + 3 * i;
      const double* xj = xyz + 3 * (size_t)bp2[(size_t)b];
      const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
      dis0[(size_t)b] = std::sqrt(dx * dx + dy * dy + dz * dz);
      // opposite bond: the first bond of p2 in the same layer pointing back
      // (particle.h:207-209)
      const int j = bp2[(size_t)b], l = bl[(size_t)b];
      const int64_t jb = l == 0 ? bptr[(size_t)j] : lptr[(size_t)j];
      const int64_t je = l == 0 ? lptr[(size_t)j] : bptr[(size_t)j + 1];
      for (int64_t c = jb; c < je; ++c)
        if (bp2[(size_t)c] == (int)i) {
          opp[(size_t)b] = (int)c;
          break;
        }
      if (opp[(size_t)b] < 0) {
        g_err = "bond without an opposite bond in the same layer";
        return LPM_ERR_TOPOLOGY;
      }
    }
  }
  lpm_handle* h = new lpm_handle();
  h->dim = dim;
  h->n = n;
  h->nb = nb;
  h->particle_volume = particle_volume;
  h->nneighbors = nneighbors;
  cudaGetDevice(&h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    int st = cuda_fail(h, e, "cudaStreamCreate");
    delete h;
    return st;
  }
  auto fail = [&](int st) {
    g_err = h->err;
    lpm_destroy(h);
    return st;
  };
  // partner-sorted view of each (particle, layer) bond segment, used by the
  // tangent's common-neighbour merge
  std::vector<int> sbond(B), sp2(B);
  for (size_t i = 0; i < N; ++i)
    for (int l = 0; l < NL; ++l) {
      const int64_t b0 = l == 0 ? bptr[i] : lptr[i], b1 = l == 0 ? lptr[i] : bptr[i + 1];
      for (int64_t b = b0; b < b1; ++b) sbond[(size_t)b] = (int)b;
      std::stable_sort(sbond.begin() + b0, sbond.begin() + b1,
                       [&](int a, int c) { return bp2[(size_t)a] < bp2[(size_t)c]; });
      for (int64_t b = b0; b < b1; ++b) sp2[(size_t)b] = bp2[(size_t)sbond[(size_t)b]];
    }
  Dev& d = h->d;
  bool ok = true;
  ok = ok && (d.sbond = upload_new(h, sbond.data(), B)) && (d.sp2 = upload_new(h, sp2.data(), B)) &&
       (d.tsum = zeros_new<double>(h, NL * 3 * N)) && (d.msum = zeros_new<double>(h, NL * 6 * N));
  ok = ok && (d.x = upload_new(h, xyz, 3 * N)) && (d.x0 = upload_new(h, xyz, 3 * N)) &&
       (d.xlast = upload_new(h, xyz, 3 * N));
  ok = ok && (d.pin = zeros_new<double>(h, 3 * N)) && (d.pex = zeros_new<double>(h, 3 * N)) &&
       (d.stress = zeros_new<double>(h, 6 * N)) && (d.dvis = zeros_new<double>(h, N)) &&
       (d.dle_tot = zeros_new<double>(h, NL * N)) && (d.tdle_tot = zeros_new<double>(h, NL * N)) &&
       (d.cs_sum = zeros_new<double>(h, NL * 3 * N)) && (d.damage = zeros_new<double>(h, N)) &&
       (d.damage_last = zeros_new<double>(h, N)) && (d.mask = zeros_new<int>(h, 3 * N)) &&
       (d.nbonds = upload_new(h, nbonds.data(), N)) && (d.fixed = zeros_new<unsigned char>(h, 3 * N));
  ok = ok && (d.bptr = upload_new(h, bptr.data(), N + 1)) && (d.lptr = upload_new(h, lptr.data(), N)) &&
       (d.bp2 = upload_new(h, bp2.data(), B)) && (d.blayer = upload_new(h, bl.data(), B)) &&
       (d.opp = upload_new(h, opp.data(), B)) && (d.Kn = upload_new(h, kn.data(), B)) &&
       (d.Tv = upload_new(h, tv.data(), B)) && (d.dis0 = upload_new(h, dis0.data(), B)) &&
       (d.dis = upload_new(h, dis0.data(), B)) && (d.dis_last = upload_new(h, dis0.data(), B));
  ok = ok && (d.dLe = zeros_new<double>(h, B)) && (d.dLp = zeros_new<double>(h, B)) &&
       (d.dLp_last = zeros_new<double>(h, B)) && (d.bstrain = zeros_new<double>(h, B)) &&
       (d.cs = zeros_new<double>(h, 3 * B)) && (d.bforce = zeros_new<double>(h, B)) &&
       (d.bforce_last = zeros_new<double>(h, B)) && (d.bdamage = zeros_new<double>(h, B)) &&
       (d.bdamage_last = zeros_new<double>(h, B));
  const size_t ndof = (size_t)dim * N;
  ok = ok && (d.rhs = zeros_new<double>(h, ndof)) && (d.disp = zeros_new<double>(h, ndof)) &&
       (d.x64 = zeros_new<double>(h, ndof)) && (d.r64 = zeros_new<double>(h, ndof)) &&
       (d.p64 = zeros_new<double>(h, ndof)) && (d.q64 = zeros_new<double>(h, ndof)) &&
       (d.invd64 = zeros_new<double>(h, ndof));
  ok = ok && (d.red.partials = zeros_new<double>(h, (size_t)kMaxRedBlocks * 4)) &&
       (d.red.ticket = zeros_new<unsigned int>(h, 16)) && (d.cg = zeros_new<CgScalars>(h, 1)) &&
       (d.norms = zeros_new<double>(h, 8)) && (d.gbar = zeros_new<unsigned long long>(h, 1));
  std::vector<double> crit(N, 1.0);
  ok = ok && (d.crit = upload_new(h, crit.data(), N)) && (d.pp = upload_new(h, crit.data(), N)) &&
       (d.ptype = zeros_new<int>(h, N)) && (d.state = zeros_new<double>(h, N)) &&
       (d.state_last = zeros_new<double>(h, N)) && (d.ddot_local = zeros_new<double>(h, N)) &&
       (d.ddot_nl = zeros_new<double>(h, N)) && (d.nonlocal_L = zeros_new<double>(h, N));
  if (!ok) return fail(h->err.empty() ? LPM_ERR_CUDA : LPM_ERR_NOMEM);
  if (cudaMallocHost((void**)&h->h_cg, sizeof(CgScalars)) != cudaSuccess ||
      cudaMallocHost((void**)&h->h_norms, 8 * sizeof(double)) != cudaSuccess) {
    h->err = "cudaMallocHost failed";
    return fail(LPM_ERR_NOMEM);
  }
  int st = build_pattern(h);
  if (st) return fail(st);
  *out = h;
  return LPM_OK;
}

int lpm_destroy(lpm_handle* h) {
  if (!h) return LPM_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->allocations) cudaFree(p);
  for (auto& c : h->checkpoints) cudaFree(c.buf);
  for (auto& g : h->groups) cudaFree(g.ids);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  if (h->fp_exec) cudaGraphExecDestroy(h->fp_exec);
  if (h->fp_graph) cudaGraphDestroy(h->fp_graph);
  if (h->mx_exec) cudaGraphExecDestroy(h->mx_exec);
  if (h->mx_graph) cudaGraphDestroy(h->mx_graph);
  if (h->h_cg) cudaFreeHost(h->h_cg);
  if (h->h_norms) cudaFreeHost(h->h_norms);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return LPM_OK;
}

int lpm_num_bonds(const lpm_handle* h, int64_t* nb) {
  if (!h || !nb) return LPM_ERR_ARG;
  *nb = h->nb;
  return LPM_OK;
}

int lpm_num_blocks(const lpm_handle* h, int64_t* nblocks) {
  if (!h || !nblocks) return LPM_ERR_ARG;
  *nblocks = h->nblk;
  return LPM_OK;
}

int lpm_get_pattern(const lpm_handle* h, int64_t* cptr, int* cidx) {
  if (!h) return LPM_ERR_ARG;
  lpm_handle* hh = const_cast<lpm_handle*>(h);
  if (cptr) LPM_CUDA(hh, cudaMemcpy(cptr, h->d.cptr, sizeof(int64_t) * (h->n + 1), cudaMemcpyDeviceToHost));
  if (cidx) LPM_CUDA(hh, cudaMemcpy(cidx, h->d.cidx, sizeof(int) * h->nblk, cudaMemcpyDeviceToHost));
  return LPM_OK;
}

int lpm_get_bonds(const lpm_handle* h, int64_t* bptr, int* bp2, int* blayer, int64_t* opp) {
  if (!h) return LPM_ERR_ARG;
  lpm_handle* hh = const_cast<lpm_handle*>(h);
  if (bptr) LPM_CUDA(hh, cudaMemcpy(bptr, h->d.bptr, sizeof(int64_t) * (h->n + 1), cudaMemcpyDeviceToHost));
  if (bp2) LPM_CUDA(hh, cudaMemcpy(bp2, h->d.bp2, sizeof(int) * h->nb, cudaMemcpyDeviceToHost));
  if (blayer) LPM_CUDA(hh, cudaMemcpy(blayer, h->d.blayer, sizeof(int) * h->nb, cudaMemcpyDeviceToHost));
  if (opp) {
    std::vector<int> o((size_t)h->nb);
    LPM_CUDA(hh, cudaMemcpy(o.data(), h->d.opp, sizeof(int) * h->nb, cudaMemcpyDeviceToHost));
    for (int64_t b = 0; b < h->nb; ++b) opp[b] = o[(size_t)b];
  }
  return LPM_OK;
}

int lpm_upload(lpm_handle* h, int field, const double* src) {
  if (!h || !src) return arg_error(h, "NULL handle or buffer");
  FieldRef f = field_ref(h, field);
  if (!f.ptr) return arg_error(h, "unknown field");
  LPM_CUDA(h, cudaMemcpyAsync(f.ptr, src, sizeof(double) * f.count, cudaMemcpyHostToDevice, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_download(lpm_handle* h, int field, double* dst) {
  if (!h || !dst) return arg_error(h, "NULL handle or buffer");
  FieldRef f = field_ref(h, field);
  if (!f.ptr) return arg_error(h, "unknown field");
  LPM_CUDA(h, cudaMemcpyAsync(dst, f.ptr, sizeof(double) * f.count, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_set_mask(lpm_handle* h, const int* mask) {
  if (!h || !mask) return arg_error(h, "NULL handle or buffer");
  LPM_CUDA(h, cudaMemcpyAsync(h->d.mask, mask, sizeof(int) * 3 * h->n, cudaMemcpyHostToDevice, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_get_mask(const lpm_handle* h, int* mask) {
  if (!h || !mask) return LPM_ERR_ARG;
  lpm_handle* hh = const_cast<lpm_handle*>(h);
  LPM_CUDA(hh, cudaMemcpyAsync(mask, h->d.mask, sizeof(int) * 3 * h->n, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(hh, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_update_damage(lpm_handle* h, int* any_new) {
  if (!h) return LPM_ERR_ARG;
  int flag = 0;
  int st = launch_static_damage(h, &flag);
  if (any_new) *any_new = flag;
  return st;
}

int lpm_fatigue_damage(lpm_handle* h, double dNdt, int* any_new) {
  if (!h) return LPM_ERR_ARG;
  int flag = 0;
  int st = launch_fatigue_damage(h, dNdt, &flag);
  if (any_new) *any_new = flag;
  return st;
}

int lpm_update_state(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  int st = launch_update_state(h);
  if (st) return st;
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_set_law(lpm_handle* h, int law, const double* params, int nparams, int per_particle) {
  if (!h) return LPM_ERR_ARG;
  static const int need[5] = {1, 3, 7, 4, 2};
  if (law < LPM_LAW_ELASTIC || law > LPM_LAW_SOFTENING) return arg_error(h, "unknown material law");
  if (nparams < need[law] || !params) return arg_error(h, "too few material parameters for the law");
  const size_t N = (size_t)h->n;
  std::vector<double> pp(N * (size_t)nparams);
  for (size_t i = 0; i < N; ++i)
    for (int k = 0; k < nparams; ++k) pp[i * nparams + k] = per_particle ? params[i * nparams + k] : params[k];
  const int ns = law == LPM_LAW_J2 ? 7 : (law == LPM_LAW_FATIGUE_HCF ? 3 : 1);
  std::vector<double> st(N * (size_t)ns, 0.0);
  if (law == LPM_LAW_FATIGUE_HCF)
    for (size_t i = 0; i < N; ++i) st[i * 3 + 1] = (double)INT_MAX;  // particle_fatigue_hcf.h:27
  Dev& d = h->d;
  double* npp = upload_new(h, pp.data(), pp.size());
  double* nst = upload_new(h, st.data(), st.size());
  double* nsl = upload_new(h, st.data(), st.size());
  if (!npp || !nst || !nsl) return h->err.empty() ? LPM_ERR_CUDA : LPM_ERR_NOMEM;
  d.pp = npp;
  d.state = nst;
  d.state_last = nsl;
  if (law == LPM_LAW_ELASTIC) {
    std::vector<double> c(N);
    for (size_t i = 0; i < N; ++i) c[i] = pp[i * nparams];
    LPM_CUDA(h, cudaMemcpy(d.crit, c.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  }
  if (law == LPM_LAW_SOFTENING) {
    // per-bond critical stretch from the owner's default; history cleared
    const size_t B = (size_t)h->nb;
    std::vector<int64_t> bptr(N + 1);
    LPM_CUDA(h, cudaMemcpy(bptr.data(), d.bptr, sizeof(int64_t) * (N + 1), cudaMemcpyDeviceToHost));
    std::vector<double> sc(B), zero(B, 0.0);
    for (size_t i = 0; i < N; ++i)
      for (int64_t b = bptr[i]; b < bptr[i + 1]; ++b) sc[(size_t)b] = pp[i * nparams + 1];
    if (!d.bcrit) d.bcrit = (double*)dev_alloc(h, sizeof(double) * std::max<size_t>(B, 1));
    if (!d.bkappa) d.bkappa = (double*)dev_alloc(h, sizeof(double) * std::max<size_t>(B, 1));
    if (!d.bkappa_last) d.bkappa_last = (double*)dev_alloc(h, sizeof(double) * std::max<size_t>(B, 1));
    if (!d.bcrit || !d.bkappa || !d.bkappa_last) return LPM_ERR_NOMEM;
    LPM_CUDA(h, cudaMemcpy(d.bcrit, sc.data(), sizeof(double) * B, cudaMemcpyHostToDevice));
    LPM_CUDA(h, cudaMemcpy(d.bkappa, zero.data(), sizeof(double) * B, cudaMemcpyHostToDevice));
    LPM_CUDA(h, cudaMemcpy(d.bkappa_last, zero.data(), sizeof(double) * B, cudaMemcpyHostToDevice));
  }
  h->law = law;
  h->law_np = nparams;
  h->nstate = ns;
  return LPM_OK;
}

int lpm_set_types(lpm_handle* h, const int* types, int undamaged_type) {
  if (!h || !types) return arg_error(h, "NULL handle or types");
  LPM_CUDA(h, cudaMemcpy(h->d.ptype, types, sizeof(int) * h->n, cudaMemcpyHostToDevice));
  h->undamaged = undamaged_type;
  return LPM_OK;
}

int lpm_set_nonlocal(lpm_handle* h, const int64_t* ptr, const int* idx, const double* L) {
  if (!h || !ptr || !L) return arg_error(h, "NULL nonlocal arrays");
  const size_t N = (size_t)h->n;
  if (ptr[0] != 0) return arg_error(h, "nonlocal pointer must start at 0");
  for (size_t i = 0; i < N; ++i)
    if (ptr[i + 1] < ptr[i]) return arg_error(h, "nonlocal pointer not ascending");
  const int64_t m = ptr[N];
  if (m > 0 && !idx) return arg_error(h, "NULL nonlocal indices");
  for (int64_t q = 0; q < m; ++q)
    if (idx[q] < 0 || idx[q] >= h->n) return arg_error(h, "nonlocal neighbour id out of range");
  Dev& d = h->d;
  int64_t* np_ = upload_new(h, ptr, N + 1);
  int* ni = (int*)dev_alloc(h, sizeof(int) * (size_t)std::max<int64_t>(m, 1));
  if (!np_ || !ni) return LPM_ERR_NOMEM;
  if (m) LPM_CUDA(h, cudaMemcpy(ni, idx, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice));
  LPM_CUDA(h, cudaMemcpy(d.nonlocal_L, L, sizeof(double) * N, cudaMemcpyHostToDevice));
  d.nl_ptr = np_;
  d.nl_idx = ni;
  return LPM_OK;
}

int lpm_add_group(lpm_handle* h, const int* ids, int count, int* group_id) {
  if (!h || !group_id || count < 0 || (count > 0 && !ids)) return arg_error(h, "bad group");
  for (int t = 0; t < count; ++t)
    if (ids[t] < 0 || ids[t] >= h->n) return arg_error(h, "group id out of range");
  Group g{nullptr, count};
  LPM_CUDA(h, cudaMalloc((void**)&g.ids, sizeof(int) * std::max(count, 1)));
  if (count) LPM_CUDA(h, cudaMemcpy(g.ids, ids, sizeof(int) * count, cudaMemcpyHostToDevice));
  h->groups.push_back(g);
  *group_id = (int)h->groups.size() - 1;
  return LPM_OK;
}

int lpm_apply_disp_bc(lpm_handle* h, int group, int axis, int mode, double value) {
  if (!h || group < 0 || group >= (int)h->groups.size() || axis < 0 || axis > 2 || (mode != 0 && mode != 1))
    return arg_error(h, "bad displacement BC");
  return launch_disp_bc(h, h->groups[(size_t)group], axis, mode, value);
}

int lpm_apply_force_bc(lpm_handle* h, int group, int mode, double fx, double fy, double fz) {
  if (!h || group < 0 || group >= (int)h->groups.size() || (mode != 0 && mode != 1))
    return arg_error(h, "bad force BC");
  return launch_force_bc(h, h->groups[(size_t)group], mode, fx, fy, fz);
}

int lpm_update_geometry_force(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  int st = launch_geometry_force(h);
  if (st) return st;
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_residual(lpm_handle* h, double* norm_residual, double* norm_reaction) {
  if (!h) return LPM_ERR_ARG;
  return launch_residual(h, norm_residual, norm_reaction);
}

int lpm_assemble(lpm_handle* h, int tangent, int bc) {
  if (!h || (tangent != LPM_TANGENT_AS_WRITTEN && tangent != LPM_TANGENT_SYMMETRIC) ||
      (bc != LPM_BC_NONE && bc != LPM_BC_ELIMINATE))
    return arg_error(h, "bad tangent or BC mode");
  int st = launch_assemble(h, tangent, bc);
  if (st) return st;
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_set_operator(lpm_handle* h, int kind) {
  if (!h) return LPM_ERR_ARG;
  if (kind != LPM_OPERATOR_ASSEMBLED && kind != LPM_OPERATOR_MATRIX_FREE) return arg_error(h, "unknown operator kind");
  const bool mf = kind == LPM_OPERATOR_MATRIX_FREE;
  if (mf != h->mf) {
    h->mf = mf;
    h->have_K = false;
    h->a32_valid = false;
  }
  return LPM_OK;
}

int lpm_get_K(const lpm_handle* h, double* vals) {
  if (!h || !vals) return LPM_ERR_ARG;
  lpm_handle* hh = const_cast<lpm_handle*>(h);
  if (h->mf) {
    hh->err = "matrix-free operator: the tangent is not assembled";
    return LPM_ERR_STATE;
  }
  if (!h->have_K) {
    hh->err = "no tangent assembled";
    return LPM_ERR_STATE;
  }
  const int dim = h->dim, e2 = dim * dim;
  const size_t ns = (size_t)h->nslots, nb = (size_t)h->nblk;
  std::vector<double> A(ns * e2);
  std::vector<int64_t> cptr((size_t)h->n + 1), sp((size_t)h->nslice + 1);
  std::vector<int> cidx(nb);
  LPM_CUDA(hh, cudaMemcpy(A.data(), h->d.A64, sizeof(double) * A.size(), cudaMemcpyDeviceToHost));
  LPM_CUDA(hh, cudaMemcpy(cptr.data(), h->d.cptr, sizeof(int64_t) * cptr.size(), cudaMemcpyDeviceToHost));
  LPM_CUDA(hh, cudaMemcpy(cidx.data(), h->d.cidx, sizeof(int) * nb, cudaMemcpyDeviceToHost));
  LPM_CUDA(hh, cudaMemcpy(sp.data(), h->d.sell_ptr, sizeof(int64_t) * sp.size(), cudaMemcpyDeviceToHost));
  // block (i, j) of K is block (j, i) of A transposed; (j, i) is the k-th
  // block of row j (sell_slot)
  for (int i = 0; i < h->n; ++i)
    for (int64_t q = cptr[(size_t)i]; q < cptr[(size_t)i + 1]; ++q) {
      const int j = cidx[(size_t)q];
      const int* b = &cidx[(size_t)cptr[(size_t)j]];
      const int* e = &cidx[(size_t)cptr[(size_t)j + 1]];
      const int* f = std::lower_bound(b, e, i);
      if (f == e || *f != i) {
        hh->err = "pattern is not structurally symmetric";
        return LPM_ERR_STATE;
      }
      const size_t slot = (size_t)lpm::sell_slot(lpm::sell_row(sp.data(), j), (int)(f - b));
      for (int r = 0; r < dim; ++r)
        for (int s = 0; s < dim; ++s) vals[(size_t)q * e2 + r * dim + s] = A[(size_t)(s * dim + r) * ns + slot];
    }
  return LPM_OK;
}

int lpm_solve(lpm_handle* h, int precision, double tol, int64_t maxit, int64_t* iters, double* relres) {
  if (!h) return LPM_ERR_ARG;
  if (!h->have_K) {
    h->err = "lpm_solve before lpm_assemble";
    return LPM_ERR_STATE;
  }
  long long it = 0;
  double rr = 0;
  int st;
  if (precision == LPM_PREC_FP64)
    st = solve_fp64(h, tol, maxit, &it, &rr);
  else if (precision == LPM_PREC_MIXED) {
    st = solve_mixed(h, tol, maxit, &it, &rr);
    if (st == LPM_ERR_NONFINITE) {  // FP32 recurrence broke down: the FP64 iteration decides
      h->stats.mixed_fallbacks++;
      st = solve_fp64(h, tol, maxit, &it, &rr);
    }
  }
  else
    return arg_error(h, "bad precision");
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return st;
}

int lpm_apply_operator(lpm_handle* h, int precision, const double* v, double* y) {
  if (!h || !v || !y) return arg_error(h, "NULL handle or buffer");
  if (precision != LPM_PREC_FP64 && precision != LPM_PREC_MIXED) return arg_error(h, "bad precision");
  if (!h->have_K) {
    h->err = "lpm_apply_operator before lpm_assemble";
    return LPM_ERR_STATE;
  }
  return apply_operator(h, precision, v, y);
}

int lpm_move_by_disp(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  int st = launch_move_by_disp(h);
  if (st) return st;
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_newton(lpm_handle* h, int max_iter, double tol, int precision, double cg_tol, int64_t cg_maxit,
               int* n_iter) {
  if (!h) return LPM_ERR_ARG;
  int st = launch_geometry_force(h);
  if (st) return st;
  double nr = 0, nR = 0;
  st = launch_residual(h, &nr, &nR);
  if (st) return st;
  const double mult = std::max(nr, nR);
  int ni = 0;
  while (nr > tol * mult) {
    if (++ni > max_iter) {
      if (n_iter) *n_iter = max_iter;
      return LPM_NOT_CONVERGED;
    }
    st = lpm_solve(h, precision, cg_tol, cg_maxit, nullptr, nullptr);
    if (st < 0 && st != LPM_ERR_NONFINITE) return st;
    st = launch_move_by_disp(h);
    if (st) return st;
    st = launch_geometry_force(h);
    if (st) return st;
    st = launch_residual(h, &nr, &nR);
    if (st) return st;
  }
  if (n_iter) *n_iter = ni;
  if (!std::isfinite(nr)) {
    h->err = "non-finite residual in the Newton iteration";
    return LPM_ERR_NONFINITE;
  }
  return LPM_OK;
}

int lpm_load_step(lpm_handle* h, const lpm_bc* bcs, int nbc, const lpm_step_opts* o, lpm_step_result* res) {
  if (!h || !o || nbc < 0 || (nbc > 0 && !bcs)) return arg_error(h, "bad load step");
  if (o->solver != LPM_SOLVER_STATIC && o->solver != LPM_SOLVER_FATIGUE_STATIC &&
      o->solver != LPM_SOLVER_STATIC_ELIMINATE)
    return arg_error(h, "bad solver kind");
  for (int k = 0; k < nbc; ++k)
    if (bcs[k].group < 0 || bcs[k].group >= (int)h->groups.size() || (bcs[k].kind != LPM_BC_DISP &&
                                                                     bcs[k].kind != LPM_BC_FORCE))
      return arg_error(h, "bad boundary condition");
  lpm_step_result r{};
  const int64_t it0 = h->stats.cg_iters_total;
  std::vector<double> pending{1.0};
  int st = LPM_OK;
  while (!pending.empty()) {
    const double s = pending.front();
    for (int k = 0; k < nbc; ++k)
      if (bcs[k].kind == LPM_BC_FORCE) {
        st = lpm_apply_force_bc(h, bcs[k].group, bcs[k].mode, bcs[k].fx * s, bcs[k].fy * s, bcs[k].fz * s);
        if (st) return st;
      }
    for (int k = 0; k < nbc; ++k)
      if (bcs[k].kind == LPM_BC_DISP) {
        st = lpm_apply_disp_bc(h, bcs[k].group, bcs[k].axis, bcs[k].mode, bcs[k].value * s);
        if (st) return st;
      }
    int ni = 0;
    bool failed = false;
    if (o->solver == LPM_SOLVER_FATIGUE_STATIC) {
      st = lpm_assemble(h, o->tangent, LPM_BC_ELIMINATE);
      if (st) return st;
      st = lpm_newton(h, o->max_iter, o->tol, o->precision, o->cg_tol, o->cg_maxit, &ni);
      if (st < 0) return st;
      failed = ni >= o->max_iter;
      if (!failed) {  // solver_fatigue.h:266-267
        st = launch_update_state(h);
        if (st) return st;
        st = lpm_store_state(h);
        if (st) return st;
      }
    } else {
      int damaged = 0;
      do {
        st = lpm_assemble(h, o->tangent, o->solver == LPM_SOLVER_STATIC_ELIMINATE ? LPM_BC_ELIMINATE : LPM_BC_NONE);
        if (st) return st;
        st = lpm_newton(h, o->max_iter, o->tol, o->precision, o->cg_tol, o->cg_maxit, &ni);
        if (st < 0) return st;
        if (ni >= o->max_iter) {
          failed = true;
          break;
        }
        st = launch_update_state(h);  // solver_static.h:122-123
        if (st) return st;
        st = launch_static_damage(h, &damaged);
        if (st) return st;
        st = lpm_store_state(h);
        if (st) return st;
        if (damaged && h->tg_ndir > 0 && h->law != LPM_LAW_SOFTENING) {
          h->err = "tangent sensitivity holds the damage fixed: a damage round ended the step";
          return LPM_ERR_STATE;
        }
        if (damaged) {
          ++r.damage_rounds;
          st = lpm_update_geometry_force(h);
          if (st) return st;
        }
      } while (damaged);
    }
    if (failed && h->tg_ndir > 0) {
      h->err = "tangent sensitivity does not follow load-step cut-backs";
      return LPM_ERR_STATE;
    }
    if (failed) {
      if (++r.cuts > o->max_cuts) {
        r.cg_iters = h->stats.cg_iters_total - it0;
        if (res) *res = r;
        h->err = "load step did not converge after the allowed cut-backs";
        return LPM_NOT_CONVERGED;
      }
      st = lpm_reset_state(h, 1);
      if (st) return st;
      pending.front() = 0.5 * s;
      pending.insert(pending.begin(), 0.5 * s);
      continue;
    }
    r.newton_iters = ni;
    pending.erase(pending.begin());
  }
  r.cg_iters = h->stats.cg_iters_total - it0;
  if (res) *res = r;
  return LPM_OK;
}

int lpm_store_state(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  Dev& d = h->d;
  const size_t N = (size_t)h->n, B = (size_t)h->nb;
  const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
  LPM_CUDA(h, cudaMemcpyAsync(d.xlast, d.x, sizeof(double) * 3 * N, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.damage_last, d.damage, sizeof(double) * N, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.dis_last, d.dis, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.bdamage_last, d.bdamage, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.bforce_last, d.bforce, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.dLp_last, d.dLp, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.state_last, d.state, sizeof(double) * N * h->nstate, k, h->stream));
  if (d.bkappa) LPM_CUDA(h, cudaMemcpyAsync(d.bkappa_last, d.bkappa, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_reset_state(lpm_handle* h, int reset_xyz) {
  if (!h) return LPM_ERR_ARG;
  Dev& d = h->d;
  const size_t N = (size_t)h->n, B = (size_t)h->nb;
  const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
  if (reset_xyz) LPM_CUDA(h, cudaMemcpyAsync(d.x, d.xlast, sizeof(double) * 3 * N, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.damage, d.damage_last, sizeof(double) * N, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.dis, d.dis_last, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.bdamage, d.bdamage_last, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.bforce, d.bforce_last, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.dLp, d.dLp_last, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaMemcpyAsync(d.state, d.state_last, sizeof(double) * N * h->nstate, k, h->stream));
  if (d.bkappa) LPM_CUDA(h, cudaMemcpyAsync(d.bkappa, d.bkappa_last, sizeof(double) * B, k, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_get_stats(const lpm_handle* h, lpm_stats* st) {
  if (!h || !st) return LPM_ERR_ARG;
  *st = h->stats;
  return LPM_OK;
}

int lpm_reset_stats(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  h->stats = lpm_stats{};
  return LPM_OK;
}

int lpm_set_cg_loop(lpm_handle* h, int mode) {
  if (!h) return LPM_ERR_ARG;
  if (mode != LPM_CG_LOOP_AUTO && mode != LPM_CG_LOOP_GRAPH && mode != LPM_CG_LOOP_PERSISTENT)
    return arg_error(h, "unknown CG loop mode");
  h->cg_loop = mode;
  return LPM_OK;
}

int lpm_set_preconditioner(lpm_handle* h, int kind, double box) {
  if (!h) return LPM_ERR_ARG;
  if (kind != LPM_PRECOND_JACOBI && kind != LPM_PRECOND_COARSE) return arg_error(h, "unknown preconditioner");
  if (!(box >= 0.0)) return arg_error(h, "box edge must be zero or positive");
  if (kind == LPM_PRECOND_COARSE && (box != h->cbox || !h->d.cagg)) {
    h->cbox = box;
    h->d.cagg = nullptr;  // aggregates rebuilt on the next solve (the old arrays stay with the handle)
    h->coarse_valid = false;
  }
  h->precond = kind;
  return LPM_OK;
}

int lpm_coarse_boxes(int dim, int n, const double* xyz0, double box, int* agg, int* nagg, double* edge) {
  if ((dim != 2 && dim != 3) || n < 0 || (n > 0 && (!xyz0 || !agg)) || !nagg || !(box >= 0.0)) {
    lpm::set_global_error("lpm_coarse_boxes: bad arguments");
    return LPM_ERR_ARG;
  }
  *nagg = lpm::coarse_boxes(dim, n, xyz0, box, agg, edge);
  return LPM_OK;
}

int lpm_set_kernel_timing(lpm_handle* h, int on) {
  if (!h) return LPM_ERR_ARG;
  h->timing = on != 0;
  return LPM_OK;
}

int lpm_get_stream(const lpm_handle* h, void** stream) {
  if (!h || !stream) return LPM_ERR_ARG;
  *stream = (void*)h->stream;
  return LPM_OK;
}

int lpm_synchronize(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}


}  // extern "C"

namespace {

int check_cycle_args(lpm_handle* h, const lpm_bc* bcs, int nbc, int n_interval, const lpm_step_opts* o) {
  if (!o || nbc < 0 || (nbc > 0 && !bcs) || n_interval < 1) return arg_error(h, "bad fatigue cycle");
  for (int k = 0; k < nbc; ++k)
    if (bcs[k].group < 0 || bcs[k].group >= (int)h->groups.size() ||
        (bcs[k].kind != LPM_BC_DISP && bcs[k].kind != LPM_BC_FORCE) || (bcs[k].mode != 0 && bcs[k].mode != 1) ||
        (bcs[k].kind == LPM_BC_DISP && (bcs[k].axis < 0 || bcs[k].axis > 2)))
      return arg_error(h, "bad boundary condition");
  return LPM_OK;
}

// One fatigue cycle (SolverFatigue::solveProblemOneCycle, solver_fatigue.h:
// 212-233).  The two load increments, loading and unloading half, come from
// the host (inc_host) or from device memory (inc_dev, the cyclic driver).
int cycle_core(lpm_handle* h, const lpm_bc* bcs, int nbc, const double* inc_host, const double* inc_dev,
               int n_interval, double dNdt, const lpm_step_opts* o, lpm_cycle_result* res) {
  lpm_cycle_result r{};
  const int64_t it0 = h->stats.cg_iters_total;
  int st = LPM_OK;
  for (int half = 0; half < 2; ++half) {
    for (int step = 0; step < n_interval; ++step) {
      // SolverFatigue::solveProblemStep (solver_fatigue.h:272-296)
      for (int k = 0; k < nbc; ++k)
        if (bcs[k].kind == LPM_BC_FORCE) {
          const Group& g = h->groups[(size_t)bcs[k].group];
          if (inc_dev)
            st = launch_force_bc_scaled(h, g, bcs[k].mode, bcs[k].fx, bcs[k].fy, bcs[k].fz, inc_dev + half);
          else
            st = lpm_apply_force_bc(h, bcs[k].group, bcs[k].mode, bcs[k].fx * inc_host[half],
                                    bcs[k].fy * inc_host[half], bcs[k].fz * inc_host[half]);
          if (st) return st;
        }
      for (int k = 0; k < nbc; ++k)
        if (bcs[k].kind == LPM_BC_DISP) {
          const Group& g = h->groups[(size_t)bcs[k].group];
          if (inc_dev)
            st = launch_disp_bc_scaled(h, g, bcs[k].axis, bcs[k].mode, bcs[k].value, inc_dev + half);
          else
            st = lpm_apply_disp_bc(h, bcs[k].group, bcs[k].axis, bcs[k].mode, bcs[k].value * inc_host[half]);
          if (st) return st;
        }
      st = lpm_assemble(h, o->tangent, LPM_BC_ELIMINATE);
      if (st) return st;
      int ni = 0;
      st = lpm_newton(h, o->max_iter, o->tol, o->precision, o->cg_tol, o->cg_maxit, &ni);
      if (st < 0) return st;
      r.newton_iters += ni;
      if (ni >= o->max_iter) ++r.unconverged_steps;
      st = launch_update_state(h);  // solver_fatigue.h:222
      if (st) return st;
    }
  }
  int any = 0;
  st = launch_fatigue_damage(h, dNdt, &any);  // solver_fatigue.h:229-232
  if (st) return st;
  st = lpm_store_state(h);
  if (st) return st;
  st = launch_geometry_force(h);
  if (st) return st;
  r.new_damage = any;
  r.cg_iters = h->stats.cg_iters_total - it0;
  if (res) *res = r;
  return r.unconverged_steps ? LPM_NOT_CONVERGED : LPM_OK;
}

}  // namespace

extern "C" {

int lpm_fatigue_cycle(lpm_handle* h, const lpm_bc* bcs, int nbc, double f0, double f1, double f2, int n_interval,
                      double dNdt, const lpm_step_opts* o, lpm_cycle_result* res) {
  if (!h) return LPM_ERR_ARG;
  int st = check_cycle_args(h, bcs, nbc, n_interval, o);
  if (st) return st;
  const double inc[2] = {(f1 - f0) / n_interval, (f2 - f1) / n_interval};
  return cycle_core(h, bcs, nbc, inc, nullptr, n_interval, dNdt, o, res);
}

int lpm_fatigue_run(lpm_handle* h, const lpm_bc* bcs, int nbc, const double* spectrum, int64_t nvalues,
                    int n_interval, int time_mode, double tau, int64_t max_cycles, const lpm_step_opts* o,
                    lpm_fatigue_record* records, int64_t capacity, int64_t* ncycles) {
  if (!h) return LPM_ERR_ARG;
  int st = check_cycle_args(h, bcs, nbc, n_interval, o);
  if (st) return st;
  if (!spectrum || nvalues < 3 || nvalues % 2 == 0)
    return arg_error(h, "spectrum: f_min then (f_max, f_min) pairs, an odd count of at least 3 values");
  if (!(tau > 0.0) || (time_mode != LPM_TIME_LINEAR && time_mode != LPM_TIME_EXPONENTIAL))
    return arg_error(h, "bad time map");
  if (capacity < 0 || (capacity > 0 && !records)) return arg_error(h, "bad record buffer");
  Dev& d = h->d;
  // the spectrum lives on the device for the run; cycle N's increments are
  // formed there and read by the BC kernels
  if (h->spectrum_cap < nvalues) {
    d.spectrum = (double*)dev_alloc(h, sizeof(double) * (size_t)nvalues);
    if (!d.spectrum) return LPM_ERR_NOMEM;
    h->spectrum_cap = nvalues;
  }
  if (!d.cycle) {
    d.cycle = (double*)zeros_dev(h, sizeof(double) * 4);
    if (!d.cycle) return LPM_ERR_NOMEM;
  }
  LPM_CUDA(h, cudaMemcpyAsync(d.spectrum, spectrum, sizeof(double) * (size_t)nvalues, cudaMemcpyHostToDevice,
                              h->stream));
  // SolverFatigue::solveProblemCyclic (solver_fatigue.h:174-210)
  const double n_cycles = 0.5 * (double)(nvalues - 1);
  long long N = 0;
  double t = 0.0;
  int64_t done = 0;
  int result = LPM_OK;
  while ((double)N < n_cycles && (max_cycles <= 0 || done < max_cycles)) {
    st = launch_cycle_increments(h, d.spectrum, N, n_interval, d.cycle);
    if (st) return st;
    const int dNdt = time_mode == LPM_TIME_LINEAR ? (int)(1 / tau) : (int)(1 / tau * exp(t / tau));
    if (time_mode == LPM_TIME_EXPONENTIAL) t += 1.0;
    lpm_cycle_result r{};
    st = cycle_core(h, bcs, nbc, nullptr, d.cycle, n_interval, (double)dNdt, o, &r);
    if (st < 0) return st;
    if (st == LPM_NOT_CONVERGED) result = LPM_NOT_CONVERGED;
    st = launch_mean_state0(h, d.cycle + 2);
    if (st) return st;
    double mean = 0.0;
    LPM_CUDA(h, cudaMemcpyAsync(&mean, d.cycle + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(h, cudaStreamSynchronize(h->stream));
    N += dNdt;
    if (done < capacity) {
      lpm_fatigue_record& rec = records[done];
      rec.N = N;
      rec.dNdt = dNdt;
      rec.newton_iters = r.newton_iters;
      rec.unconverged_steps = r.unconverged_steps;
      rec.new_damage = r.new_damage;
      rec.cg_iters = r.cg_iters;
      rec.mean_energy = mean;
    }
    ++done;
    if (dNdt <= 0) break;  // a time map below one cycle per step would never end
  }
  if (ncycles) *ncycles = done;
  return result;
}

int lpm_backward_step(lpm_handle* h, const double* dJdx, const double* dJdpin, double cg_tol, int64_t cg_maxit,
                      int accumulate, double* dJdKn, double* dJdTv, lpm_adjoint_result* res) {
  if (!h) return arg_error(h, "NULL handle");
  if (!(cg_tol > 0.0)) return arg_error(h, "cg_tol must be positive");
  int st = adjoint_buffers(h);
  if (st) return st;
  Dev& d = h->d;
  const size_t m = (size_t)h->n * h->dim;
  if (dJdx) LPM_CUDA(h, cudaMemcpyAsync(d.adj_a, dJdx, sizeof(double) * m, cudaMemcpyHostToDevice, h->stream));
  if (dJdpin) LPM_CUDA(h, cudaMemcpyAsync(d.adj_c, dJdpin, sizeof(double) * m, cudaMemcpyHostToDevice, h->stream));
  long long it = 0;
  double rel = 0.0;
  st = adjoint_step(h, dJdx ? d.adj_a : nullptr, dJdpin ? d.adj_c : nullptr, cg_tol, (long long)cg_maxit,
                    accumulate ? 1 : 0, d.adj_gkn, d.adj_gtv, &it, &rel);
  if (st < 0) return st;
  const size_t B = (size_t)h->nb;
  if (dJdKn) LPM_CUDA(h, cudaMemcpyAsync(dJdKn, d.adj_gkn, sizeof(double) * B, cudaMemcpyDeviceToHost, h->stream));
  if (dJdTv) LPM_CUDA(h, cudaMemcpyAsync(dJdTv, d.adj_gtv, sizeof(double) * B, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (res) {
    res->cg_iters = it;
    res->relres = rel;
  }
  h->stats.cg_iters_total += it;
  return st;
}

int lpm_apply_jacobian(lpm_handle* h, const double* v, double* y) {
  if (!h || !v || !y) return arg_error(h, "NULL handle or buffer");
  int st = adjoint_buffers(h);
  if (st) return st;
  Dev& d = h->d;
  const size_t m = (size_t)h->n * h->dim;
  LPM_CUDA(h, cudaMemcpyAsync(d.adj_p, v, sizeof(double) * m, cudaMemcpyHostToDevice, h->stream));
  st = adjoint_apply(h, d.adj_p, d.adj_q);
  if (st) return st;
  LPM_CUDA(h, cudaMemcpyAsync(y, d.adj_q, sizeof(double) * m, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(h, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_tangent_begin(lpm_handle* h, int ndir, const double* dparams, double tol) {
  if (!h) return LPM_ERR_ARG;
  return tangent_begin(h, ndir, dparams, tol);
}

int lpm_tangent_bond_constants(lpm_handle* h, int dir, const double* dKn, const double* dTv) {
  if (!h) return LPM_ERR_ARG;
  return tangent_bond_constants(h, dir, dKn, dTv);
}

int lpm_tangent_bond_scrit(lpm_handle* h, int dir, const double* dscrit) {
  if (!h) return LPM_ERR_ARG;
  return tangent_bond_scrit(h, dir, dscrit);
}

int lpm_tangent_get(const lpm_handle* h, int dir, int field, double* dst) {
  if (!h || !dst || dir < 0 || dir >= h->tg_ndir || (field != LPM_T_PIN && field != LPM_T_XYZ &&
                                                     field != LPM_T_DAMAGE))
    return LPM_ERR_ARG;
  lpm_handle* hh = const_cast<lpm_handle*>(h);
  if (field == LPM_T_DAMAGE) {
    LPM_CUDA(hh, cudaMemcpyAsync(dst, h->d.tg_dD + (size_t)dir * h->n, sizeof(double) * h->n,
                                 cudaMemcpyDeviceToHost, h->stream));
    LPM_CUDA(hh, cudaStreamSynchronize(h->stream));
    return LPM_OK;
  }
  const size_t m = (size_t)h->n * h->dim;
  const double* src = (field == LPM_T_PIN ? h->d.tg_pin : h->d.tg_x) + (size_t)dir * m;
  LPM_CUDA(hh, cudaMemcpyAsync(dst, src, sizeof(double) * m, cudaMemcpyDeviceToHost, h->stream));
  LPM_CUDA(hh, cudaStreamSynchronize(h->stream));
  return LPM_OK;
}

int lpm_tangent_end(lpm_handle* h) {
  if (!h) return LPM_ERR_ARG;
  h->tg_ndir = 0;
  return LPM_OK;
}

int lpm_checkpoint_save(lpm_handle* h, int* id) {
  if (!h || !id) return arg_error(h, "NULL handle or id");
  return checkpoint_save(h, id);
}

int lpm_checkpoint_restore(lpm_handle* h, int id) {
  if (!h) return arg_error(h, "NULL handle");
  return checkpoint_restore(h, id);
}

int lpm_checkpoint_drop(lpm_handle* h, int id) {
  if (!h) return arg_error(h, "NULL handle");
  return checkpoint_drop(h, id);
}

}  // extern "C"
