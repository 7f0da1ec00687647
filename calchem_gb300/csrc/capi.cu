// capi.cu -- the library's C ABI (include/calchem_xc.h).
//
// Device state lives in a process-wide map keyed by the caller's grid id, guarded by one mutex,
// as in the reference (crates/calchem-cuda/src/cuda_kernels.cu:6004-6041, 7354-7562).  Every
// input is validated on the host before anything is enqueued, so malformed uploads are rejected
// with an error code and never reach a kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "grid_build.h"
#include "host_prep.h"
#include "launch.h"


using namespace cxc;

namespace {

constexpr int kPlanes = 5;

struct Entry {
  int n_pts = 0, n_ao = 0, n_shells = 0, n_batches = 0, max_m = 0;
  int n_prims = 0, n_comps = 0;
  size_t n_cand = 0, n_bao = 0;
  // molecules: one for an uploaded grid; several for a group (calchem_xc_group_create), whose
  // densities and Vxc are packed blocks (n_ao then counts the rows of all blocks)
  int n_mols = 1, max_n = 0;
  long long nn_total = 0;
  std::vector<int> h_mol_n, h_mol_ao_off, h_mol_boff;
  std::vector<long long> h_mol_off;
  int* d_mol_n = nullptr;
  long long* d_mol_off = nullptr;
  int* d_mol_ao_off = nullptr;
  int* d_mol_boff = nullptr;
  bool ws = false;  // evaluation workspace allocated (ensure_ws)
  size_t bytes = 0;
  size_t mem_limit = SIZE_MAX;  // the caller's device-memory budget for this grid
  bool has_w = false;
  double sum_m2n = 0, sum_m2 = 0;
  AoShellGpu* d_shells = nullptr;
  AoPrimGpu* d_prims = nullptr;
  AoCompGpu* d_comps = nullptr;
  float4* d_prim_f = nullptr;
  float2* d_comp_f = nullptr;
  float2* d_shell_cf = nullptr;
  double* d_pts = nullptr;  // SoA x | y | z | w, n_pts each
  BatchDesc* d_batches = nullptr;
  int* d_cand = nullptr;
  int* d_cand_loc = nullptr;
  int* d_bao = nullptr;
  int* d_order = nullptr;
  double* d_P = nullptr;
  double* d_Pb = nullptr;
  double* d_V = nullptr;
  double* d_Vb = nullptr;
  double* d_rg = nullptr;
  double* d_red = nullptr;
  double* d_res = nullptr;
  int* d_counter = nullptr;
  double* d_slab = nullptr;
  size_t slab_stride = 0;
  int n_ctas = 0;
  void* d_mixed_ws = nullptr;  // split copies of the density for the tensor-core path
  size_t mixed_slab_stride = 0;
  double* d_mixed_slab = nullptr;
  int mixed_ctas = 0;               // tensor-core CTAs the workspace has slabs for
  int tile_n = 64;                  // tensor-core GEMM1 N chunk (calchem_xc_set_tile)
  double* h_stage = nullptr;  // pinned: 2 n^2 + 4 doubles
  cudaStream_t stream = nullptr;
  int last_launches = 0;
  bool profiling = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraphExec_t graph = nullptr;  // captured evaluation (calchem_xc_graph_capture_*)
  double* d_pt_out = nullptr;       // per-point outputs (calchem_xc_evaluate_rks_points), 2 per point
  double* d_fxc = nullptr;          // TD-DFT kernel coefficients, 11 per point (calchem_xc_fxc_prepare)
  int fxc_code = -1;                // functional of d_fxc (-1: not prepared)
  double* d_fxc_m = nullptr;        // trial matrices / results of host-buffer contractions
  double* d_fxc_v = nullptr;
  int fxc_cap = 0;                  // trial matrices d_fxc_m and d_fxc_v hold
  // AO cache of the tensor-core form (EvalArgs::ao_cache): 0 = decide at the next tensor-core
  // evaluation, 1 = off (disabled, over the cap or no memory), 2 = allocated
  int ao_cache_state = 0;
  unsigned char* d_ao_cache = nullptr;
  long long* d_ao_cache_off = nullptr;
  int* d_ao_cache_ok = nullptr;
  size_t ao_cache_bytes = 0;
  // per-atom share sums (calchem_xc_set_point_atoms): planned point indices grouped by host atom
  int n_share_atoms = 0;
  int* d_atom_pts = nullptr;
  int* d_atom_off = nullptr;
  double* d_atom_out = nullptr;     // 2 per atom (host-buffer calls)
  std::vector<int> h_host;          // host atom of every uploaded point (reference-layout uploads)
  std::vector<int> h_orig;          // caller's index of every uploaded point (empty: identity)
  int n_orig = 0;                   // points the caller passed (calchem_xc_upload_points*)

  void free_all() {
    void* ptrs[] = {d_shells, d_prims, d_comps, d_prim_f, d_comp_f, d_shell_cf, d_pts,  d_batches, d_cand,  d_cand_loc, d_bao,   d_order,
                    d_P,      d_Pb,    d_V,     d_Vb,   d_rg,      d_red,   d_res,      d_counter, d_slab,
                    d_mixed_ws, d_mixed_slab, d_mol_n, d_mol_off, d_mol_ao_off, d_mol_boff, d_pt_out,
                    d_fxc, d_fxc_m, d_fxc_v, d_ao_cache, d_ao_cache_off, d_ao_cache_ok, d_atom_pts, d_atom_off,
                    d_atom_out};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    if (graph) cudaGraphExecDestroy(graph);
    if (h_stage) cudaFreeHost(h_stage);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
    *this = Entry();
  }
};

struct Built {
  int n = 0;
  double* d_xyzw = nullptr;
  double* d_raw_w = nullptr;
  int* d_host = nullptr;
};

std::mutex g_mu;
std::map<uint64_t, Entry*> g_grids;
std::map<uint64_t, Built*> g_built;
int g_sm_count = -1;

bool device_ok() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return false;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) return false;
  if (g_sm_count < 0) g_sm_count = prop.multiProcessorCount;
  return prop.major == 10 && prop.minor == 3;
}

bool mul_ok(size_t a, size_t b, size_t* out) {
  if (a != 0 && b > SIZE_MAX / a) return false;
  *out = a * b;
  return true;
}

template <typename T>
bool dalloc(T** p, size_t count) {
  if (count == 0) count = 1;
  return cudaMalloc((void**)p, count * sizeof(T)) == cudaSuccess;
}

// Host-side tables derived from a reference-layout upload.
struct HostPlan {
  std::vector<BatchDesc> batches;
  std::vector<int> cand, cand_loc, bao, order;
  int max_m = 0;
  double sum_m2n = 0, sum_m2 = 0;
};

// Validates the reference layout and splits it into <=128-point batches.
int build_host_plan(const AoShellGpu* sh, int n_shells, int n_prims, const AoCompGpu* co, int n_comps,
                    const GridPtGpu* pts, int n_pts, const int* co_off, int n_off, const int* cs, int n_cs, int n_ao,
                    HostPlan& hp) {
  for (int s = 0; s < n_shells; ++s) {
    const AoShellGpu& a = sh[s];
    if (a.n_funcs < 1 || a.n_funcs > 10 || a.n_prims < 1 || a.prim_start < 0 || a.comp_start < 0 ||
        a.ao_offset < 0 || (long long)a.prim_start + a.n_prims > n_prims ||
        (long long)a.comp_start + a.n_funcs > n_comps || (long long)a.ao_offset + a.n_funcs > n_ao)
      return -1;
    for (int c = 0; c < a.n_funcs; ++c) {
      const AoCompGpu& q = co[a.comp_start + c];
      if (q.lx < 0 || q.ly < 0 || q.lz < 0 || q.lx > 3 || q.ly > 3 || q.lz > 3) return -1;
    }
  }
  const int nb = n_off - 1;
  if (co_off[0] < 0) return -1;
  for (int b = 0; b < nb; ++b)
    if (co_off[b + 1] < co_off[b] || co_off[b + 1] > n_cs) return -1;
  for (int i = 0; i < n_cs; ++i)
    if (cs[i] < 0 || cs[i] >= n_shells) return -1;
  // points grouped by non-decreasing batch id
  int prev = -1;
  for (int g = 0; g < n_pts; ++g) {
    const int b = pts[g].batch_id;
    if (b < 0 || b >= nb || b < prev) return -1;
    prev = b;
  }
  int g = 0;
  while (g < n_pts) {
    const int b = pts[g].batch_id;
    int e = g;
    while (e < n_pts && pts[e].batch_id == b) ++e;
    int m = 0;
    const int c0 = co_off[b], c1 = co_off[b + 1];
    for (int s0 = g; s0 < e; s0 += kBlockPts) {
      BatchDesc d{};
      d.pt_start = s0;
      d.n_pts = std::min(kBlockPts, e - s0);
      d.cand_start = (int)hp.cand.size();
      d.n_cand = c1 - c0;
      d.ao_start = (int)hp.bao.size();
      m = 0;
      for (int c = c0; c < c1; ++c) {
        const AoShellGpu& a = sh[cs[c]];
        hp.cand.push_back(cs[c]);
        hp.cand_loc.push_back(m);
        for (int k = 0; k < a.n_funcs; ++k) hp.bao.push_back(a.ao_offset + k);
        m += a.n_funcs;
      }
      d.m = m;
      hp.max_m = std::max(hp.max_m, m);
      hp.sum_m2n += (double)m * m * d.n_pts;
      hp.sum_m2 += (double)m * m;
      hp.batches.push_back(d);
    }
    g = e;
  }
  const int n = (int)hp.batches.size();
  hp.order.resize(n);
  for (int i = 0; i < n; ++i) hp.order[i] = i;
  std::stable_sort(hp.order.begin(), hp.order.end(), [&](int a, int b) {
    const double ca = (double)hp.batches[a].m * hp.batches[a].m * hp.batches[a].n_pts;
    const double cb = (double)hp.batches[b].m * hp.batches[b].m * hp.batches[b].n_pts;
    return ca > cb;
  });
  return 0;
}

// Bytes of the evaluation workspace of an entry (densities, Vxc, split densities, slabs, partials).
size_t workspace_bytes(const Entry& e) {
  const size_t nn = (size_t)e.nn_total;
  size_t t = nn * sizeof(double) * 4;                                           // P, Pb, V, Vb
  t += nn * sizeof(uint2) * 2 + (size_t)e.n_ao * 2 * sizeof(int);              // split densities
  if (e.n_mols == 1) t += (size_t)e.n_pts * 4 * sizeof(double);                // rho / wv staging
  t += (size_t)e.n_batches * 3 * sizeof(double) + (3 * (size_t)e.n_mols + 8) * sizeof(double) + 64;
  t += e.slab_stride * e.n_ctas * sizeof(double);
  t += e.mixed_slab_stride * e.mixed_ctas * sizeof(double);
  return t;
}

// Allocates the evaluation workspace on first use.  Uploads through calchem_xc_upload_points and
// groups defer it, so that grids uploaded only to be grouped hold no workspace.
int ensure_ws(Entry& e) {
  if (e.ws) return 0;
  const size_t nn = (size_t)e.nn_total;
  bool ok = dalloc(&e.d_P, nn) && dalloc(&e.d_Pb, nn) && dalloc(&e.d_V, nn) && dalloc(&e.d_Vb, nn) &&
            (e.n_mols != 1 || dalloc(&e.d_rg, (size_t)e.n_pts * 4)) && dalloc(&e.d_red, (size_t)e.n_batches * 3) &&
            dalloc(&e.d_res, 3 * (size_t)e.n_mols + 8) && dalloc(&e.d_counter, 4) &&
            dalloc(&e.d_slab, e.slab_stride * e.n_ctas) &&
            cudaMalloc(&e.d_mixed_ws, nn * sizeof(uint2) * 2 + (size_t)e.n_ao * 2 * sizeof(int)) == cudaSuccess &&
            dalloc(&e.d_mixed_slab, e.mixed_slab_stride * e.mixed_ctas) &&
            cudaMallocHost((void**)&e.h_stage, (2 * nn + 3 * (size_t)e.n_mols + 8) * sizeof(double)) == cudaSuccess &&
            cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    void* ptrs[] = {e.d_P, e.d_Pb, e.d_V, e.d_Vb, e.d_rg, e.d_red, e.d_res, e.d_counter, e.d_slab, e.d_mixed_ws,
                    e.d_mixed_slab};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    if (e.h_stage) cudaFreeHost(e.h_stage);
    if (e.stream) cudaStreamDestroy(e.stream);
    e.d_P = e.d_Pb = e.d_V = e.d_Vb = e.d_rg = e.d_red = e.d_res = e.d_slab = e.d_mixed_slab = nullptr;
    e.d_counter = nullptr;
    e.d_mixed_ws = nullptr;
    e.h_stage = nullptr;
    e.stream = nullptr;
    return -4;
  }
  e.ws = true;
  return 0;
}

int upload_impl(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                const AoCompGpu* h_comps, int n_comps, const GridPtGpu* h_pts, int n_pts, const int* h_off, int n_off,
                const int* h_cs, int n_cs, int n_ao, uint64_t grid_id, size_t mem_limit, const double* h_w,
                bool eager_ws) {
  if (!h_shells || !h_prims || !h_comps || !h_pts || !h_off || !h_cs || n_shells <= 0 || n_prims <= 0 ||
      n_comps <= 0 || n_pts <= 0 || n_off <= 1 || n_cs <= 0 || n_ao <= 0 || grid_id == 0)
    return -1;
  if (!device_ok()) return -3;
  auto it = g_grids.find(grid_id);
  if (it != g_grids.end()) return (it->second->n_pts == n_pts && it->second->n_ao == n_ao) ? 0 : -2;
  HostPlan hp;
  const int rc = build_host_plan(h_shells, n_shells, n_prims, h_comps, n_comps, h_pts, n_pts, h_off, n_off, h_cs,
                                 n_cs, n_ao, hp);
  if (rc) return rc;
  const int nb = (int)hp.batches.size();
  size_t nn;
  if (!mul_ok((size_t)n_ao, (size_t)n_ao, &nn) || nn > (size_t)1 << 31) return -2;
  const int m_pad = (hp.max_m + 63) / 64 * 64;
  const int per_sm = 1;  // FP64 kernel: 202 registers x 256 threads -> one resident CTA per SM
  const int n_ctas = std::max(1, std::min(nb, g_sm_count * per_sm));
  const size_t slab_stride = (size_t)kPlanes * m_pad * kBlockPts;
  const int mixed_ctas = std::max(1, std::min(nb, g_sm_count * mixed_ctas_per_sm(64)));
  const size_t mixed_stride = mixed_slab_doubles(hp.max_m);
  size_t total = 0;
  total += (size_t)n_shells * sizeof(AoShellGpu) + (size_t)n_prims * sizeof(AoPrimGpu) +
           (size_t)n_comps * sizeof(AoCompGpu);
  total += (size_t)n_pts * 4 * sizeof(double);
  total += (size_t)nb * sizeof(BatchDesc) + (hp.cand.size() * 2 + hp.bao.size() + hp.order.size()) * sizeof(int);
  total += nn * sizeof(double) * 4;           // P, Pb, V, Vb
  total += nn * sizeof(uint2) * 2 + (size_t)n_ao * 2 * sizeof(int);  // split densities (mixed path)
  total += (size_t)n_pts * 4 * sizeof(double);  // rho / wv staging
  total += (size_t)nb * 3 * sizeof(double) + 64;
  total += slab_stride * n_ctas * sizeof(double);
  total += mixed_stride * mixed_ctas * sizeof(double);
  if (total > mem_limit) return -3;

  Entry* e = new Entry;
  e->n_pts = n_pts;
  e->n_ao = n_ao;
  e->n_shells = n_shells;
  e->n_batches = nb;
  e->max_m = hp.max_m;
  e->bytes = total;
  e->mem_limit = mem_limit;
  e->sum_m2n = hp.sum_m2n;
  e->sum_m2 = hp.sum_m2;
  e->n_ctas = n_ctas;
  e->slab_stride = slab_stride;
  e->mixed_ctas = mixed_ctas;
  e->mixed_slab_stride = mixed_stride;
  e->n_prims = n_prims;
  e->n_comps = n_comps;
  e->n_cand = hp.cand.size();
  e->n_bao = hp.bao.size();
  e->n_mols = 1;
  e->max_n = n_ao;
  e->nn_total = (long long)nn;
  e->h_mol_n = {n_ao};
  e->h_mol_off = {0};
  e->h_mol_ao_off = {0, n_ao};
  e->h_mol_boff = {0, nb};
  bool ok = dalloc(&e->d_shells, n_shells) && dalloc(&e->d_prims, n_prims) && dalloc(&e->d_comps, n_comps) &&
            dalloc(&e->d_prim_f, n_prims) && dalloc(&e->d_comp_f, n_comps) && dalloc(&e->d_shell_cf, 3 * (size_t)n_shells) &&
            dalloc(&e->d_pts, (size_t)n_pts * 4) && dalloc(&e->d_batches, nb) && dalloc(&e->d_cand, hp.cand.size()) &&
            dalloc(&e->d_cand_loc, hp.cand_loc.size()) && dalloc(&e->d_bao, hp.bao.size()) &&
            dalloc(&e->d_order, hp.order.size()) && (!eager_ws || ensure_ws(*e) == 0);
  if (!ok) {
    cudaGetLastError();
    e->free_all();
    delete e;
    return -4;
  }
  std::vector<double> soa((size_t)n_pts * 4, 0.0);
  for (int g = 0; g < n_pts; ++g) {
    soa[g] = h_pts[g].x;
    soa[(size_t)n_pts + g] = h_pts[g].y;
    soa[2 * (size_t)n_pts + g] = h_pts[g].z;
    soa[3 * (size_t)n_pts + g] = h_w ? h_w[g] : 0.0;
  }
  e->has_w = h_w != nullptr;
  e->h_host.resize(n_pts);
  for (int g = 0; g < n_pts; ++g) e->h_host[g] = h_pts[g].host_atom;
  // float-pair copies of the basis constants: hi = float(x), lo = float(x - hi)
  std::vector<float4> pf(n_prims);
  for (int i = 0; i < n_prims; ++i) {
    const float ah = (float)h_prims[i].exponent, wh = (float)h_prims[i].weighted_norm;
    pf[i] = make_float4(ah, (float)(h_prims[i].exponent - (double)ah), wh,
                        (float)(h_prims[i].weighted_norm - (double)wh));
  }
  std::vector<float2> cf(n_comps);
  for (int i = 0; i < n_comps; ++i) {
    const float sh = (float)h_comps[i].scale;
    cf[i] = make_float2(sh, (float)(h_comps[i].scale - (double)sh));
  }
  std::vector<float2> scf(3 * (size_t)n_shells);
  for (int i = 0; i < n_shells; ++i)
    for (int k = 0; k < 3; ++k) {
      const float hi = (float)h_shells[i].center[k];
      scf[3 * (size_t)i + k] = make_float2(hi, (float)(h_shells[i].center[k] - (double)hi));
    }
  ok = cudaMemcpy(e->d_prim_f, pf.data(), n_prims * sizeof(float4), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_shell_cf, scf.data(), scf.size() * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_comp_f, cf.data(), n_comps * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_shells, h_shells, n_shells * sizeof(AoShellGpu), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_prims, h_prims, n_prims * sizeof(AoPrimGpu), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_comps, h_comps, n_comps * sizeof(AoCompGpu), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_pts, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_batches, hp.batches.data(), nb * sizeof(BatchDesc), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_cand, hp.cand.data(), hp.cand.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_cand_loc, hp.cand_loc.data(), hp.cand_loc.size() * sizeof(int), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(e->d_bao, hp.bao.data(), hp.bao.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(e->d_order, hp.order.data(), hp.order.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    e->free_all();
    delete e;
    return -5;
  }
  g_grids[grid_id] = e;
  return 0;
}

DevGrid dev_grid(const Entry& e) {
  DevGrid G{};
  G.n_pts = e.n_pts;
  G.n_ao = e.n_ao;
  G.n_shells = e.n_shells;
  G.n_batches = e.n_batches;
  G.shells = e.d_shells;
  G.prims = e.d_prims;
  G.comps = e.d_comps;
  G.px = e.d_pts;
  G.py = e.d_pts + e.n_pts;
  G.pz = e.d_pts + 2 * (size_t)e.n_pts;
  G.pw = e.d_pts + 3 * (size_t)e.n_pts;
  G.batches = e.d_batches;
  G.cand_shells = e.d_cand;
  G.cand_loc = e.d_cand_loc;
  G.batch_ao = e.d_bao;
  G.order = e.d_order;
  G.prim_f = e.d_prim_f;
  G.comp_f = e.d_comp_f;
  G.shell_cf = e.d_shell_cf;
  G.mol_n = e.d_mol_n;  // nullptr unless the entry is a group
  G.mol_off = e.d_mol_off;
  G.mol_ao_off = e.d_mol_ao_off;
  G.nn_total = e.nn_total;
  G.n_total = e.n_ao;
  return G;
}

// Enqueues one evaluation.  Pa/Pb/Va/Vb are device pointers; result gets (exc, n_a[, n_b]).
// The AO cache's byte cap: CALCHEM_MAX_AO_GRID_BYTES when set (CalChem's variable for the cap of
// its cache of per-batch AO values and gradients, vxc.rs:600-640), else 32 GiB: CalChem's default
// of 2560 MiB sizes host memory, and the cache here lives in the GPU's HBM.
size_t ao_cache_cap() {
  const char* v = std::getenv("CALCHEM_MAX_AO_GRID_BYTES");
  if (v && *v) {
    char* end = nullptr;
    const unsigned long long x = std::strtoull(v, &end, 10);
    if (end && *end == '\0') return (size_t)x;
  }
  return (size_t)32 << 30;
}

void ao_cache_free(Entry& e) {
  if (e.d_ao_cache) cudaFree(e.d_ao_cache);
  if (e.d_ao_cache_off) cudaFree(e.d_ao_cache_off);
  if (e.d_ao_cache_ok) cudaFree(e.d_ao_cache_ok);
  e.d_ao_cache = nullptr;
  e.d_ao_cache_off = nullptr;
  e.d_ao_cache_ok = nullptr;
  e.ao_cache_bytes = 0;
}

// Decides and allocates the AO cache on the first tensor-core evaluation (not inside a stream
// capture: callers that capture decide first).  The per-batch AO values and gradients depend only on
// the grid and basis, so CalChem's engine computes them once per geometry and reuses them every
// SCF iteration (vxc.rs:386-394, 600-716); here the cache also holds the packed GEMM1 operand and
// the row exponents.  Off when the blocks exceed the cap or the free device memory (minus 1 GiB).
void ao_cache_decide(Entry& e) {
  if (e.ao_cache_state != 0) return;
  e.ao_cache_state = 1;
  std::vector<BatchDesc> hb(e.n_batches);
  if (cudaMemcpy(hb.data(), e.d_batches, hb.size() * sizeof(BatchDesc), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  size_t free_b = 0, tot_b = 0;
  if (cudaMemGetInfo(&free_b, &tot_b) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  // the cache's limit: the cap, the grid's budget and the free device memory less 1 GiB; batches (in
  // batch order) whose blocks fit within it get one (offset -1: evaluated every time)
  const size_t reserve = (size_t)1 << 30;
  const size_t budget = e.mem_limit > e.bytes ? e.mem_limit - e.bytes : 0;  // within the grid's budget
  const size_t limit = std::min({ao_cache_cap(), budget, free_b > reserve ? free_b - reserve : (size_t)0});
  std::vector<long long> off(e.n_batches, -1);
  size_t total = 0;
  for (int b = 0; b < e.n_batches; ++b) {
    const size_t bb = ao_cache_block_bytes(hb[b].m);
    if (total + bb > limit) continue;
    off[b] = (long long)total;
    total += bb;
  }
  if (total == 0) return;
  const bool ok = cudaMalloc(&e.d_ao_cache, total) == cudaSuccess &&
                  cudaMalloc(&e.d_ao_cache_off, off.size() * sizeof(long long)) == cudaSuccess &&
                  cudaMalloc(&e.d_ao_cache_ok, (size_t)e.n_batches * sizeof(int)) == cudaSuccess &&
                  cudaMemcpy(e.d_ao_cache_off, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice) ==
                      cudaSuccess &&
                  cudaMemset(e.d_ao_cache_ok, 0, (size_t)e.n_batches * sizeof(int)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    ao_cache_free(e);
    return;
  }
  e.ao_cache_bytes = total;
  e.ao_cache_state = 2;
}

// Tensor-core CTAs to launch for the grid's tile (never more than the workspace has slabs for).
int mixed_launch_ctas(const Entry& e) {
  return std::max(1, std::min(e.mixed_ctas, g_sm_count * mixed_ctas_per_sm(e.tile_n)));
}

// shares_only (closed shell, with point_out): the per-point shares, Exc and Nelec without the Vxc
// contraction; Va is not touched.
int enqueue_eval(Entry& e, int mode, int xc, int precision, const double* Pa, const double* Pb, double* Va,
                 double* Vb, const double* wv, double* rho_out, double* result, cudaStream_t st,
                 double* point_out = nullptr, bool shares_only = false) {
  const size_t nn = (size_t)e.nn_total;
  int launches = 0;
  if (mode != kModeRho && !shares_only) {
    if (cudaMemsetAsync(Va, 0, nn * sizeof(double), st) != cudaSuccess) return -5;
    if (mode == kModeUks && cudaMemsetAsync(Vb, 0, nn * sizeof(double), st) != cudaSuccess) return -5;
  }
  if (cudaMemsetAsync(e.d_counter, 0, 4 * sizeof(int), st) != cudaSuccess) return -5;  // queues + status
  EvalArgs A{};
  A.mode = mode;
  A.xc = xc;
  A.Pa = Pa;
  A.Pb = Pb;
  A.Va = Va;
  A.Vb = Vb;
  A.rho_out = rho_out;
  A.wv_in = wv;
  A.batch_red = e.d_red;
  A.counter = e.d_counter;
  A.max_m = e.max_m;
  A.point_out = point_out;
  A.shares_only = shares_only ? 1 : 0;
  const DevGrid G = dev_grid(e);
  cudaError_t err;
  const bool prof = e.profiling && e.ev0 && e.ev1;
  if (precision == CALCHEM_XC_MIXED) {
    // packed fixed-point densities: [alpha n^2][beta n^2] uint2, then row exponents [alpha n][beta n]
    uint2* pk = reinterpret_cast<uint2*>(e.d_mixed_ws);
    int* fx = reinterpret_cast<int*>(pk + 2 * nn);
    if (launch_mixed_prepare(Pa, e.n_ao, e.d_mol_n, e.d_mol_off, e.d_mol_ao_off, e.n_mols, pk, fx, st) !=
        cudaSuccess)
      return -5;
    ++launches;
    if (mode == kModeUks) {
      if (launch_mixed_prepare(Pb, e.n_ao, e.d_mol_n, e.d_mol_off, e.d_mol_ao_off, e.n_mols, pk + nn, fx + e.n_ao,
                               st) != cudaSuccess)
        return -5;
      ++launches;
    }
    A.slab = e.d_mixed_slab;
    A.slab_stride = e.mixed_slab_stride;
    A.Pa = (const double*)e.d_mixed_ws;  // the tensor-core kernel reads the split copies
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) ao_cache_decide(e);
    if (e.ao_cache_state == 2) {
      A.ao_cache = e.d_ao_cache;
      A.ao_cache_off = e.d_ao_cache_off;
      A.ao_cache_ok = e.d_ao_cache_ok;
    }
    A.tile_n = e.tile_n;
    if (prof) cudaEventRecord(e.ev0, st);
    err = launch_mixed(G, A, mixed_launch_ctas(e), st);
    if (prof) cudaEventRecord(e.ev1, st);
  } else {
    A.slab = e.d_slab;
    A.slab_stride = e.slab_stride;
    if (prof) cudaEventRecord(e.ev0, st);
    err = launch_fp64(G, A, e.n_ctas, st);
    if (prof) cudaEventRecord(e.ev1, st);
  }
  if (err != cudaSuccess) return -5;
  ++launches;
  if (mode == kModeRks || mode == kModeUks) {
    if (launch_reduce(e.d_red, e.n_batches, e.d_mol_boff, e.n_mols, result, mode == kModeRks ? 2 : 3, st) !=
        cudaSuccess)
      return -5;
    const int from_upper = precision == CALCHEM_XC_MIXED ? 1 : 0;
    ++launches;
    if (!shares_only) {
      if (launch_mirror(Va, e.max_n, e.d_mol_n, e.d_mol_off, e.n_mols, from_upper, st) != cudaSuccess) return -5;
      ++launches;
    }
    if (mode == kModeUks) {
      if (launch_mirror(Vb, e.max_n, e.d_mol_n, e.d_mol_off, e.n_mols, from_upper, st) != cudaSuccess) return -5;
      ++launches;
    }
  }
  e.last_launches = launches;
  return 0;
}

// TD-DFT kernel contraction of n_trials symmetric matrices d_m (each n x n) into d_v.
int enqueue_fxc(Entry& e, int triplet, const double* d_m, int n_trials, double* d_v, cudaStream_t st) {
  const size_t nn = (size_t)e.n_ao * e.n_ao;
  if (cudaMemsetAsync(d_v, 0, nn * n_trials * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(e.d_counter, 0, 4 * sizeof(int), st) != cudaSuccess)
    return -5;
  EvalArgs A{};
  A.mode = kModeFxc;
  A.xc = e.fxc_code;
  A.Pa = d_m;
  A.Va = d_v;
  A.n_trials = n_trials;
  A.triplet = triplet ? 1 : 0;
  A.fxc_coef = e.d_fxc;
  A.batch_red = e.d_red;
  A.counter = e.d_counter;
  A.max_m = e.max_m;
  A.slab = e.d_slab;
  A.slab_stride = e.slab_stride;
  if (launch_fp64(dev_grid(e), A, e.n_ctas, st) != cudaSuccess) return -5;
  for (int t = 0; t < n_trials; ++t)
    if (launch_mirror(d_v + t * nn, e.n_ao, 0, st) != cudaSuccess) return -5;
  e.last_launches = 1 + n_trials;
  return 0;
}

// The same contraction in the tensor-core form: one launch per trial matrix, each the closed-shell
// pipeline with M_b in place of D and the kernel coefficients in place of the functional; the AO cache
// (filled by the first launch) serves every trial.  The upper triangles the kernel adds are mirrored.
int enqueue_fxc_mixed(Entry& e, int triplet, const double* d_m, int n_trials, double* d_v, cudaStream_t st) {
  const size_t nn = (size_t)e.n_ao * e.n_ao;
  if (mixed_set_attributes() != cudaSuccess) return -5;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) ao_cache_decide(e);
  uint2* pk = reinterpret_cast<uint2*>(e.d_mixed_ws);
  int* fx = reinterpret_cast<int*>(pk + 2 * nn);
  const DevGrid G = dev_grid(e);
  for (int t = 0; t < n_trials; ++t) {
    double* v = d_v + t * nn;
    if (cudaMemsetAsync(v, 0, nn * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(e.d_counter, 0, 4 * sizeof(int), st) != cudaSuccess)
      return -5;
    if (launch_mixed_prepare(d_m + t * nn, e.n_ao, nullptr, nullptr, nullptr, 1, pk, fx, st) != cudaSuccess)
      return -5;
    EvalArgs A{};
    A.mode = kModeFxc;
    A.Pa = (const double*)e.d_mixed_ws;
    A.Va = v;
    A.fxc_coef = e.d_fxc;
    A.triplet = triplet ? 1 : 0;
    A.n_trials = 1;
    A.batch_red = e.d_red;
    A.counter = e.d_counter;
    A.max_m = e.max_m;
    A.slab = e.d_mixed_slab;
    A.slab_stride = e.mixed_slab_stride;
    if (e.ao_cache_state == 2) {
      A.ao_cache = e.d_ao_cache;
      A.ao_cache_off = e.d_ao_cache_off;
      A.ao_cache_ok = e.d_ao_cache_ok;
    }
    A.tile_n = e.tile_n;
    if (launch_mixed(G, A, mixed_launch_ctas(e), st) != cudaSuccess) return -5;
    if (launch_mirror(v, e.n_ao, 1, st) != cudaSuccess) return -5;
  }
  e.last_launches = 3 * n_trials;
  return 0;
}

bool valid_xc(int xc) { return xc >= 0 && xc <= 8; }
bool valid_prec(int p, int mode) {
  if (p == CALCHEM_XC_FP64) return true;
  return p == CALCHEM_XC_MIXED && mixed_supported(mode);
}

Entry* find(uint64_t id) {
  auto it = g_grids.find(id);
  return it == g_grids.end() ? nullptr : it->second;
}

}  // namespace

namespace {
// Expands the radial shells into points on the device, Becke weights, compaction (caller holds g_mu).
int grid_build_impl(int n_atoms, const int* z, const double* xyz_bohr, const std::vector<RadialShell>& rs,
                    long long n_raw, uint64_t grid_handle, int* n_pts_out) {
  std::vector<double> inv_r, a_ij;
  becke_tables(n_atoms, z, xyz_bohr, inv_r, a_ij);
  const LebedevTables& T = lebedev_tables();
  const int ns = (int)rs.size();
  if (ns == 0) return -1;
  std::vector<RadialShellDev> rsd(ns);
  for (int i = 0; i < ns; ++i) rsd[i] = {rs[i].atom, rs[i].leb_offset, rs[i].n_ang, 0, rs[i].r, rs[i].w_rad,
                                         rs[i].raw_start};
  GridBuildArgs a{};
  double *d_xyz = nullptr, *d_inv = nullptr, *d_aij = nullptr, *d_leb = nullptr, *d_raw = nullptr, *d_raww = nullptr;
  RadialShellDev* d_rs = nullptr;
  unsigned char* d_flags = nullptr;
  int* d_counts = nullptr;
  long long* d_off = nullptr;
  auto cleanup = [&]() {
    void* p[] = {d_xyz, d_inv, d_aij, d_leb, d_raw, d_raww, d_rs, d_flags, d_counts, d_off};
    for (void* q : p)
      if (q) cudaFree(q);
  };
  bool ok = dalloc(&d_xyz, 3 * (size_t)n_atoms) && dalloc(&d_inv, inv_r.size()) && dalloc(&d_aij, a_ij.size()) &&
            dalloc(&d_leb, T.xyzw.size()) && dalloc(&d_rs, ns) && dalloc(&d_raw, 4 * (size_t)n_raw) &&
            dalloc(&d_raww, (size_t)n_raw) && dalloc(&d_flags, (size_t)n_raw) && dalloc(&d_counts, ns) &&
            dalloc(&d_off, (size_t)ns + 1);
  if (!ok) {
    cudaGetLastError();
    cleanup();
    return -4;
  }
  ok = cudaMemcpy(d_xyz, xyz_bohr, 3 * n_atoms * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(d_inv, inv_r.data(), inv_r.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(d_aij, a_ij.data(), a_ij.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(d_leb, T.xyzw.data(), T.xyzw.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(d_rs, rsd.data(), ns * sizeof(RadialShellDev), cudaMemcpyHostToDevice) == cudaSuccess;
  a.n_atoms = n_atoms;
  a.xyz = d_xyz;
  a.inv_r = d_inv;
  a.a_ij = d_aij;
  a.lebedev = d_leb;
  a.shells = d_rs;
  a.raw = d_raw;
  a.raw_w = d_raww;
  a.flags = d_flags;
  a.counts = d_counts;
  ok = ok && launch_grid_expand(a, ns, 0) == cudaSuccess && launch_grid_scan(d_counts, ns, d_off, 0) == cudaSuccess;
  long long n_keep = 0;
  ok = ok && cudaMemcpy(&n_keep, d_off + ns, sizeof(long long), cudaMemcpyDeviceToHost) == cudaSuccess;
  if (!ok || n_keep > 0x7fffffffLL) {
    cudaGetLastError();
    cleanup();
    return ok ? -2 : -5;
  }
  Built* b = new Built;
  b->n = (int)n_keep;
  if (!(dalloc(&b->d_xyzw, 4 * (size_t)n_keep) && dalloc(&b->d_raw_w, (size_t)n_keep) &&
        dalloc(&b->d_host, (size_t)n_keep))) {
    cudaGetLastError();
    if (b->d_xyzw) cudaFree(b->d_xyzw);
    if (b->d_raw_w) cudaFree(b->d_raw_w);
    if (b->d_host) cudaFree(b->d_host);
    delete b;
    cleanup();
    return -4;
  }
  a.out_xyzw = b->d_xyzw;
  a.out_raw_w = b->d_raw_w;
  a.out_host = b->d_host;
  ok = launch_grid_compact(a, d_off, ns, 0) == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  cleanup();
  if (!ok) {
    cudaGetLastError();
    cudaFree(b->d_xyzw);
    cudaFree(b->d_raw_w);
    cudaFree(b->d_host);
    delete b;
    return -5;
  }
  g_built[grid_handle] = b;
  *n_pts_out = b->n;
  return 0;
}

// Device buffers of one gradient evaluation, freed on every return path.
struct GradBufs {
  double *pa = nullptr, *pb = nullptr, *wxc = nullptr, *raw = nullptr, *xyz = nullptr, *inv = nullptr,
         *aij = nullptr, *part = nullptr, *slab = nullptr, *grad = nullptr;
  int *host = nullptr, *ao_atom = nullptr, *counter = nullptr;
  int2* pairs = nullptr;
  float2* pair_df = nullptr;
  double *fx = nullptr, *part2 = nullptr;  // tensor-core form: per-point f, weight-derivative rows
  ~GradBufs() {
    void* ptrs[] = {pa, pb, wxc, raw, xyz, inv, aij, part, slab, grad, host, ao_atom, counter, pairs, pair_df,
                    fx, part2};
    for (void* p : ptrs)
      if (p) cudaFree(p);
  }
};

// Runs the gradient kernel on an uploaded single-molecule grid.  xc >= 0: fused form (h_raw and
// the atoms' z / xyz used); xc < 0: drop-in form with h_wxc.  host_up: host atom per uploaded
// point.  Returns 0, -1 (arguments), -3 (memory limit), -4 (allocation) or -5 (CUDA).
int gradient_run(Entry& e, int xc, int precision, bool closed, const double* h_pa, const double* h_pb,
                 const double* h_wxc, const double* h_raw, const int* host_up, int n_atoms, const int* z,
                 const double* xyz, double* h_grad, size_t mem_limit) {
  const int n = e.n_ao;
  const bool mixed = precision == CALCHEM_XC_MIXED;
  if (mixed && (xc < 0 || e.max_m > grad_mixed_max_m())) return -2;
  std::vector<AoShellGpu> sh(e.n_shells);
  if (cudaMemcpy(sh.data(), e.d_shells, sh.size() * sizeof(AoShellGpu), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -5;
  std::vector<int> ao_atom(n, 0);
  for (const AoShellGpu& a : sh) {
    if (a.atom_index < 0 || a.atom_index >= n_atoms) return -1;
    for (int c = 0; c < a.n_funcs; ++c) ao_atom[a.ao_offset + c] = a.atom_index;
  }
  for (int g = 0; g < e.n_pts; ++g)
    if (host_up[g] < 0 || host_up[g] >= n_atoms) return -1;
  std::vector<double> inv_r, a_ij;
  std::vector<int2> pairs;
  std::vector<float2> pair_df;  // per ordered pair: 1 / R, a, (R_a - R_b) / R as float pairs
  if (xc >= 0) {
    becke_tables(n_atoms, z, xyz, inv_r, a_ij);
    for (int c = 0; c < n_atoms; ++c)
      for (int d = c + 1; d < n_atoms; ++d) pairs.push_back(make_int2(c, d));
    auto fpair = [](double v) {
      const float hi = (float)v;
      return make_float2(hi, (float)(v - (double)hi));
    };
    pair_df.resize((size_t)n_atoms * n_atoms * 5);
    for (int a = 0; a < n_atoms; ++a)
      for (int b = 0; b < n_atoms; ++b) {
        const size_t k = (size_t)a * n_atoms + b;
        const double inv = inv_r[k];
        pair_df[5 * k] = fpair(inv);
        pair_df[5 * k + 1] = fpair(a_ij[k]);
        for (int q = 0; q < 3; ++q) pair_df[5 * k + 2 + q] = fpair((xyz[3 * a + q] - xyz[3 * b + q]) * inv);
      }
  }
  const size_t nn = (size_t)n * n, na3 = 3 * (size_t)n_atoms;
  const size_t slab_stride = mixed ? grad_mixed_slab_doubles(e.max_m, n_atoms) : grad_slab_doubles(e.max_m, n_atoms);
  // persistent CTAs (one per SM for FP64, two for the tensor-core form), fewer when the per-CTA
  // scratch (AO planes and the warps' atom-pair tables) would take more than half of the free memory
  int n_ctas = std::max(1, std::min(e.n_batches, g_sm_count * (mixed ? 2 : 1)));
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    const size_t fit = free_b / 2 / (slab_stride * sizeof(double));
    n_ctas = (int)std::max<size_t>(1, std::min<size_t>(n_ctas, fit));
  }
  size_t total = nn * sizeof(double) * (closed ? 1 : 2) + (size_t)e.n_pts * (xc < 0 ? 8 : 1) * sizeof(double) +
                 (size_t)e.n_pts * sizeof(int) + (size_t)n * sizeof(int) + (inv_r.size() * 2 + na3) * sizeof(double) +
                 ((size_t)e.n_batches + 1) * na3 * sizeof(double) + slab_stride * n_ctas * sizeof(double) +
                 pairs.size() * sizeof(int2) + pair_df.size() * sizeof(float2) + 64;
  if (total > mem_limit) return -3;
  GradBufs B;
  bool ok = dalloc(&B.pa, nn) && (closed || dalloc(&B.pb, nn)) && dalloc(&B.host, e.n_pts) &&
            dalloc(&B.ao_atom, n) && dalloc(&B.part, (size_t)e.n_batches * na3) && dalloc(&B.grad, na3) &&
            dalloc(&B.slab, slab_stride * n_ctas) && dalloc(&B.counter, 2) &&
            (xc < 0 ? dalloc(&B.wxc, (size_t)e.n_pts * 8)
                    : dalloc(&B.raw, e.n_pts) && dalloc(&B.xyz, na3) && dalloc(&B.inv, inv_r.size()) &&
                          dalloc(&B.aij, a_ij.size()) && dalloc(&B.pairs, pairs.size()) &&
                          dalloc(&B.pair_df, pair_df.size()));
  // the tensor-core form runs the weight derivative as its own kernel when its tables fit
  const bool becke_apart = mixed && xc >= 0 && becke_kernel_fits(n_atoms);
  const int n_bk = becke_apart ? becke_kernel_ctas(e.n_pts) : 0;
  if (ok && becke_apart) ok = dalloc(&B.fx, e.n_pts) && dalloc(&B.part2, (size_t)n_bk * na3);
  if (!ok) {
    cudaGetLastError();
    return -4;
  }
  cudaStream_t st = e.stream;
  ok = cudaMemcpyAsync(B.pa, h_pa, nn * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
       (closed || cudaMemcpyAsync(B.pb, h_pb, nn * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess) &&
       cudaMemcpyAsync(B.host, host_up, (size_t)e.n_pts * sizeof(int), cudaMemcpyHostToDevice, st) == cudaSuccess &&
       cudaMemcpyAsync(B.ao_atom, ao_atom.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st) ==
           cudaSuccess &&
       cudaMemsetAsync(B.counter, 0, 2 * sizeof(int), st) == cudaSuccess &&
       (!mixed || cudaMemsetAsync(B.part, 0, (size_t)e.n_batches * na3 * sizeof(double), st) == cudaSuccess) &&
       (!becke_apart || cudaMemsetAsync(B.fx, 0, (size_t)e.n_pts * sizeof(double), st) == cudaSuccess);
  if (ok && xc < 0)
    ok = cudaMemcpyAsync(B.wxc, h_wxc, (size_t)e.n_pts * 8 * sizeof(double), cudaMemcpyHostToDevice, st) ==
         cudaSuccess;
  if (ok && xc >= 0)
    ok = cudaMemcpyAsync(B.raw, h_raw, (size_t)e.n_pts * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
         cudaMemcpyAsync(B.xyz, xyz, na3 * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess &&
         cudaMemcpyAsync(B.inv, inv_r.data(), inv_r.size() * sizeof(double), cudaMemcpyHostToDevice, st) ==
             cudaSuccess &&
         cudaMemcpyAsync(B.aij, a_ij.data(), a_ij.size() * sizeof(double), cudaMemcpyHostToDevice, st) ==
             cudaSuccess &&
         (pairs.empty() || cudaMemcpyAsync(B.pairs, pairs.data(), pairs.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                           st) == cudaSuccess) &&
         cudaMemcpyAsync(B.pair_df, pair_df.data(), pair_df.size() * sizeof(float2), cudaMemcpyHostToDevice, st) ==
             cudaSuccess;
  if (!ok) return -5;
  GradArgs A{};
  A.xc = xc;
  A.closed = closed ? 1 : 0;
  A.Pa = B.pa;
  A.Pb = closed ? B.pa : B.pb;
  A.wxc = B.wxc;
  A.raw_w = B.raw;
  A.host = B.host;
  A.ao_atom = B.ao_atom;
  A.xyz = B.xyz;
  A.inv_r = B.inv;
  A.a_ij = B.aij;
  A.pairs = B.pairs;
  A.n_pairs = (int)pairs.size();
  A.pair_df = B.pair_df;
  A.fx_out = B.fx;
  A.n_atoms = n_atoms;
  A.max_m = e.max_m;
  A.part = B.part;
  A.counter = B.counter;
  A.slab = B.slab;
  A.slab_stride = slab_stride;
  int launches = 0;
  if (e.profiling) cudaEventRecord(e.ev0, st);
  if (mixed) {
    // split copies of the spin densities for the tensor-core contractions (alpha, then beta)
    uint2* pk = reinterpret_cast<uint2*>(e.d_mixed_ws);
    int* fx = reinterpret_cast<int*>(pk + 2 * nn);
    if (launch_mixed_prepare(B.pa, n, nullptr, nullptr, nullptr, 1, pk, fx, st) != cudaSuccess) return -5;
    ++launches;
    if (!closed) {
      if (launch_mixed_prepare(B.pb, n, nullptr, nullptr, nullptr, 1, pk + nn, fx + n, st) != cudaSuccess) return -5;
      ++launches;
    }
    A.Pa = reinterpret_cast<const double*>(e.d_mixed_ws);
    A.Pb = nullptr;
    if (launch_xc_grad_mixed(dev_grid(e), A, n_ctas, B.counter + 1, st) != cudaSuccess) return -5;
    if (becke_apart) {
      if (launch_becke_mixed(dev_grid(e), A, B.fx, B.part2, st) != cudaSuccess) return -5;
      ++launches;
    }
  } else if (launch_xc_grad(dev_grid(e), A, n_ctas, st) != cudaSuccess) {
    return -5;
  }
  if (launch_grad_reduce(B.part, e.n_batches, n_atoms, B.grad, st) != cudaSuccess) return -5;
  launches += 2;
  if (becke_apart) {
    if (launch_grad_accumulate(B.part2, n_bk, n_atoms, B.grad, st) != cudaSuccess) return -5;
    ++launches;
  }
  if (e.profiling) cudaEventRecord(e.ev1, st);
  e.last_launches = launches;
  int status = 0;
  if (cudaMemcpyAsync(h_grad, B.grad, na3 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&status, B.counter + 1, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return -5;
  return status ? -7 : 0;
}

}  // namespace

extern "C" {

int calchem_cuda_is_available(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return device_ok() ? 1 : 0;
}

const char* calchem_xc_version(void) { return "calchem-xc-gb300 0.1 (sm_103a)"; }

int calchem_cuda_vxc_upload_grid(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                                 const AoCompGpu* h_comps, int n_comps, const GridPtGpu* h_pts, int n_pts,
                                 const int* h_cand_offsets, int n_cand_offsets, const int* h_cand_shells,
                                 int n_cand_shells, int n_ao, uint64_t grid_id, size_t memory_limit_bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  return upload_impl(h_shells, n_shells, h_prims, n_prims, h_comps, n_comps, h_pts, n_pts, h_cand_offsets,
                     n_cand_offsets, h_cand_shells, n_cand_shells, n_ao, grid_id, memory_limit_bytes, nullptr, true);
}

int calchem_cuda_vxc_eval_rho(uint64_t grid_id, const double* h_p_mat, double* h_rho_grad_out, int n_pts, int n_ao) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_p_mat || !h_rho_grad_out || n_pts <= 0 || n_ao <= 0 || grid_id == 0) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || e->n_pts != n_pts || e->n_ao != n_ao) return -2;
  if (int rc0 = ensure_ws(*e)) return rc0;
  const size_t nn = (size_t)n_ao * n_ao;
  std::memcpy(e->h_stage, h_p_mat, nn * sizeof(double));
  if (cudaMemcpyAsync(e->d_P, e->h_stage, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) != cudaSuccess)
    return -5;
  int rc = enqueue_eval(*e, kModeRho, 0, CALCHEM_XC_FP64, e->d_P, nullptr, nullptr, nullptr, nullptr, e->d_rg,
                        nullptr, e->stream);
  if (rc) return rc;
  if (cudaMemcpyAsync(h_rho_grad_out, e->d_rg, (size_t)n_pts * 4 * sizeof(double), cudaMemcpyDeviceToHost,
                      e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  return 0;
}

int calchem_cuda_vxc_accum(uint64_t grid_id, const double* h_wv_in, double* h_vxc_out, int n_pts, int n_ao) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_wv_in || !h_vxc_out || n_pts <= 0 || n_ao <= 0 || grid_id == 0) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || e->n_pts != n_pts || e->n_ao != n_ao) return -2;
  if (int rc0 = ensure_ws(*e)) return rc0;
  const size_t nn = (size_t)n_ao * n_ao;
  if (cudaMemcpyAsync(e->d_rg, h_wv_in, (size_t)n_pts * 4 * sizeof(double), cudaMemcpyHostToDevice, e->stream) !=
      cudaSuccess)
    return -5;
  int rc = enqueue_eval(*e, kModeAccum, 0, CALCHEM_XC_FP64, nullptr, nullptr, e->d_V, nullptr, e->d_rg, nullptr,
                        nullptr, e->stream);
  if (rc) return rc;
  if (cudaMemcpyAsync(e->h_stage, e->d_V, nn * sizeof(double), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  std::memcpy(h_vxc_out, e->h_stage, nn * sizeof(double));
  return 0;
}

int calchem_cuda_vxc_grad_force(uint64_t grid_id, const double* h_pa, const double* h_pb, int is_rks,
                                const double* h_wxc_in, double* h_grad_out, int n_pts, int n_ao, int n_atoms,
                                size_t memory_limit_bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (grid_id == 0 || !h_pa || (!is_rks && !h_pb) || !h_wxc_in || !h_grad_out || n_pts <= 0 || n_ao <= 0 ||
      n_atoms <= 0 || n_atoms > grad_max_atoms())
    return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || e->n_pts != n_pts || e->n_ao != n_ao || (int)e->h_host.size() != n_pts) return -2;
  if (int rc0 = ensure_ws(*e)) return rc0;
  return gradient_run(*e, -1, CALCHEM_XC_FP64, is_rks != 0, h_pa, h_pb, h_wxc_in, nullptr, e->h_host.data(), n_atoms,
                      nullptr,
                      nullptr, h_grad_out, memory_limit_bytes ? memory_limit_bytes : SIZE_MAX);
}

int calchem_cuda_vxc_release(uint64_t grid_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (grid_id != 0) {
    auto it = g_grids.find(grid_id);
    if (it != g_grids.end()) {
      if (it->second->stream) cudaStreamSynchronize(it->second->stream);
      it->second->free_all();
      delete it->second;
      g_grids.erase(it);
    }
  }
  return 0;
}

int calchem_xc_prepare_shells(int n_shells, const int* l, const int* atom_index, const double* centers,
                              const int* n_prims, const double* exponents, const double* raw_coefs,
                              AoShellGpu* shells_out, AoPrimGpu* prims_out, AoCompGpu* comps_out, int* n_ao_out) {
  if (n_shells <= 0 || !l || !atom_index || !centers || !n_prims || !exponents || !raw_coefs || !shells_out ||
      !prims_out || !comps_out || !n_ao_out)
    return -1;
  return prepare_shells(n_shells, l, atom_index, centers, n_prims, exponents, raw_coefs, shells_out, prims_out,
                        comps_out, n_ao_out);
}

int calchem_xc_overlap(const AoShellGpu* shells, int n_shells, const AoPrimGpu* prims, const AoCompGpu* comps,
                       int n_ao, double* s_out) {
  if (!shells || !prims || !comps || !s_out || n_shells <= 0 || n_ao <= 0) return -1;
  overlap_matrix(shells, n_shells, prims, comps, n_ao, s_out);
  return 0;
}

int calchem_xc_grid_build(int n_atoms, const int* z, const double* xyz_bohr, int level, int radial_min,
                          uint64_t grid_handle, int* n_pts_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (n_atoms <= 0 || !z || !xyz_bohr || level < 0 || level > 3 || radial_min < 0 || radial_min > 4096 ||
      grid_handle == 0 || !n_pts_out)
    return -1;
  for (int a = 0; a < n_atoms; ++a)
    if (z[a] < 1 || z[a] > 86 || !std::isfinite(xyz_bohr[3 * a]) || !std::isfinite(xyz_bohr[3 * a + 1]) ||
        !std::isfinite(xyz_bohr[3 * a + 2]))
      return -1;
  if (!device_ok()) return -3;
  if (g_built.count(grid_handle)) return -2;
  std::vector<RadialShell> rs;
  long long n_raw = 0;
  radial_shells(n_atoms, z, level, radial_min, rs, &n_raw);
  return grid_build_impl(n_atoms, z, xyz_bohr, rs, n_raw, grid_handle, n_pts_out);
}

int calchem_xc_grid_build_atoms(int n_atoms, const int* z, const double* xyz_bohr, const int* n_rad,
                                const int* region_leb, const double* x_max, uint64_t grid_handle, int* n_pts_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (n_atoms <= 0 || !z || !xyz_bohr || !n_rad || !region_leb || !x_max || grid_handle == 0 || !n_pts_out)
    return -1;
  for (int a = 0; a < n_atoms; ++a) {
    if (z[a] < 1 || z[a] > 86 || !std::isfinite(xyz_bohr[3 * a]) || !std::isfinite(xyz_bohr[3 * a + 1]) ||
        !std::isfinite(xyz_bohr[3 * a + 2]) || n_rad[a] > 4096 || !(x_max[a] == x_max[a]))
      return -1;
    for (int k = 0; k < 5; ++k)
      if (region_leb[5 * a + k] > 0 && lebedev_index(region_leb[5 * a + k]) < 0) return -1;
  }
  if (!device_ok()) return -3;
  if (g_built.count(grid_handle)) return -2;
  std::vector<RadialShell> rs;
  long long n_raw = 0;
  radial_shells_atoms(n_atoms, z, n_rad, region_leb, x_max, rs, &n_raw);
  return grid_build_impl(n_atoms, z, xyz_bohr, rs, n_raw, grid_handle, n_pts_out);
}

int calchem_xc_grid_fetch(uint64_t grid_handle, double* xyzw, double* raw_w, int* host_atom) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_built.find(grid_handle);
  if (it == g_built.end()) return -2;
  if (!xyzw) return -1;
  const Built& b = *it->second;
  if (b.n == 0) return 0;
  if (cudaMemcpy(xyzw, b.d_xyzw, 4 * (size_t)b.n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return -5;
  if (raw_w && cudaMemcpy(raw_w, b.d_raw_w, (size_t)b.n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -5;
  if (host_atom && cudaMemcpy(host_atom, b.d_host, (size_t)b.n * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -5;
  return 0;
}

int calchem_xc_grid_release(uint64_t grid_handle) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_built.find(grid_handle);
  if (it != g_built.end()) {
    cudaFree(it->second->d_xyzw);
    cudaFree(it->second->d_raw_w);
    cudaFree(it->second->d_host);
    delete it->second;
    g_built.erase(it);
  }
  return 0;
}

static int upload_points_impl(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                              const AoCompGpu* h_comps, int n_comps, const double* h_xyzw, int n_pts, int n_ao,
                              int batch_pts, uint64_t grid_id, size_t memory_limit_bytes, bool spatial,
                              double ao_floor = kZeroFloor) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_shells || !h_prims || !h_comps || !h_xyzw || n_shells <= 0 || n_prims <= 0 || n_comps <= 0 || n_pts <= 0 ||
      n_ao <= 0 || grid_id == 0 || batch_pts < 16 || batch_pts > kBlockPts || !(ao_floor >= kZeroFloor) ||
      !(ao_floor <= 1e-6))
    return -1;
  if (g_grids.count(grid_id)) return -2;
  for (int s = 0; s < n_shells; ++s)
    if (!(h_shells[s].r2_cutoff >= 0.0)) return -1;
  Plan plan;
  if (spatial) {
    const ValueScreen vs{h_prims, h_comps, n_prims, n_comps, ao_floor};
    plan_batches_spatial(h_shells, n_shells, h_xyzw, n_pts, plan, batch_pts, &vs);
  } else
    plan_batches(h_shells, n_shells, h_xyzw, n_pts, plan, batch_pts);
  if (plan.pts.empty()) return -1;
  const int rc = upload_impl(h_shells, n_shells, h_prims, n_prims, h_comps, n_comps, plan.pts.data(),
                             (int)plan.pts.size(), plan.cand_offsets.data(), (int)plan.cand_offsets.size(),
                             plan.cand_shells.data(), (int)plan.cand_shells.size(), n_ao, grid_id, memory_limit_bytes,
                             plan.weights.data(), false);
  if (rc == 0) {
    Entry* e = find(grid_id);
    e->h_orig = std::move(plan.orig);
    e->n_orig = n_pts;
  }
  return rc;
}

int calchem_xc_plan_points(const AoShellGpu* h_shells, int n_shells, const double* h_xyzw, int n_pts, int batch_pts,
                           int spatial, int* n_batches, int* n_kept, int* n_cand, double* sum_m2n, int* max_m,
                           int* h_order, int* h_batch_of, int* h_cand_offsets, int* h_cand_shells, int cand_capacity) {
  if (!h_shells || !h_xyzw || n_shells <= 0 || n_pts <= 0 || batch_pts < 16 || batch_pts > kBlockPts) return -1;
  for (int s = 0; s < n_shells; ++s)
    if (!(h_shells[s].r2_cutoff >= 0.0)) return -1;
  Plan plan;
  if (spatial)
    plan_batches_spatial(h_shells, n_shells, h_xyzw, n_pts, plan, batch_pts);
  else
    plan_batches(h_shells, n_shells, h_xyzw, n_pts, plan, batch_pts);
  const int nb = (int)plan.cand_offsets.size() - 1;
  double s2 = 0.0;
  int mm = 0;
  std::vector<int> bpts(std::max(nb, 0), 0);
  for (const GridPtGpu& p : plan.pts) ++bpts[p.batch_id];
  for (int b = 0; b < nb; ++b) {
    int m = 0;
    for (int c = plan.cand_offsets[b]; c < plan.cand_offsets[b + 1]; ++c) m += h_shells[plan.cand_shells[c]].n_funcs;
    s2 += (double)m * m * bpts[b];
    mm = std::max(mm, m);
  }
  // a candidate buffer that is too small fails the call before any output is written
  if (h_cand_shells && (int)plan.cand_shells.size() > cand_capacity) return -2;
  if (n_batches) *n_batches = nb;
  if (n_kept) *n_kept = (int)plan.orig.size();
  if (n_cand) *n_cand = (int)plan.cand_shells.size();
  if (sum_m2n) *sum_m2n = s2;
  if (max_m) *max_m = mm;
  if (h_order) std::copy(plan.orig.begin(), plan.orig.end(), h_order);
  if (h_batch_of)
    for (size_t k = 0; k < plan.pts.size(); ++k) h_batch_of[k] = plan.pts[k].batch_id;
  if (h_cand_offsets) std::copy(plan.cand_offsets.begin(), plan.cand_offsets.end(), h_cand_offsets);
  if (h_cand_shells) std::copy(plan.cand_shells.begin(), plan.cand_shells.end(), h_cand_shells);
  return 0;
}

int calchem_xc_upload_points_ex(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                                const AoCompGpu* h_comps, int n_comps, const double* h_xyzw, int n_pts, int n_ao,
                                int batch_pts, uint64_t grid_id, size_t memory_limit_bytes) {
  return upload_points_impl(h_shells, n_shells, h_prims, n_prims, h_comps, n_comps, h_xyzw, n_pts, n_ao, batch_pts,
                            grid_id, memory_limit_bytes, false);
}

int calchem_xc_upload_points_spatial(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims,
                                     int n_prims, const AoCompGpu* h_comps, int n_comps, const double* h_xyzw,
                                     int n_pts, int n_ao, int batch_pts, uint64_t grid_id,
                                     size_t memory_limit_bytes) {
  return upload_points_impl(h_shells, n_shells, h_prims, n_prims, h_comps, n_comps, h_xyzw, n_pts, n_ao, batch_pts,
                            grid_id, memory_limit_bytes, true);
}

int calchem_xc_upload_points_screened(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims,
                                      int n_prims, const AoCompGpu* h_comps, int n_comps, const double* h_xyzw,
                                      int n_pts, int n_ao, int batch_pts, uint64_t grid_id,
                                      size_t memory_limit_bytes, double ao_floor) {
  return upload_points_impl(h_shells, n_shells, h_prims, n_prims, h_comps, n_comps, h_xyzw, n_pts, n_ao, batch_pts,
                            grid_id, memory_limit_bytes, true, ao_floor);
}

int calchem_xc_upload_points(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                             const AoCompGpu* h_comps, int n_comps, const double* h_xyzw, int n_pts, int n_ao,
                             uint64_t grid_id, size_t memory_limit_bytes) {
  return calchem_xc_upload_points_ex(h_shells, n_shells, h_prims, n_prims, h_comps, n_comps, h_xyzw, n_pts, n_ao,
                                     kBlockPts, grid_id, memory_limit_bytes);
}

int calchem_xc_set_weights(uint64_t grid_id, const double* h_weights, int n_pts) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_weights || n_pts <= 0) return -1;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || e->n_pts != n_pts) return -2;
  if (cudaMemcpy(e->d_pts + 3 * (size_t)n_pts, h_weights, n_pts * sizeof(double), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return -5;
  e->has_w = true;
  return 0;
}

int calchem_xc_set_ao_cache(uint64_t grid_id, int enable, size_t* bytes_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (enable < 0) {  // query only
    if (bytes_out) *bytes_out = e->ao_cache_bytes;
    return 0;
  }
  if (bytes_out) *bytes_out = 0;
  const int want = enable ? 0 : 1;  // 0: allowed (decided at the next evaluation), 1: off
  if (enable && e->ao_cache_state != 1) {  // already allowed
    if (bytes_out) *bytes_out = e->ao_cache_bytes;
    return 0;
  }
  // evaluations in flight on any stream may still read the cache
  if (cudaDeviceSynchronize() != cudaSuccess) return -5;
  if (e->graph) {  // a captured graph holds the cache pointers
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  ao_cache_free(*e);
  e->ao_cache_state = want;
  return 0;
}

int calchem_xc_plan_stats(uint64_t grid_id, int* n_batches, double* sum_m2n, double* sum_m2, int* max_m) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (n_batches) *n_batches = e->n_batches;
  if (sum_m2n) *sum_m2n = e->sum_m2n;
  if (sum_m2) *sum_m2 = e->sum_m2;
  if (max_m) *max_m = e->max_m;
  return 0;
}

int calchem_xc_eval_closed_shell(int xc_code, int precision, int n, const double* h_rho, const double* h_gamma,
                                 double* h_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_rho || !h_gamma || !h_out || n <= 0 || !valid_xc(xc_code) || (precision != CALCHEM_XC_FP64 &&
                                                                       precision != CALCHEM_XC_MIXED))
    return -1;
  if (!device_ok()) return -3;
  double* d = nullptr;
  if (cudaMalloc(&d, (size_t)n * 5 * sizeof(double)) != cudaSuccess) return -4;
  double* d_rho = d;
  double* d_gam = d + n;
  double* d_out = d + 2 * (size_t)n;
  int rc = 0;
  if (cudaMemcpy(d_rho, h_rho, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_gam, h_gamma, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      launch_closed_shell_points(xc_code, precision, n, d_rho, d_gam, d_out, 0) != cudaSuccess ||
      cudaMemcpy(h_out, d_out, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = -5;
  cudaFree(d);
  return rc;
}

int calchem_xc_evaluate_rks(uint64_t grid_id, int xc_code, int precision, const double* h_d_total, double* exc_out,
                            double* nelec_out, double* h_v_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_d_total || !exc_out || !nelec_out || !h_v_out || !valid_xc(xc_code)) return -1;
  if (!valid_prec(precision, kModeRks)) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  const size_t nn = (size_t)e->nn_total;
  const int M = e->n_mols;
  std::memcpy(e->h_stage, h_d_total, nn * sizeof(double));
  if (cudaMemcpyAsync(e->d_P, e->h_stage, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) != cudaSuccess)
    return -5;
  int rc = enqueue_eval(*e, kModeRks, xc_code, precision, e->d_P, nullptr, e->d_V, nullptr, nullptr, nullptr,
                        e->d_res, e->stream);
  if (rc) return rc;
  double* h_res = e->h_stage + 2 * nn;
  int* h_status = reinterpret_cast<int*>(h_res + 3 * (size_t)M + 1);
  if (cudaMemcpyAsync(e->h_stage, e->d_V, nn * sizeof(double), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(h_res, e->d_res, 2 * (size_t)M * sizeof(double), cudaMemcpyDeviceToHost, e->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(h_status, e->d_counter + 2, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  if (*h_status != 0) return -7;
  std::memcpy(h_v_out, e->h_stage, nn * sizeof(double));
  for (int i = 0; i < M; ++i) {
    exc_out[i] = h_res[2 * i];
    nelec_out[i] = h_res[2 * i + 1];
  }
  return 0;
}

int calchem_xc_evaluate_rks_points(uint64_t grid_id, int xc_code, int precision, const double* h_d_total,
                                   double* exc_out, double* nelec_out, double* h_point_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_d_total || !exc_out || !nelec_out || !h_point_out || !valid_xc(xc_code)) return -1;
  if (!valid_prec(precision, kModeRks)) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  const size_t np2 = 2 * (size_t)e->n_pts;
  if (!e->d_pt_out && !dalloc(&e->d_pt_out, np2)) {
    cudaGetLastError();
    return -4;
  }
  const size_t nn = (size_t)e->nn_total;
  const int M = e->n_mols;
  std::memcpy(e->h_stage, h_d_total, nn * sizeof(double));
  if (cudaMemsetAsync(e->d_pt_out, 0, np2 * sizeof(double), e->stream) != cudaSuccess ||
      cudaMemcpyAsync(e->d_P, e->h_stage, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) != cudaSuccess)
    return -5;
  int rc = enqueue_eval(*e, kModeRks, xc_code, precision, e->d_P, nullptr, e->d_V, nullptr, nullptr, nullptr,
                        e->d_res, e->stream, e->d_pt_out);
  if (rc) return rc;
  double* h_res = e->h_stage + 2 * nn;
  int* h_status = reinterpret_cast<int*>(h_res + 3 * (size_t)M + 1);
  if (cudaMemcpyAsync(h_res, e->d_res, 2 * (size_t)M * sizeof(double), cudaMemcpyDeviceToHost, e->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(h_status, e->d_counter + 2, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  if (*h_status != 0) return -7;
  if (e->h_orig.empty()) {
    if (cudaMemcpy(h_point_out, e->d_pt_out, np2 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return -5;
  } else {  // back to the caller's point order; points the plan dropped (no AO reaches them) get 0
    std::vector<double> tmp(np2);
    if (cudaMemcpy(tmp.data(), e->d_pt_out, np2 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return -5;
    std::memset(h_point_out, 0, 2 * (size_t)e->n_orig * sizeof(double));
    for (size_t k = 0; k < e->h_orig.size(); ++k) {
      h_point_out[2 * (size_t)e->h_orig[k]] = tmp[2 * k];
      h_point_out[2 * (size_t)e->h_orig[k] + 1] = tmp[2 * k + 1];
    }
  }
  for (int i = 0; i < M; ++i) {
    exc_out[i] = h_res[2 * i];
    nelec_out[i] = h_res[2 * i + 1];
  }
  return 0;
}

int calchem_xc_evaluate_uks(uint64_t grid_id, int xc_code, int precision, const double* h_pa, const double* h_pb,
                            double* exc_out, double* nelec_out, double* h_va_out, double* h_vb_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_pa || !h_pb || !exc_out || !nelec_out || !h_va_out || !h_vb_out || !valid_xc(xc_code)) return -1;
  if (!valid_prec(precision, kModeUks)) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  const size_t nn = (size_t)e->nn_total;
  const int M = e->n_mols;
  std::memcpy(e->h_stage, h_pa, nn * sizeof(double));
  std::memcpy(e->h_stage + nn, h_pb, nn * sizeof(double));
  if (cudaMemcpyAsync(e->d_P, e->h_stage, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(e->d_Pb, e->h_stage + nn, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) !=
          cudaSuccess)
    return -5;
  int rc = enqueue_eval(*e, kModeUks, xc_code, precision, e->d_P, e->d_Pb, e->d_V, e->d_Vb, nullptr, nullptr,
                        e->d_res, e->stream);
  if (rc) return rc;
  double* h_res = e->h_stage + 2 * nn;
  int* h_status = reinterpret_cast<int*>(h_res + 3 * (size_t)M + 1);
  if (cudaMemcpyAsync(e->h_stage, e->d_V, nn * sizeof(double), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(e->h_stage + nn, e->d_Vb, nn * sizeof(double), cudaMemcpyDeviceToHost, e->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(h_res, e->d_res, 3 * (size_t)M * sizeof(double), cudaMemcpyDeviceToHost, e->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(h_status, e->d_counter + 2, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  if (*h_status != 0) return -7;
  std::memcpy(h_va_out, e->h_stage, nn * sizeof(double));
  std::memcpy(h_vb_out, e->h_stage + nn, nn * sizeof(double));
  for (int i = 0; i < M; ++i) {
    exc_out[i] = h_res[3 * i];
    nelec_out[2 * i] = h_res[3 * i + 1];
    nelec_out[2 * i + 1] = h_res[3 * i + 2];
  }
  return 0;
}

int calchem_xc_evaluate_rks_device(uint64_t grid_id, int xc_code, int precision, const double* d_total,
                                   double* d_result, double* d_v, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_total || !d_result || !d_v || !valid_xc(xc_code) || !valid_prec(precision, kModeRks)) return -1;
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  return enqueue_eval(*e, kModeRks, xc_code, precision, d_total, nullptr, d_v, nullptr, nullptr, nullptr, d_result,
                      (cudaStream_t)stream);
}

int calchem_xc_evaluate_uks_device(uint64_t grid_id, int xc_code, int precision, const double* d_pa,
                                   const double* d_pb, double* d_result, double* d_va, double* d_vb, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_pa || !d_pb || !d_result || !d_va || !d_vb || !valid_xc(xc_code) || !valid_prec(precision, kModeUks))
    return -1;
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  return enqueue_eval(*e, kModeUks, xc_code, precision, d_pa, d_pb, d_va, d_vb, nullptr, nullptr, d_result,
                      (cudaStream_t)stream);
}

int calchem_xc_set_tile(uint64_t grid_id, int tile_n) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (tile_n != 64 && tile_n != 128) return -1;
  Entry* e = find(grid_id);
  if (!e) return -2;
  e->tile_n = tile_n;
  return 0;
}

int calchem_xc_get_tile(uint64_t grid_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  return e ? e->tile_n : -2;
}

int calchem_xc_set_point_atoms(uint64_t grid_id, const int* h_host_atom, int n_points, int n_atoms) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_host_atom || n_points <= 0 || n_atoms <= 0) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1) return -2;
  const int n_caller = e->h_orig.empty() ? e->n_pts : e->n_orig;
  if (n_points != n_caller) return -2;
  for (int k = 0; k < n_points; ++k)
    if (h_host_atom[k] < 0 || h_host_atom[k] >= n_atoms) return -1;
  // planned point k came from the caller's point h_orig[k] (identity without a plan); counting sort
  // by atom keeps the planned order within each atom
  std::vector<int> off(n_atoms + 1, 0), pts(e->n_pts);
  auto atom_of = [&](int k) { return h_host_atom[e->h_orig.empty() ? k : e->h_orig[k]]; };
  for (int k = 0; k < e->n_pts; ++k) ++off[atom_of(k) + 1];
  for (int a = 0; a < n_atoms; ++a) off[a + 1] += off[a];
  std::vector<int> fill(off.begin(), off.end() - 1);
  for (int k = 0; k < e->n_pts; ++k) pts[fill[atom_of(k)]++] = k;
  for (int* p : {e->d_atom_pts, e->d_atom_off}) if (p) cudaFree(p);
  if (e->d_atom_out) cudaFree(e->d_atom_out);
  e->d_atom_pts = e->d_atom_off = nullptr;
  e->d_atom_out = nullptr;
  e->n_share_atoms = 0;
  if (!dalloc(&e->d_atom_pts, pts.size()) || !dalloc(&e->d_atom_off, off.size()) ||
      !dalloc(&e->d_atom_out, 2 * (size_t)n_atoms)) {
    cudaGetLastError();
    return -4;
  }
  if (cudaMemcpy(e->d_atom_pts, pts.data(), pts.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->d_atom_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return -5;
  e->n_share_atoms = n_atoms;
  return 0;
}

namespace {
// Per-point shares and their per-atom sums, enqueued on st; with d_v the full build (Vxc into d_v)
// as well, without it the shares alone (no Vxc contraction).
int enqueue_atom_shares(Entry& e, int xc_code, int precision, const double* d_total, double* d_result, double* d_v,
                        double* d_atom_out, cudaStream_t st) {
  if (int rc0 = ensure_ws(e)) return rc0;
  const size_t np2 = 2 * (size_t)e.n_pts;
  if (!e.d_pt_out && !dalloc(&e.d_pt_out, np2)) {
    cudaGetLastError();
    return -4;
  }
  if (cudaMemsetAsync(e.d_pt_out, 0, np2 * sizeof(double), st) != cudaSuccess) return -5;
  int rc = enqueue_eval(e, kModeRks, xc_code, precision, d_total, nullptr, d_v, nullptr, nullptr, nullptr, d_result,
                        st, e.d_pt_out, d_v == nullptr);
  if (rc) return rc;
  if (launch_atom_shares(e.d_pt_out, e.d_atom_pts, e.d_atom_off, e.n_share_atoms, d_atom_out, st) != cudaSuccess)
    return -5;
  e.last_launches += 1;
  return 0;
}
}  // namespace

int calchem_xc_evaluate_rks_atoms(uint64_t grid_id, int xc_code, int precision, const double* h_d_total,
                                  double* exc_out, double* nelec_out, double* h_atom_out, double* h_v_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_d_total || !exc_out || !nelec_out || !h_atom_out || !valid_xc(xc_code)) return -1;
  if (!valid_prec(precision, kModeRks)) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || e->n_share_atoms <= 0) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  const size_t nn = (size_t)e->nn_total;
  std::memcpy(e->h_stage, h_d_total, nn * sizeof(double));
  if (cudaMemcpyAsync(e->d_P, e->h_stage, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) != cudaSuccess)
    return -5;
  int rc = enqueue_atom_shares(*e, xc_code, precision, e->d_P, e->d_res, h_v_out ? e->d_V : nullptr, e->d_atom_out,
                               e->stream);
  if (rc) return rc;
  double* h_res = e->h_stage + 2 * nn;
  int* h_status = reinterpret_cast<int*>(h_res + 4);
  if (h_v_out && cudaMemcpyAsync(e->h_stage, e->d_V, nn * sizeof(double), cudaMemcpyDeviceToHost, e->stream) !=
                     cudaSuccess)
    return -5;
  if (cudaMemcpyAsync(h_res, e->d_res, 2 * sizeof(double), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(h_status, e->d_counter + 2, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(h_atom_out, e->d_atom_out, 2 * (size_t)e->n_share_atoms * sizeof(double), cudaMemcpyDeviceToHost,
                      e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  if (*h_status != 0) return -7;
  *exc_out = h_res[0];
  *nelec_out = h_res[1];
  if (h_v_out) std::memcpy(h_v_out, e->h_stage, nn * sizeof(double));
  return 0;
}

int calchem_xc_evaluate_rks_atoms_device(uint64_t grid_id, int xc_code, int precision, const double* d_total,
                                         double* d_result, double* d_v, double* d_atom_out, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_total || !d_result || !d_atom_out || !valid_xc(xc_code) || !valid_prec(precision, kModeRks)) return -1;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || e->n_share_atoms <= 0) return -2;
  if (!e->has_w) return -1;
  return enqueue_atom_shares(*e, xc_code, precision, d_total, d_result, d_v, d_atom_out, (cudaStream_t)stream);
}

int calchem_xc_fxc_prepare(uint64_t grid_id, int xc_code, const double* h_d_total) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_d_total || !valid_xc(xc_code)) return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  if (!e->d_fxc && !dalloc(&e->d_fxc, 11 * (size_t)e->n_pts)) {
    cudaGetLastError();
    return -4;
  }
  const size_t nn = (size_t)e->n_ao * e->n_ao;
  std::memcpy(e->h_stage, h_d_total, nn * sizeof(double));
  if (cudaMemcpyAsync(e->d_P, e->h_stage, nn * sizeof(double), cudaMemcpyHostToDevice, e->stream) != cudaSuccess)
    return -5;
  int rc = enqueue_eval(*e, kModeRho, 0, CALCHEM_XC_FP64, e->d_P, nullptr, nullptr, nullptr, nullptr, e->d_rg,
                        nullptr, e->stream);
  if (rc) return rc;
  if (launch_fxc_coef(e->d_rg, e->d_pts + 3 * (size_t)e->n_pts, e->n_pts, xc_code, e->d_fxc, e->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  e->fxc_code = xc_code;
  return 0;
}

int calchem_xc_fxc_contract_device(uint64_t grid_id, int triplet, const double* d_m, int n_trials, double* d_v_out,
                                   void* stream) {
  return calchem_xc_fxc_contract_device_ex(grid_id, triplet, CALCHEM_XC_FP64, d_m, n_trials, d_v_out, stream);
}

int calchem_xc_fxc_contract_device_ex(uint64_t grid_id, int triplet, int precision, const double* d_m, int n_trials,
                                      double* d_v_out, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_m || !d_v_out || n_trials <= 0 || (precision != CALCHEM_XC_FP64 && precision != CALCHEM_XC_MIXED))
    return -1;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1) return -2;
  if (e->fxc_code < 0) return -1;
  if (precision == CALCHEM_XC_MIXED) {
    if (e->max_m > mixed_max_m()) return -2;
    return enqueue_fxc_mixed(*e, triplet, d_m, n_trials, d_v_out, (cudaStream_t)stream);
  }
  return enqueue_fxc(*e, triplet, d_m, n_trials, d_v_out, (cudaStream_t)stream);
}

int calchem_xc_fxc_contract(uint64_t grid_id, int triplet, const double* h_m, int n_trials, double* h_v_out) {
  return calchem_xc_fxc_contract_ex(grid_id, triplet, CALCHEM_XC_FP64, h_m, n_trials, h_v_out);
}

int calchem_xc_fxc_contract_ex(uint64_t grid_id, int triplet, int precision, const double* h_m, int n_trials,
                               double* h_v_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!h_m || !h_v_out || n_trials <= 0 || (precision != CALCHEM_XC_FP64 && precision != CALCHEM_XC_MIXED))
    return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1) return -2;
  if (e->fxc_code < 0) return -1;
  const size_t nn = (size_t)e->n_ao * e->n_ao;
  if (n_trials > e->fxc_cap) {
    if (e->d_fxc_m) cudaFree(e->d_fxc_m);
    if (e->d_fxc_v) cudaFree(e->d_fxc_v);
    e->d_fxc_m = e->d_fxc_v = nullptr;
    e->fxc_cap = 0;
    if (!dalloc(&e->d_fxc_m, nn * n_trials) || !dalloc(&e->d_fxc_v, nn * n_trials)) {
      cudaGetLastError();
      return -4;
    }
    e->fxc_cap = n_trials;
  }
  int st = 0;
  if (cudaMemcpyAsync(e->d_fxc_m, h_m, nn * n_trials * sizeof(double), cudaMemcpyHostToDevice, e->stream) !=
      cudaSuccess)
    return -5;
  if (precision == CALCHEM_XC_MIXED && e->max_m > mixed_max_m()) return -2;
  if (int rc = precision == CALCHEM_XC_MIXED
                   ? enqueue_fxc_mixed(*e, triplet, e->d_fxc_m, n_trials, e->d_fxc_v, e->stream)
                   : enqueue_fxc(*e, triplet, e->d_fxc_m, n_trials, e->d_fxc_v, e->stream))
    return rc;
  if (cudaMemcpyAsync(h_v_out, e->d_fxc_v, nn * n_trials * sizeof(double), cudaMemcpyDeviceToHost, e->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(&st, e->d_counter + 2, sizeof(int), cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return -5;
  return st != 0 ? -7 : 0;
}

int calchem_xc_nuclear_gradient(uint64_t grid_id, int xc_code, int precision, int n_atoms, const int* z,
                                const double* xyz_bohr, const double* h_raw_w, const int* h_host_atom, int n_grid_pts,
                                const double* h_pa, const double* h_pb, double* h_grad_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (grid_id == 0 || !z || !xyz_bohr || !h_raw_w || !h_host_atom || !h_pa || !h_grad_out || n_atoms <= 0 ||
      n_atoms > grad_max_atoms() || !valid_xc(xc_code) ||
      (precision != CALCHEM_XC_FP64 && precision != CALCHEM_XC_MIXED))
    return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e || e->n_mols != 1 || !e->has_w) return -2;
  const int n_caller = e->h_orig.empty() ? e->n_pts : e->n_orig;
  if (n_grid_pts != n_caller) return -2;
  std::fill(h_grad_out, h_grad_out + 3 * (size_t)n_atoms, 0.0);
  if (n_atoms == 1) return 0;  // translational invariance: no gradient for one atom (vxc.rs:1922-1924)
  if (int rc0 = ensure_ws(*e)) return rc0;
  std::vector<double> raw(e->n_pts);
  std::vector<int> host(e->n_pts);
  for (int g = 0; g < e->n_pts; ++g) {
    const int o = e->h_orig.empty() ? g : e->h_orig[g];
    raw[g] = h_raw_w[o];
    host[g] = h_host_atom[o];
  }
  return gradient_run(*e, xc_code, precision, h_pb == nullptr, h_pa, h_pb, nullptr, raw.data(), host.data(), n_atoms,
                      z,
                      xyz_bohr, h_grad_out, SIZE_MAX);
}

int calchem_xc_group_create(const uint64_t* member_ids, int n_members, uint64_t group_id, size_t memory_limit_bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!member_ids || n_members <= 0 || group_id == 0) return -1;
  if (!device_ok()) return -3;
  if (g_grids.count(group_id)) return -2;
  std::vector<Entry*> mem(n_members);
  for (int i = 0; i < n_members; ++i) {
    mem[i] = find(member_ids[i]);
    if (!mem[i] || mem[i]->n_mols != 1) return -2;
    if (!mem[i]->has_w) return -1;
    for (int j = 0; j < i; ++j)
      if (member_ids[j] == member_ids[i]) return -1;
  }
  // offsets of every member's arrays inside the group's
  long long n_pts = 0, n_shells = 0, n_prims = 0, n_comps = 0, n_cand = 0, n_bao = 0, n_b = 0, n_rows = 0, nn = 0;
  int max_m = 0, max_n = 0;
  double s_m2n = 0, s_m2 = 0;
  std::vector<long long> o_pts(n_members), o_sh(n_members), o_pr(n_members), o_co(n_members), o_ca(n_members),
      o_bao(n_members), o_b(n_members);
  Entry* g = new Entry;
  for (int i = 0; i < n_members; ++i) {
    const Entry& m = *mem[i];
    o_pts[i] = n_pts; o_sh[i] = n_shells; o_pr[i] = n_prims; o_co[i] = n_comps; o_ca[i] = n_cand;
    o_bao[i] = n_bao; o_b[i] = n_b;
    g->h_mol_n.push_back(m.n_ao);
    g->h_mol_off.push_back(nn);
    g->h_mol_ao_off.push_back((int)n_rows);
    g->h_mol_boff.push_back((int)n_b);
    n_pts += m.n_pts; n_shells += m.n_shells; n_prims += m.n_prims; n_comps += m.n_comps;
    n_cand += (long long)m.n_cand; n_bao += (long long)m.n_bao; n_b += m.n_batches; n_rows += m.n_ao;
    nn += (long long)m.n_ao * m.n_ao;
    max_m = std::max(max_m, m.max_m);
    max_n = std::max(max_n, m.n_ao);
    s_m2n += m.sum_m2n;
    s_m2 += m.sum_m2;
  }
  g->h_mol_ao_off.push_back((int)n_rows);
  g->h_mol_boff.push_back((int)n_b);
  if (n_pts > INT32_MAX || n_cand > INT32_MAX || n_bao > INT32_MAX || n_rows > INT32_MAX || n_b > INT32_MAX ||
      n_shells > INT32_MAX) {
    delete g;
    return -2;
  }
  g->n_pts = (int)n_pts;
  g->n_ao = (int)n_rows;
  g->n_shells = (int)n_shells;
  g->n_prims = (int)n_prims;
  g->n_comps = (int)n_comps;
  g->n_batches = (int)n_b;
  g->n_cand = (size_t)n_cand;
  g->n_bao = (size_t)n_bao;
  g->max_m = max_m;
  g->max_n = max_n;
  g->n_mols = n_members;
  g->nn_total = nn;
  g->sum_m2n = s_m2n;
  g->sum_m2 = s_m2;
  g->has_w = true;
  const int m_pad = (max_m + 63) / 64 * 64;
  g->n_ctas = std::max(1, std::min(g->n_batches, g_sm_count));
  g->slab_stride = (size_t)kPlanes * m_pad * kBlockPts;
  g->mixed_ctas = std::max(1, std::min(g->n_batches, g_sm_count * mixed_ctas_per_sm(64)));
  g->mixed_slab_stride = mixed_slab_doubles(max_m);
  size_t total = (size_t)n_shells * sizeof(AoShellGpu) + (size_t)n_prims * (sizeof(AoPrimGpu) + sizeof(float4)) +
                 (size_t)n_comps * (sizeof(AoCompGpu) + sizeof(float2)) + (size_t)n_shells * 3 * sizeof(float2) +
                 (size_t)n_pts * 4 * sizeof(double) + (size_t)n_b * (sizeof(BatchDesc) + sizeof(int)) +
                 (size_t)n_cand * 2 * sizeof(int) + (size_t)n_bao * sizeof(int) + (size_t)n_members * 32;
  total += workspace_bytes(*g);
  g->bytes = total;
  g->mem_limit = memory_limit_bytes;
  if (total > memory_limit_bytes) {
    delete g;
    return -3;
  }
  auto fail = [&](int code) {
    cudaGetLastError();
    g->free_all();
    delete g;
    return code;
  };
  if (!(dalloc(&g->d_shells, n_shells) && dalloc(&g->d_prims, n_prims) && dalloc(&g->d_comps, n_comps) &&
        dalloc(&g->d_prim_f, n_prims) && dalloc(&g->d_comp_f, n_comps) && dalloc(&g->d_shell_cf, 3 * (size_t)n_shells) &&
        dalloc(&g->d_pts, (size_t)n_pts * 4) && dalloc(&g->d_batches, n_b) && dalloc(&g->d_cand, n_cand) &&
        dalloc(&g->d_cand_loc, n_cand) && dalloc(&g->d_bao, n_bao) && dalloc(&g->d_order, n_b) &&
        dalloc(&g->d_mol_n, n_members) && dalloc(&g->d_mol_off, n_members) &&
        dalloc(&g->d_mol_ao_off, n_members + 1) && dalloc(&g->d_mol_boff, n_members + 1)))
    return fail(-4);
  // device-to-device copies of the arrays that need no renumbering; host renumbering of the rest
  std::vector<AoShellGpu> shells((size_t)n_shells);
  std::vector<BatchDesc> batches((size_t)n_b);
  std::vector<int> cand((size_t)n_cand);
  bool ok = true;
  for (int i = 0; i < n_members && ok; ++i) {
    const Entry& m = *mem[i];
    const auto d2d = cudaMemcpyDeviceToDevice;
    for (int k = 0; k < 4 && ok; ++k)
      ok = cudaMemcpy(g->d_pts + (size_t)k * n_pts + o_pts[i], m.d_pts + (size_t)k * m.n_pts,
                      (size_t)m.n_pts * sizeof(double), d2d) == cudaSuccess;
    ok = ok &&
         cudaMemcpy(g->d_prims + o_pr[i], m.d_prims, (size_t)m.n_prims * sizeof(AoPrimGpu), d2d) == cudaSuccess &&
         cudaMemcpy(g->d_prim_f + o_pr[i], m.d_prim_f, (size_t)m.n_prims * sizeof(float4), d2d) == cudaSuccess &&
         cudaMemcpy(g->d_comps + o_co[i], m.d_comps, (size_t)m.n_comps * sizeof(AoCompGpu), d2d) == cudaSuccess &&
         cudaMemcpy(g->d_comp_f + o_co[i], m.d_comp_f, (size_t)m.n_comps * sizeof(float2), d2d) == cudaSuccess &&
         cudaMemcpy(g->d_shell_cf + 3 * o_sh[i], m.d_shell_cf, 3 * (size_t)m.n_shells * sizeof(float2), d2d) ==
             cudaSuccess &&
         cudaMemcpy(g->d_cand_loc + o_ca[i], m.d_cand_loc, m.n_cand * sizeof(int), d2d) == cudaSuccess &&
         cudaMemcpy(g->d_bao + o_bao[i], m.d_bao, m.n_bao * sizeof(int), d2d) == cudaSuccess &&
         cudaMemcpy(shells.data() + o_sh[i], m.d_shells, (size_t)m.n_shells * sizeof(AoShellGpu),
                    cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(batches.data() + o_b[i], m.d_batches, (size_t)m.n_batches * sizeof(BatchDesc),
                    cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(cand.data() + o_ca[i], m.d_cand, m.n_cand * sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
    if (!ok) break;
    for (int k = 0; k < m.n_shells; ++k) {
      AoShellGpu& sh = shells[(size_t)o_sh[i] + k];
      sh.prim_start += (int)o_pr[i];
      sh.comp_start += (int)o_co[i];
    }
    for (size_t k = 0; k < m.n_cand; ++k) cand[(size_t)o_ca[i] + k] += (int)o_sh[i];
    for (int k = 0; k < m.n_batches; ++k) {
      BatchDesc& d = batches[(size_t)o_b[i] + k];
      d.pt_start += (int)o_pts[i];
      d.cand_start += (int)o_ca[i];
      d.ao_start += (int)o_bao[i];
      d.mol = i;
    }
  }
  if (!ok) return fail(-5);
  // one work queue over all molecules, most expensive batches first
  std::vector<int> order((size_t)n_b);
  for (long long i = 0; i < n_b; ++i) order[(size_t)i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const double cx = (double)batches[x].m * batches[x].m * batches[x].n_pts;
    const double cy = (double)batches[y].m * batches[y].m * batches[y].n_pts;
    return cx > cy;
  });
  ok = cudaMemcpy(g->d_shells, shells.data(), shells.size() * sizeof(AoShellGpu), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(g->d_batches, batches.data(), batches.size() * sizeof(BatchDesc), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(g->d_cand, cand.data(), cand.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(g->d_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(g->d_mol_n, g->h_mol_n.data(), n_members * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(g->d_mol_off, g->h_mol_off.data(), n_members * sizeof(long long), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(g->d_mol_ao_off, g->h_mol_ao_off.data(), (n_members + 1) * sizeof(int), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(g->d_mol_boff, g->h_mol_boff.data(), (n_members + 1) * sizeof(int), cudaMemcpyHostToDevice) ==
           cudaSuccess;
  if (!ok) return fail(-5);
  g_grids[group_id] = g;
  return 0;
}

int calchem_xc_group_layout(uint64_t grid_id, int* n_mols_out, int* mol_n_out, long long* mol_off_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!n_mols_out) return -1;
  *n_mols_out = e->n_mols;
  for (int i = 0; i < e->n_mols; ++i) {
    if (mol_n_out) mol_n_out[i] = e->h_mol_n[i];
    if (mol_off_out) mol_off_out[i] = e->h_mol_off[i];
  }
  return 0;
}

int calchem_xc_graph_capture(uint64_t grid_id, int mode, int xc_code, int precision, const double* d_pa,
                             const double* d_pb, double* d_result, double* d_va, double* d_vb) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (mode != 0 && mode != 1) return -1;
  const int kmode = mode == 0 ? kModeRks : kModeUks;
  if (!d_pa || !d_result || !d_va || (kmode == kModeUks && (!d_pb || !d_vb)) || !valid_xc(xc_code) ||
      !valid_prec(precision, kmode))
    return -1;
  if (!device_ok()) return -3;
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->has_w) return -1;
  if (int rc0 = ensure_ws(*e)) return rc0;
  // kernel attributes are set, and the AO cache decided, outside the capture
  if (fp64_set_attributes() != cudaSuccess || mixed_set_attributes() != cudaSuccess) return -5;
  if (precision == CALCHEM_XC_MIXED) ao_cache_decide(*e);
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  const bool prof = e->profiling;
  e->profiling = false;
  if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    e->profiling = prof;
    return -5;
  }
  const int rc = enqueue_eval(*e, kmode, xc_code, precision, d_pa, kmode == kModeUks ? d_pb : nullptr, d_va,
                              kmode == kModeUks ? d_vb : nullptr, nullptr, nullptr, d_result, e->stream);
  cudaGraph_t graph = nullptr;
  const cudaError_t end = cudaStreamEndCapture(e->stream, &graph);
  e->profiling = prof;
  if (rc || end != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc ? rc : -5;
  }
  const cudaError_t inst = cudaGraphInstantiate(&e->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (inst != cudaSuccess) {
    e->graph = nullptr;
    cudaGetLastError();
    return -5;
  }
  return 0;
}

int calchem_xc_graph_launch(uint64_t grid_id, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->graph) return -1;
  return cudaGraphLaunch(e->graph, (cudaStream_t)stream) == cudaSuccess ? 0 : -5;
}

int calchem_xc_last_status(uint64_t grid_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!e->ws) return 0;
  int st = 0;
  if (cudaMemcpy(&st, e->d_counter + 2, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -5;
  return st != 0 ? -7 : 0;
}

int calchem_xc_last_launch_count(uint64_t grid_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  return e ? e->last_launches : -2;
}

int calchem_xc_set_profiling(uint64_t grid_id, int enable) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (enable && !e->ev0) {
    if (cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess) return -5;
  }
  e->profiling = enable != 0;
  return 0;
}

int calchem_xc_last_kernel_ms(uint64_t grid_id, float* ms_out) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry* e = find(grid_id);
  if (!e) return -2;
  if (!ms_out || !e->profiling || !e->ev1) return -1;
  if (cudaEventSynchronize(e->ev1) != cudaSuccess) return -5;
  return cudaEventElapsedTime(ms_out, e->ev0, e->ev1) == cudaSuccess ? 0 : -5;
}

}  // extern "C"
