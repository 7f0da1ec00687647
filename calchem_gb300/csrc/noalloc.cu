// noalloc.cu -- closed-shell FP64 Vxc evaluation that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc -- a host framework that owns all device memory
// through its own pool (and would have its accounting bypassed or its memory fragmented), or a
// serving loop that must not pay cudaMalloc's implicit device-wide synchronisation in the middle
// of an SCF iteration.  Such a caller passes every input and output as device buffers it already
// owns; the kernel's working memory (the per-CTA AO slabs, the derived batch tables, the per-batch
// Exc/Nelec partials, the work-queue head and a status word) comes from the one fixed array below.
//
// Properties of that array:
//   * it is a file-scope static __device__ array of kStaticScratchBytes (96 MiB); every GPU that
//     loads this library holds it until the process exits;
//   * host code cannot use the symbol name as a device address, so the first call on each device
//     looks the address up with cudaGetSymbolAddress while that device is current and caches it;
//     that first call should therefore come before any stream capture on the device.  The cached
//     address belongs to the device's current primary context: after a cudaDeviceReset the entry
//     point must not be called again in the same process;
//   * every call reuses it and it keeps the previous call's contents: the queue head and status
//     word are cleared at the start of each call, everything else is overwritten before it is read;
//   * calls whose work overlaps on the GPU (other streams, other host threads) race on it.  The
//     entry point is synchronous and serialised by a mutex, so calls through it never overlap.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace cxc {
cudaError_t launch_fp64(const DevGrid& G, const EvalArgs& A, int n_ctas, cudaStream_t st);
cudaError_t launch_reduce(const double* part, int n_batches, double* out, int n_out, cudaStream_t st);
cudaError_t launch_mirror(double* V, int n, int from_upper, cudaStream_t st);
}  // namespace cxc

namespace {

using namespace cxc;

constexpr size_t kStaticScratchBytes = (size_t)96 << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Status bits written by the table kernels when the caller's layout is inconsistent.
enum : int { kBadBatch = 1, kBadShell = 2, kBadSize = 4 };

// Points (AoS with batch ids) -> SoA coordinates and weights.  Also checks the batch ids: each in
// [0, n_batches) and none smaller than its predecessor's (the later kernels find a batch's points by
// binary search over the ids).  With ids in range and in order, the per-batch point ranges partition
// the points, so their counts add up to n_pts.
__global__ void soa_points_kernel(const GridPtGpu* __restrict__ pts, const double* __restrict__ w, int n_pts,
                                  int n_batches, double* __restrict__ soa, int* __restrict__ status) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_pts) return;
  const GridPtGpu p = pts[g];
  if (p.batch_id < 0 || p.batch_id >= n_batches || (g > 0 && pts[g - 1].batch_id > p.batch_id))
    atomicOr(status, kBadBatch);
  soa[g] = p.x;
  soa[(size_t)n_pts + g] = p.y;
  soa[2 * (size_t)n_pts + g] = p.z;
  soa[3 * (size_t)n_pts + g] = w[g];
}

// One thread per batch: point range (points are grouped by non-decreasing batch id), candidate
// range, AO count; every index the later kernels use is checked here.
__global__ void batch_tables_kernel(const AoShellGpu* __restrict__ shells, int n_shells, int n_prims, int n_comps,
                                    const GridPtGpu* __restrict__ pts, int n_pts, const int* __restrict__ cand_off,
                                    const int* __restrict__ cand_sh, int n_batches, int n_cand, int n_ao, int max_m,
                                    BatchDesc* __restrict__ bd, int* __restrict__ m_out, int* __restrict__ status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_batches) return;
  int lo = 0, hi = n_pts;  // first point with batch_id >= b
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pts[mid].batch_id < b) lo = mid + 1; else hi = mid;
  }
  const int start = lo;
  hi = n_pts;  // first point with batch_id > b
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pts[mid].batch_id <= b) lo = mid + 1; else hi = mid;
  }
  int np = lo - start;
  if (np > kBlockPts) { atomicOr(status, kBadBatch); np = 0; }
  const int c0 = cand_off[b], c1 = cand_off[b + 1];
  int m = 0;
  bool ok = c0 >= 0 && c1 >= c0 && c1 <= n_cand;
  for (int c = c0; ok && c < c1; ++c) {
    const int s = cand_sh[c];
    if (s < 0 || s >= n_shells) { ok = false; break; }
    const AoShellGpu sh = shells[s];
    if (sh.n_funcs < 1 || sh.n_funcs > 10 || sh.n_prims < 1 || sh.prim_start < 0 || sh.comp_start < 0 ||
        sh.ao_offset < 0 || sh.prim_start + sh.n_prims > n_prims || sh.comp_start + sh.n_funcs > n_comps ||
        sh.ao_offset + sh.n_funcs > n_ao) {
      ok = false;
      break;
    }
    m += sh.n_funcs;
  }
  if (!ok) { atomicOr(status, kBadShell); m = 0; np = 0; }
  if (m > max_m) { atomicOr(status, kBadSize); m = 0; np = 0; }
  BatchDesc d{};
  d.pt_start = start;
  d.n_pts = np;
  d.cand_start = ok ? c0 : 0;
  d.n_cand = (ok && m > 0) ? c1 - c0 : 0;
  d.m = m;
  bd[b] = d;
  m_out[b] = m;
}

// Exclusive prefix of the per-batch AO counts (one CTA) -> BatchDesc::ao_start; identity order.
__global__ void __launch_bounds__(1024) ao_offsets_kernel(const int* __restrict__ m, int n, BatchDesc* __restrict__ bd,
                                                          int* __restrict__ order) {
  __shared__ int s[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < n ? m[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) {
      bd[i].ao_start = carry + s[threadIdx.x] - v;
      order[i] = i;
    }
    __syncthreads();
    if (threadIdx.x == 1023) carry += s[1023];
    __syncthreads();
  }
}

// One thread per batch: local AO offset of each candidate and the local -> global AO list.  Skipped
// entirely when an earlier kernel flagged the layout: the AO list's capacity (10 entries per
// candidate) holds only for candidate ranges that are all valid.
__global__ void ao_lists_kernel(const AoShellGpu* __restrict__ shells, const int* __restrict__ cand_sh,
                                const BatchDesc* __restrict__ bd, int n_batches, int* __restrict__ cand_loc,
                                int* __restrict__ batch_ao, const int* __restrict__ status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_batches || *status != 0) return;
  const BatchDesc d = bd[b];
  int loc = 0;
  for (int c = 0; c < d.n_cand; ++c) {
    const AoShellGpu sh = shells[cand_sh[d.cand_start + c]];
    cand_loc[d.cand_start + c] = loc;
    for (int k = 0; k < sh.n_funcs; ++k) batch_ao[d.ao_start + loc + k] = sh.ao_offset + k;
    loc += sh.n_funcs;
  }
}

// Address of the static scratch on the current device (looked up once per device).
int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -3;
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return -3;
    }
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return 0;
}

}  // namespace

extern "C" int calchem_xc_evaluate_rks_static(const AoShellGpu* d_shells, int n_shells, const AoPrimGpu* d_prims,
                                              int n_prims, const AoCompGpu* d_comps, int n_comps,
                                              const GridPtGpu* d_pts, const double* d_weights, int n_pts,
                                              const int* d_cand_offsets, const int* d_cand_shells, int n_batches,
                                              int n_cand_shells, int n_ao, int max_batch_ao, int xc_code,
                                              const double* d_total, double* d_result, double* d_v, void* stream) {
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!d_shells || !d_prims || !d_comps || !d_pts || !d_weights || !d_cand_offsets || !d_cand_shells || !d_total ||
      !d_result || !d_v || n_shells <= 0 || n_prims <= 0 || n_comps <= 0 || n_pts <= 0 || n_batches <= 0 ||
      n_cand_shells <= 0 || n_ao <= 0 || max_batch_ao <= 0 || xc_code < 0 || xc_code > 8)
    return -1;
  void* base = nullptr;
  if (static_scratch(&base) != 0) return -3;
  // carve the static array: header | SoA points | batch tables | AO lists | partials | slabs
  const int m_pad = (max_batch_ao + 63) / 64 * 64;
  const size_t slab_stride = (size_t)5 * m_pad * kBlockPts;  // doubles per CTA
  size_t off = 256;
  const size_t o_soa = off;  off = align256(off + (size_t)n_pts * 4 * sizeof(double));
  const size_t o_bd = off;   off = align256(off + (size_t)n_batches * sizeof(BatchDesc));
  const size_t o_m = off;    off = align256(off + (size_t)n_batches * sizeof(int));
  const size_t o_ord = off;  off = align256(off + (size_t)n_batches * sizeof(int));
  const size_t o_loc = off;  off = align256(off + (size_t)n_cand_shells * sizeof(int));
  const size_t o_ao = off;   off = align256(off + (size_t)n_cand_shells * 10 * sizeof(int));
  const size_t o_red = off;  off = align256(off + (size_t)n_batches * 3 * sizeof(double));
  const size_t o_slab = off;
  if (o_slab + slab_stride * sizeof(double) > kStaticScratchBytes) return -3;  // too large for the static scratch
  int sms = 1, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t fit = (kStaticScratchBytes - o_slab) / (slab_stride * sizeof(double));
  const int n_ctas = (int)std::min<size_t>(std::min<size_t>(fit, (size_t)sms), (size_t)n_batches);

  unsigned char* sc = static_cast<unsigned char*>(base);
  int* status = reinterpret_cast<int*>(sc);     // [0] status, [1..3] queue heads
  double* soa = reinterpret_cast<double*>(sc + o_soa);
  BatchDesc* bd = reinterpret_cast<BatchDesc*>(sc + o_bd);
  int* mcount = reinterpret_cast<int*>(sc + o_m);
  int* order = reinterpret_cast<int*>(sc + o_ord);
  int* cand_loc = reinterpret_cast<int*>(sc + o_loc);
  int* batch_ao = reinterpret_cast<int*>(sc + o_ao);
  double* red = reinterpret_cast<double*>(sc + o_red);
  double* slab = reinterpret_cast<double*>(sc + o_slab);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t nn = (size_t)n_ao * n_ao;

  bool ok = cudaMemsetAsync(status, 0, 4 * sizeof(int), st) == cudaSuccess;
  if (ok) {
    soa_points_kernel<<<(n_pts + 255) / 256, 256, 0, st>>>(d_pts, d_weights, n_pts, n_batches, soa, status);
    batch_tables_kernel<<<(n_batches + 127) / 128, 128, 0, st>>>(d_shells, n_shells, n_prims, n_comps, d_pts, n_pts,
                                                                 d_cand_offsets, d_cand_shells, n_batches,
                                                                 n_cand_shells, n_ao, max_batch_ao, bd, mcount, status);
    ao_offsets_kernel<<<1, 1024, 0, st>>>(mcount, n_batches, bd, order);
    ao_lists_kernel<<<(n_batches + 127) / 128, 128, 0, st>>>(d_shells, d_cand_shells, bd, n_batches, cand_loc,
                                                             batch_ao, status);
    ok = cudaGetLastError() == cudaSuccess;
  }
  int h_status = 0;
  ok = ok && cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
       cudaStreamSynchronize(st) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return -5;
  }
  if (h_status != 0) return -2;  // the caller's layout is inconsistent (bad batch ids, shells or sizes)

  DevGrid G{};
  G.n_pts = n_pts;
  G.n_ao = n_ao;
  G.n_shells = n_shells;
  G.n_batches = n_batches;
  G.shells = d_shells;
  G.prims = d_prims;
  G.comps = d_comps;
  G.px = soa;
  G.py = soa + n_pts;
  G.pz = soa + 2 * (size_t)n_pts;
  G.pw = soa + 3 * (size_t)n_pts;
  G.batches = bd;
  G.cand_shells = d_cand_shells;
  G.cand_loc = cand_loc;
  G.batch_ao = batch_ao;
  G.order = order;
  EvalArgs A{};
  A.mode = kModeRks;
  A.xc = xc_code;
  A.Pa = d_total;
  A.Va = d_v;
  A.batch_red = red;
  A.counter = status + 1;
  A.slab = slab;
  A.slab_stride = slab_stride;
  A.max_m = max_batch_ao;
  ok = cudaMemsetAsync(d_v, 0, nn * sizeof(double), st) == cudaSuccess &&
       launch_fp64(G, A, n_ctas, st) == cudaSuccess && launch_reduce(red, n_batches, d_result, 2, st) == cudaSuccess &&
       launch_mirror(d_v, n_ao, 0, st) == cudaSuccess && cudaStreamSynchronize(st) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return -5;
  }
  return 0;
}
