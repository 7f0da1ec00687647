// grid_build.cu -- molecular grid construction on the GPU (FP64).
//
// The host enumerates the radial shells (atom, r, w_rad, Lebedev rule); the device expands every
// shell into its Lebedev points, evaluates the screened Becke partition weight of each point in
// FP64 and keeps points with w = w_rad w_ang B > 1e-18, preserving CalChem's point order
// (atom-major, radial-shell-major, Lebedev order: grid.rs:732-828).  The Becke weight is CalChem's
// two-pass screened form (grid.rs:338-419): pass 1 multiplies the host atom's cell function over
// all neighbours with an early exit below 1e-20 and marks neighbours with 1 - s > 1e-17 as
// active; pass 2 adds the cell functions of the active neighbours.  Here pass 2 re-derives the
// active set instead of storing it, which gives the same values without per-thread arrays.
//
// This file is compiled with -fmad=false: no multiply-add contraction, so every product and sum
// rounds as in the reference and the GPU grid matches the CPU grid point for point.
#include <cuda_runtime.h>

#include "grid_build.h"

namespace cxc {

namespace {

__device__ __forceinline__ double step3(double nu) {
  if (nu <= -1.0) return 1.0;
  if (nu >= 1.0) return 0.0;
  const double f1 = 0.5 * nu * (3.0 - nu * nu);
  const double f2 = 0.5 * f1 * (3.0 - f1 * f1);
  const double f3 = 0.5 * f2 * (3.0 - f2 * f2);
  return 0.5 * (1.0 - f3);
}

__device__ __forceinline__ double dist_to(const double* __restrict__ xyz, int a, double x, double y, double z) {
  const double dx = x - xyz[3 * a], dy = y - xyz[3 * a + 1], dz = z - xyz[3 * a + 2];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

__device__ __forceinline__ double clamp1(double v) { return v < -1.0 ? -1.0 : (v > 1.0 ? 1.0 : v); }

// Molecules with at most this many atoms keep every point-atom distance of pass 1 in a per-thread
// array, which pass 2 reads instead of recomputing an FP64 square root per (active atom, atom) pair;
// the values are the same, so the weights are too.
constexpr int kBeckeDistCache = 256;

__device__ double becke_weight(int n, const double* __restrict__ xyz, const double* __restrict__ inv_r,
                               const double* __restrict__ a_ij, int host, double x, double y, double z) {
  if (n <= 1) return 1.0;
  double rd[kBeckeDistCache];
  const bool cached = n <= kBeckeDistCache;
  const double r_host = dist_to(xyz, host, x, y, z);
  const size_t row_h = (size_t)host * n;
  double p_host = 1.0;
  int n_active = 0;
  int b_done = 0;  // distances rd[0 .. b_done) are filled
  for (int b = 0; b < n; ++b) {
    if (cached) {
      rd[b] = b == host ? r_host : dist_to(xyz, b, x, y, z);
      b_done = b + 1;
    }
    if (b == host) continue;
    const double inv = inv_r[row_h + b];
    if (inv == 0.0) continue;
    const double r_b = cached ? rd[b] : dist_to(xyz, b, x, y, z);
    const double mu = clamp1((r_host - r_b) * inv);
    const double nu = mu + a_ij[row_h + b] * (1.0 - mu * mu);
    const double s = step3(nu);
    p_host *= s;
    if (p_host < 1e-20) return 0.0;
    if (1.0 - s > 1e-17) ++n_active;
  }
  if (n_active == 0) return 1.0;
  if (cached)  // pass 1 ran to the end (it returns early only with p_host < 1e-20)
    for (int b = b_done; b < n; ++b) rd[b] = dist_to(xyz, b, x, y, z);
  double sum_p = p_host;
  for (int a = 0; a < n; ++a) {
    if (a == host) continue;
    const double inv_ha = inv_r[row_h + a];
    if (inv_ha == 0.0) continue;
    const double r_a = cached ? rd[a] : dist_to(xyz, a, x, y, z);
    const double mu_ha = clamp1((r_host - r_a) * inv_ha);
    const double s_ha = step3(mu_ha + a_ij[row_h + a] * (1.0 - mu_ha * mu_ha));
    if (!(1.0 - s_ha > 1e-17)) continue;
    double p_a = 1.0 - s_ha;
    if (p_a < 1e-20) continue;
    const size_t row_a = (size_t)a * n;
    for (int b = 0; b < n; ++b) {
      if (b == host || b == a) continue;
      const double inv = inv_r[row_a + b];
      if (inv == 0.0) continue;
      const double mu = clamp1((r_a - (cached ? rd[b] : dist_to(xyz, b, x, y, z))) * inv);
      p_a *= step3(mu + a_ij[row_a + b] * (1.0 - mu * mu));
      if (p_a < 1e-20) break;
    }
    sum_p += p_a;
  }
  return sum_p <= 0.0 ? 0.0 : p_host / sum_p;
}

// One CTA per radial shell: expand, weight, flag, count kept points.
constexpr int kShellThreads = 256;
__global__ void __launch_bounds__(kShellThreads) shell_points_kernel(GridBuildArgs a) {
  const int sh = blockIdx.x;
  const RadialShellDev rs = a.shells[sh];
  const double ax = a.xyz[3 * rs.atom], ay = a.xyz[3 * rs.atom + 1], az = a.xyz[3 * rs.atom + 2];
  __shared__ int s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  int cnt = 0;
  for (int j = threadIdx.x; j < rs.n_ang; j += blockDim.x) {
    const double* u = a.lebedev + 4 * (size_t)(rs.leb_offset + j);
    const double raw_w = rs.w_rad * u[3];
    const double x = ax + rs.r * u[0], y = ay + rs.r * u[1], z = az + rs.r * u[2];
    const double bw = becke_weight(a.n_atoms, a.xyz, a.inv_r, a.a_ij, rs.atom, x, y, z);
    const double w = raw_w * bw;
    const long long k = rs.raw_start + j;
    a.raw[4 * k] = x;
    a.raw[4 * k + 1] = y;
    a.raw[4 * k + 2] = z;
    a.raw[4 * k + 3] = w;
    a.raw_w[k] = raw_w;
    const int keep = w > 1e-18 ? 1 : 0;
    a.flags[k] = (unsigned char)keep;
    cnt += keep;
  }
  atomicAdd(&s_cnt, cnt);
  __syncthreads();
  if (threadIdx.x == 0) a.counts[sh] = s_cnt;
}

// Exclusive scan of the per-shell counts (one CTA, sequential chunks).
__global__ void __launch_bounds__(1024) scan_counts_kernel(const int* __restrict__ counts, int n,
                                                           long long* __restrict__ offsets) {
  __shared__ long long s[1024];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const long long v = i < n ? counts[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const long long t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) offsets[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) offsets[n] = carry;
}

// Order-preserving compaction of each shell's kept points.
__global__ void __launch_bounds__(256) compact_kernel(GridBuildArgs a, const long long* __restrict__ offsets) {
  const int sh = blockIdx.x;
  const RadialShellDev rs = a.shells[sh];
  __shared__ int warp_tot[8];
  __shared__ int s_base;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j0 = 0; j0 < rs.n_ang; j0 += 256) {
    const int j = j0 + threadIdx.x;
    const long long k = rs.raw_start + j;
    const int keep = (j < rs.n_ang) ? (int)a.flags[k] : 0;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    const int before_in_warp = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) warp_tot[wid] = __popc(bal);
    __syncthreads();
    int before = s_base;
    for (int w = 0; w < wid; ++w) before += warp_tot[w];
    if (keep) {
      const long long dst = offsets[sh] + before + before_in_warp;
      a.out_xyzw[4 * dst] = a.raw[4 * k];
      a.out_xyzw[4 * dst + 1] = a.raw[4 * k + 1];
      a.out_xyzw[4 * dst + 2] = a.raw[4 * k + 2];
      a.out_xyzw[4 * dst + 3] = a.raw[4 * k + 3];
      a.out_raw_w[dst] = a.raw_w[k];
      a.out_host[dst] = rs.atom;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < 8; ++w) t += warp_tot[w];
      s_base += t;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_grid_expand(const GridBuildArgs& a, int n_shells, cudaStream_t st) {
  shell_points_kernel<<<n_shells, kShellThreads, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_grid_scan(const int* counts, int n, long long* offsets, cudaStream_t st) {
  scan_counts_kernel<<<1, 1024, 0, st>>>(counts, n, offsets);
  return cudaGetLastError();
}

cudaError_t launch_grid_compact(const GridBuildArgs& a, const long long* offsets, int n_shells, cudaStream_t st) {
  compact_kernel<<<n_shells, 256, 0, st>>>(a, offsets);
  return cudaGetLastError();
}

}  // namespace cxc
