// vxc_fp64.cu -- plain all-FP64 XC quadrature kernels (the drop-in form).
//
// One persistent CTA works through a device queue of 128-point batches, largest first.  For each
// batch it
//   (A) evaluates the candidate AOs phi, d/dx phi, d/dy phi, d/dz phi at the batch's points into a
//       per-CTA scratch slab (rows = local AO, columns = point), with the reference's screening
//       (shell cutoff r^2 > (40+4l)/alpha_min, radial parts below 1e-18, components whose value and
//       gradient are all <= 1e-16 left at zero: ao_grid.rs:182-230);
//   (B) forms T = D_sub Phi tile by tile and reduces rho_g = sum_i Phi_ig T_ig and
//       grad rho_g = 2 sum_i grad Phi_ig T_ig without storing T (vxc.rs:859-888);
//   (C) evaluates the functional in FP64, one thread per point, and reduces the batch's Exc and
//       electron count (vxc.rs:890-920);
//   (D) builds Z = (w v_rho / 2) Phi + (w u) . grad Phi (vxc.rs:925-939);
//   (E) accumulates the symmetric rank-2k update W = Z Phi^T + Phi Z^T on lower-triangular tile
//       pairs and adds it into V with one FP64 atomic per (batch, AO pair) (vxc.rs:941-960) --
//       the reference GPU kernel adds once per (point, AO pair) (cuda_kernels.cu:469-480).
// The drop-in eval_rho / accum entry points reuse phases A+B and A+D+E with the per-point values
// supplied by the caller.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "xc_device.cuh"

namespace cxc {

constexpr int kThreads = 256;
constexpr int kRowTile = 64;
constexpr int kKTile = 32;
constexpr int kWTile = 32;
constexpr int kWChunk = 64;
constexpr int kWPitch = kWChunk + 1;

struct Fp64Smem {
  union {
    struct {
      double ds[kRowTile][kKTile];   // D_sub tile
      double ps[kKTile][kBlockPts];  // Phi tile
    } t;
    struct {
      double zi[kWTile][kWPitch];
      double fi[kWTile][kWPitch];
      double zj[kWTile][kWPitch];
      double fj[kWTile][kWPitch];
    } w;
  } u;
  double coef[8][kBlockPts];     // per point: (c0, cx, cy, cz) for alpha then beta
  double dens[2][4][kBlockPts];  // rho and grad partial sums (per half)
  double red[3][kThreads / 32];
  int batch;
};

__host__ size_t fp64_smem_bytes() { return sizeof(Fp64Smem); }

__device__ __forceinline__ void pow_d1(double x, int l, double& p, double& d) {
  if (l == 0) { p = 1.0; d = 0.0; }
  else if (l == 1) { p = x; d = 1.0; }
  else if (l == 2) { p = x * x; d = 2.0 * x; }
  else { p = x * x * x; d = 3.0 * x * x; }
}

// (A) AO values and gradients of the batch into the slab planes 0..3.
__device__ void eval_batch_aos(const DevGrid& G, const BatchDesc& bd, double* __restrict__ slab, int m_pad) {
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const bool live = g < bd.n_pts;
  double x = 0, y = 0, z = 0;
  if (live) {
    x = G.px[bd.pt_start + g];
    y = G.py[bd.pt_start + g];
    z = G.pz[bd.pt_start + g];
  }
  const size_t plane = (size_t)m_pad * kBlockPts;
  for (int ci = tid >> 7; ci < bd.n_cand; ci += kThreads / kBlockPts) {
    const AoShellGpu sh = G.shells[G.cand_shells[bd.cand_start + ci]];
    const int loc = G.cand_loc[bd.cand_start + ci];
    double r0 = 0.0, r1 = 0.0, dx = 0, dy = 0, dz = 0;
    bool on = false;
    if (live) {
      dx = x - sh.center[0];
      dy = y - sh.center[1];
      dz = z - sh.center[2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (!(r2 > sh.r2_cutoff)) {
        for (int p = 0; p < sh.n_prims; ++p) {
          const AoPrimGpu pr = G.prims[sh.prim_start + p];
          const double e = pr.weighted_norm * exp(-pr.exponent * r2);
          r0 += e;
          r1 -= 2.0 * pr.exponent * e;
        }
        on = !(fabs(r0) < 1e-18 && fabs(r1) < 1e-18);
      }
    }
    for (int c = 0; c < sh.n_funcs; ++c) {
      double v = 0, gx = 0, gy = 0, gz = 0;
      if (on) {
        const AoCompGpu cp = G.comps[sh.comp_start + c];
        double px, dpx, py, dpy, pz, dpz;
        pow_d1(dx, cp.lx, px, dpx);
        pow_d1(dy, cp.ly, py, dpy);
        pow_d1(dz, cp.lz, pz, dpz);
        const double mm = px * py * pz;
        v = cp.scale * mm * r0;
        gx = cp.scale * (dpx * py * pz * r0 + mm * dx * r1);
        gy = cp.scale * (px * dpy * pz * r0 + mm * dy * r1);
        gz = cp.scale * (px * py * dpz * r0 + mm * dz * r1);
        if (!(fabs(v) > 1e-16 || fabs(gx) > 1e-16 || fabs(gy) > 1e-16 || fabs(gz) > 1e-16)) v = gx = gy = gz = 0;
      }
      const size_t o = (size_t)(loc + c) * kBlockPts + g;
      slab[o] = v;
      slab[plane + o] = gx;
      slab[2 * plane + o] = gy;
      slab[3 * plane + o] = gz;
    }
  }
}

// (B) rho and grad rho (unscaled sum of grad Phi T) of density P for the batch; result in dens[0][..]
// after the call (summed over both halves).
__device__ void batch_density(const DevGrid& G, const BatchDesc& bd, const double* __restrict__ P,
                              const double* __restrict__ slab, int m_pad, Fp64Smem& S) {
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const int h = tid >> 7;
  const int m = bd.m;
  const int n = mol_nao(G, bd.mol);
  P += mol_mat(G, bd.mol);
  const int* __restrict__ ao = G.batch_ao + bd.ao_start;
  const size_t plane = (size_t)m_pad * kBlockPts;
  double rho = 0, sx = 0, sy = 0, sz = 0;
  for (int I = 0; I < m; I += kRowTile) {
    double acc[32];
#pragma unroll
    for (int r = 0; r < 32; ++r) acc[r] = 0.0;
    for (int K = 0; K < m; K += kKTile) {
      __syncthreads();
      for (int e = tid; e < kRowTile * kKTile; e += kThreads) {
        const int r = e / kKTile, kk = e % kKTile;
        const int i = I + r, k = K + kk;
        S.u.t.ds[r][kk] = (i < m && k < m) ? P[(size_t)ao[i] * n + ao[k]] : 0.0;
      }
      for (int e = tid; e < kKTile * kBlockPts; e += kThreads) {
        const int kk = e / kBlockPts, gg = e % kBlockPts;
        const int k = K + kk;
        S.u.t.ps[kk][gg] = k < m ? slab[(size_t)k * kBlockPts + gg] : 0.0;
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < kKTile; ++kk) {
        const double ph = S.u.t.ps[kk][g];
#pragma unroll
        for (int r = 0; r < 32; ++r) acc[r] = fma(S.u.t.ds[h * 32 + r][kk], ph, acc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < 32; ++r) {
      const int i = I + h * 32 + r;
      if (i < m) {
        const size_t o = (size_t)i * kBlockPts + g;
        const double t = acc[r];
        rho += slab[o] * t;
        sx += slab[plane + o] * t;
        sy += slab[2 * plane + o] * t;
        sz += slab[3 * plane + o] * t;
      }
    }
  }
  S.dens[h][0][g] = rho;
  S.dens[h][1][g] = sx;
  S.dens[h][2][g] = sy;
  S.dens[h][3][g] = sz;
  __syncthreads();
  if (h == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) S.dens[0][q][g] += S.dens[1][q][g];
  }
  __syncthreads();
}

// (D) Z plane for spin s from coef[4s..4s+3].
__device__ void build_z(const BatchDesc& bd, double* __restrict__ slab, int m_pad, int zplane, const Fp64Smem& S,
                        int s) {
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const size_t plane = (size_t)m_pad * kBlockPts;
  const double c0 = S.coef[4 * s][g], cx = S.coef[4 * s + 1][g], cy = S.coef[4 * s + 2][g],
               cz = S.coef[4 * s + 3][g];
  for (int i = tid >> 7; i < bd.m; i += 2) {
    const size_t o = (size_t)i * kBlockPts + g;
    slab[zplane * plane + o] = c0 * slab[o] + cx * slab[plane + o] + cy * slab[2 * plane + o] + cz * slab[3 * plane + o];
  }
}

// (E) V_lower += Z Phi^T + Phi Z^T over the batch (zplane holds Z).
__device__ void accumulate_v(const DevGrid& G, const BatchDesc& bd, const double* __restrict__ slab, int m_pad,
                             int zplane, double* __restrict__ V, Fp64Smem& S) {
  const int tid = threadIdx.x;
  const int m = bd.m;
  const int n = mol_nao(G, bd.mol);
  V += mol_mat(G, bd.mol);
  const int* __restrict__ ao = G.batch_ao + bd.ao_start;
  const size_t plane = (size_t)m_pad * kBlockPts;
  const double* __restrict__ phi = slab;
  const double* __restrict__ zz = slab + zplane * plane;
  const int ti = tid / 16, tj = tid % 16;
  const int np = bd.n_pts;
  for (int I = 0; I < m; I += kWTile) {
    for (int J = 0; J <= I; J += kWTile) {
      double a00 = 0, a01 = 0, a10 = 0, a11 = 0;
      for (int G0 = 0; G0 < np; G0 += kWChunk) {
        __syncthreads();
        for (int e = tid; e < kWTile * kWChunk; e += kThreads) {
          const int r = e / kWChunk, gg = e % kWChunk;
          const int gi = G0 + gg;
          const int i = I + r, j = J + r;
          const bool gok = gi < np;
          S.u.w.zi[r][gg] = (gok && i < m) ? zz[(size_t)i * kBlockPts + gi] : 0.0;
          S.u.w.fi[r][gg] = (gok && i < m) ? phi[(size_t)i * kBlockPts + gi] : 0.0;
          S.u.w.zj[r][gg] = (gok && j < m) ? zz[(size_t)j * kBlockPts + gi] : 0.0;
          S.u.w.fj[r][gg] = (gok && j < m) ? phi[(size_t)j * kBlockPts + gi] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int gg = 0; gg < kWChunk; ++gg) {
          const double z0 = S.u.w.zi[2 * ti][gg], z1 = S.u.w.zi[2 * ti + 1][gg];
          const double f0 = S.u.w.fi[2 * ti][gg], f1 = S.u.w.fi[2 * ti + 1][gg];
          const double q0 = S.u.w.fj[2 * tj][gg], q1 = S.u.w.fj[2 * tj + 1][gg];
          const double y0 = S.u.w.zj[2 * tj][gg], y1 = S.u.w.zj[2 * tj + 1][gg];
          a00 = fma(z0, q0, fma(f0, y0, a00));
          a01 = fma(z0, q1, fma(f0, y1, a01));
          a10 = fma(z1, q0, fma(f1, y0, a10));
          a11 = fma(z1, q1, fma(f1, y1, a11));
        }
      }
      const double vals[4] = {a00, a01, a10, a11};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = I + 2 * ti + (q >> 1), j = J + 2 * tj + (q & 1);
        if (i < m && j < m && i >= j) {
          const int mi = ao[i], mj = ao[j];
          const int r = mi >= mj ? mi : mj, c = mi >= mj ? mj : mi;
          atomicAdd(&V[(size_t)r * n + c], vals[q]);
        }
      }
    }
  }
}

__device__ __forceinline__ double block_sum(double v, double* red_row) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red_row[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < kThreads / 32; ++k) s += red_row[k];
  return s;  // valid in thread 0
}

__global__ void __launch_bounds__(kThreads, 1) vxc_fp64_kernel(DevGrid G, EvalArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Fp64Smem& S = *reinterpret_cast<Fp64Smem*>(smem_raw);
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  double* slab = A.slab + (size_t)blockIdx.x * A.slab_stride;
  const int m_pad = (A.max_m + kRowTile - 1) / kRowTile * kRowTile;
  const bool uks = A.mode == kModeUks;

  while (true) {
    if (tid == 0) S.batch = atomicAdd(A.counter, 1);
    __syncthreads();
    const int q = S.batch;
    __syncthreads();
    if (q >= G.n_batches) break;
    const int b = G.order[q];
    const BatchDesc bd = G.batches[b];
    eval_batch_aos(G, bd, slab, m_pad);
    __syncthreads();
    if (A.mode == kModeFxc) {
      // The batch's AOs serve every trial matrix: response density eta = sum M phi phi and its
      // gradient xi, the kernel-weighted coefficients, then dV_b += Z Phi^T + Phi Z^T.
      const size_t nn = (size_t)G.n_ao * G.n_ao;
      for (int t = 0; t < A.n_trials; ++t) {
        batch_density(G, bd, A.Pa + t * nn, slab, m_pad, S);
        if (tid < kBlockPts) {
          const bool live = g < bd.n_pts;
          const size_t pt = (size_t)bd.pt_start + g;
          for (int k = 0; k < 4; ++k) S.coef[k][g] = 0.0;
          if (live) {
            const double* c = A.fxc_coef + 11 * pt;
            const double* kc = c + (A.triplet ? 7 : 3);
            const double w = G.pw[pt];
            const double eta = S.dens[0][0][g];
            const double xi[3] = {2.0 * S.dens[0][1][g], 2.0 * S.dens[0][2][g], 2.0 * S.dens[0][3][g]};
            const double sigma = c[0] * xi[0] + c[1] * xi[1] + c[2] * xi[2];
            const double dv = kc[0] * eta + kc[1] * sigma;
            const double gc = kc[1] * eta + kc[2] * sigma;
            S.coef[0][g] = 0.5 * w * dv;
            S.coef[1][g] = w * (kc[3] * xi[0] + gc * c[0]);
            S.coef[2][g] = w * (kc[3] * xi[1] + gc * c[1]);
            S.coef[3][g] = w * (kc[3] * xi[2] + gc * c[2]);
          }
        }
        __syncthreads();
        build_z(bd, slab, m_pad, 4, S, 0);
        __syncthreads();
        accumulate_v(G, bd, slab, m_pad, 4, A.Va + t * nn, S);
        __syncthreads();
      }
      continue;
    }

    double e_loc = 0, na_loc = 0, nb_loc = 0;
    if (A.mode == kModeAccum) {
      if (tid < kBlockPts) {
        const bool live = g < bd.n_pts;
#pragma unroll
        for (int k = 0; k < 4; ++k) S.coef[k][g] = live ? A.wv_in[4 * (size_t)(bd.pt_start + g) + k] : 0.0;
      }
    } else {
      batch_density(G, bd, A.Pa, slab, m_pad, S);
      double ra = 0, gax = 0, gay = 0, gaz = 0;
      if (tid < kBlockPts) {
        ra = S.dens[0][0][g];
        gax = 2.0 * S.dens[0][1][g];
        gay = 2.0 * S.dens[0][2][g];
        gaz = 2.0 * S.dens[0][3][g];
      }
      __syncthreads();
      if (uks) batch_density(G, bd, A.Pb, slab, m_pad, S);
      if (tid < kBlockPts) {
        const bool live = g < bd.n_pts;
        const size_t pt = (size_t)bd.pt_start + g;
        for (int k = 0; k < 8; ++k) S.coef[k][g] = 0.0;
        if (A.mode == kModeRho) {
          if (live) {
            A.rho_out[4 * pt] = ra;
            A.rho_out[4 * pt + 1] = gax;
            A.rho_out[4 * pt + 2] = gay;
            A.rho_out[4 * pt + 3] = gaz;
          }
        } else if (!uks) {
          if (live && !(ra < 1e-18)) {
            const double w = G.pw[pt];
            const double rs = 0.5 * ra;
            const double gss = 0.25 * (gax * gax + gay * gay + gaz * gaz);
            const XcVal o = xc_eval(A.xc, rs, rs, gss, gss, gss);
            e_loc = w * o.f;
            na_loc = w * ra;
            S.coef[0][g] = 0.5 * w * o.vra;
            const double us = w * (o.vgaa + 0.5 * o.vgab);
            S.coef[1][g] = us * gax;
            S.coef[2][g] = us * gay;
            S.coef[3][g] = us * gaz;
            if (A.point_out) {
              A.point_out[2 * pt] = e_loc;
              A.point_out[2 * pt + 1] = w * o.vra * ra + us * (gax * gax + gay * gay + gaz * gaz);
            }
          }
        } else {
          const double rb0 = S.dens[0][0][g];
          const double gbx = 2.0 * S.dens[0][1][g], gby = 2.0 * S.dens[0][2][g], gbz = 2.0 * S.dens[0][3][g];
          const double rpa = fmax(ra, 0.0), rpb = fmax(rb0, 0.0);
          if (live && !(rpa + rpb < 1e-18)) {
            const double w = G.pw[pt];
            const double gaa = gax * gax + gay * gay + gaz * gaz;
            const double gab = gax * gbx + gay * gby + gaz * gbz;
            const double gbb = gbx * gbx + gby * gby + gbz * gbz;
            const XcVal o = xc_eval(A.xc, rpa, rpb, gaa, gab, gbb);
            e_loc = w * o.f;
            na_loc = w * rpa;
            nb_loc = w * rpb;
            S.coef[0][g] = 0.5 * w * o.vra;
            S.coef[1][g] = w * (2.0 * o.vgaa * gax + o.vgab * gbx);
            S.coef[2][g] = w * (2.0 * o.vgaa * gay + o.vgab * gby);
            S.coef[3][g] = w * (2.0 * o.vgaa * gaz + o.vgab * gbz);
            S.coef[4][g] = 0.5 * w * o.vrb;
            S.coef[5][g] = w * (2.0 * o.vgbb * gbx + o.vgab * gax);
            S.coef[6][g] = w * (2.0 * o.vgbb * gby + o.vgab * gay);
            S.coef[7][g] = w * (2.0 * o.vgbb * gbz + o.vgab * gaz);
          }
        }
      }
    }
    __syncthreads();
    if (A.mode == kModeRks || A.mode == kModeUks) {
      const double es = block_sum(e_loc, S.red[0]);
      const double nas = block_sum(na_loc, S.red[1]);
      const double nbs = block_sum(nb_loc, S.red[2]);
      if (tid == 0) {
        A.batch_red[3 * (size_t)b] = es;
        A.batch_red[3 * (size_t)b + 1] = nas;
        A.batch_red[3 * (size_t)b + 2] = nbs;
      }
    }
    if (A.mode != kModeRho && !A.shares_only) {
      build_z(bd, slab, m_pad, 4, S, 0);
      __syncthreads();
      accumulate_v(G, bd, slab, m_pad, 4, A.Va, S);
      if (uks) {
        __syncthreads();
        build_z(bd, slab, m_pad, 4, S, 1);
        __syncthreads();
        accumulate_v(G, bd, slab, m_pad, 4, A.Vb, S);
      }
    }
    __syncthreads();
  }
}

// Deterministic final reduction of the per-batch (Exc, N_a, N_b) partials.
__global__ void __launch_bounds__(256) reduce_batches_kernel(const double* __restrict__ part, int n_batches,
                                                             const int* __restrict__ batch_off,
                                                             double* __restrict__ out, int n_out) {
  __shared__ double s[3][256];
  const int t = threadIdx.x;
  // one CTA per molecule: its batches are [batch_off[mol], batch_off[mol + 1])
  const int b0 = batch_off ? batch_off[blockIdx.x] : 0;
  const int b1 = batch_off ? batch_off[blockIdx.x + 1] : n_batches;
  out += (size_t)blockIdx.x * n_out;
  double a = 0, b = 0, c = 0;
  for (int i = b0 + t; i < b1; i += 256) {
    a += part[3 * (size_t)i];
    b += part[3 * (size_t)i + 1];
    c += part[3 * (size_t)i + 2];
  }
  s[0][t] = a;
  s[1][t] = b;
  s[2][t] = c;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (t < o) {
      s[0][t] += s[0][t + o];
      s[1][t] += s[1][t + o];
      s[2][t] += s[2][t + o];
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = s[0][0];
    if (n_out == 2) out[1] = s[1][0] + s[2][0];
    else { out[1] = s[1][0]; out[2] = s[2][0]; }
  }
}

// Per-atom sums of the per-point shares (point_out[2 g], point_out[2 g + 1]): one CTA per atom over
// its points atom_pts[atom_off[a] .. atom_off[a + 1]) (planned point indices, ascending), strided
// partial sums and a fixed tree, so the result does not depend on scheduling.
__global__ void __launch_bounds__(256) atom_shares_kernel(const double* __restrict__ point_out,
                                                          const int* __restrict__ atom_pts,
                                                          const int* __restrict__ atom_off, double* __restrict__ out) {
  __shared__ double s[2][256];
  const int t = threadIdx.x, a = blockIdx.x;
  double e = 0, v = 0;
  for (int k = atom_off[a] + t; k < atom_off[a + 1]; k += 256) {
    const int g = atom_pts[k];
    e += point_out[2 * (size_t)g];
    v += point_out[2 * (size_t)g + 1];
  }
  s[0][t] = e;
  s[1][t] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (t < o) {
      s[0][t] += s[0][t + o];
      s[1][t] += s[1][t + o];
    }
    __syncthreads();
  }
  if (t == 0) {
    out[2 * (size_t)a] = s[0][0];
    out[2 * (size_t)a + 1] = s[1][0];
  }
}

// Completes a symmetric matrix from one triangle: from_upper = 0 copies the lower triangle into
// the upper one (FP64 path), from_upper = 1 the upper into the lower (tensor-core path).
__global__ void mirror_kernel(double* __restrict__ V, int n_single, const int* __restrict__ mol_n,
                              const long long* __restrict__ mol_off, int from_upper) {
  // blockIdx.y = molecule; grid-stride over its n^2 elements
  const int n = mol_n ? mol_n[blockIdx.y] : n_single;
  double* Vm = V + (mol_off ? mol_off[blockIdx.y] : 0ll);
  const size_t nn = (size_t)n * n;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / n), j = (int)(idx % n);
    if (from_upper ? (j < i) : (j > i)) Vm[idx] = Vm[(size_t)j * n + i];
  }
}

}  // namespace cxc

// Launch helpers used by the C ABI layer.
namespace cxc {

cudaError_t fp64_set_attributes() {
  static bool attr_set = false;
  if (attr_set) return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(vxc_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Fp64Smem));
  if (e == cudaSuccess) attr_set = true;
  return e;
}

cudaError_t launch_fp64(const DevGrid& G, const EvalArgs& A, int n_ctas, cudaStream_t st) {
  const cudaError_t e = fp64_set_attributes();
  if (e != cudaSuccess) return e;
  vxc_fp64_kernel<<<n_ctas, kThreads, sizeof(Fp64Smem), st>>>(G, A);
  return cudaGetLastError();
}

cudaError_t launch_reduce(const double* part, int n_batches, const int* batch_off, int n_mols, double* out, int n_out,
                          cudaStream_t st) {
  reduce_batches_kernel<<<n_mols, 256, 0, st>>>(part, n_batches, batch_off, out, n_out);
  return cudaGetLastError();
}

cudaError_t launch_reduce(const double* part, int n_batches, double* out, int n_out, cudaStream_t st) {
  return launch_reduce(part, n_batches, nullptr, 1, out, n_out, st);
}

cudaError_t launch_mirror(double* V, int max_n, const int* mol_n, const long long* mol_off, int n_mols, int from_upper,
                          cudaStream_t st) {
  const size_t nn = (size_t)max_n * max_n;
  const unsigned bx = (unsigned)std::min<size_t>((nn + 255) / 256, 4096);
  mirror_kernel<<<dim3(bx, (unsigned)n_mols), 256, 0, st>>>(V, max_n, mol_n, mol_off, from_upper);
  return cudaGetLastError();
}

cudaError_t launch_mirror(double* V, int n, int from_upper, cudaStream_t st) {
  return launch_mirror(V, n, nullptr, nullptr, 1, from_upper, st);
}

cudaError_t launch_atom_shares(const double* point_out, const int* atom_pts, const int* atom_off, int n_atoms,
                               double* out, cudaStream_t st) {
  atom_shares_kernel<<<n_atoms, 256, 0, st>>>(point_out, atom_pts, atom_off, out);
  return cudaGetLastError();
}

}  // namespace cxc
