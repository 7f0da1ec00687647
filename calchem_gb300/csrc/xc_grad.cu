// xc_grad.cu -- XC nuclear gradient dExc/dR_A at fixed spin densities, all FP64.
//
// The quantity is CalChem's xc_nuclear_gradient (vxc.rs:1769-1912, 1903-1912):
//   dExc/dR_A = -2 sum_g sum_s sum_{i on A} [ (w v_rho_s dphi_i + (w u_s . Hphi_i)) (P_s phi)_i
//                                               + dphi_i (P_s (w u_s . grad phi))_i ]
//               + (host-atom term: minus the same sum over all AOs, for every point of A's cells)
//               + sum_g raw_w_g f_g d(Becke weight_g)/dR_A        (grid.rs:423-584)
// with u_a = 2 v_gamma_aa grad rho_a + v_gamma_ab grad rho_b (and a <-> b).
//
// One persistent CTA of 256 threads takes 128-point batches from a device queue.  Per batch:
//   (A) phi, grad phi and the six second derivatives of every candidate AO at the batch's points
//       into ten planes of a per-CTA scratch slab (screening of ao_grid.rs for the Hessian form:
//       shell cutoff r^2 > r2_cutoff; radial value, slope and curvature all below 1e-18);
//   (B) T_s = P_s Phi by 64-row x 32-deep tiles (stored: plane 12 / 13), then rho_s and grad rho_s;
//   (C) the functional per point: (w v_rho_s, w u_s) and f (vxc.rs:1830-1860);
//   (D) psi_s = (w u_s) . grad phi, and Y_s = P_s Psi_s by the same tiles; the tile epilogue forms
//       each AO row's force from T, Y, grad phi and the Hessian, reduces it over the points with
//       warp shuffles and adds it, row by row in a fixed order, into the batch's per-atom sums;
//       every point's total goes to its host atom with the opposite sign;
//   (E) the Becke weight derivative, one warp per point, lanes over atoms (two passes of O(n^2)
//       pair terms: cell functions, then the derivative of P_host / Z for every atom but the host,
//       whose term is minus their sum);
//   (F) the batch's per-atom sums go to its own row of a [batch][atom][3] array; a second kernel
//       adds the rows in batch order.  Results are therefore deterministic.
// The drop-in form (calchem_cuda_vxc_grad_force, cuda_kernels.cu:4351-4580) skips (B), (C) and
// (E): the per-point coefficients come from the caller, and only the AO term is returned.
#include <cuda_runtime.h>

#include "becke_grad.cuh"
#include "common.cuh"
#include "launch.h"
#include "xc_device.cuh"

namespace cxc {

namespace {

using becke::BeckeScratch;
using becke::becke_point;
using becke::becke_scratch_doubles;

constexpr int kGT = 256;        // threads
constexpr int kGRows = 64;      // AO rows per tile (32 per half)
constexpr int kGK = 32;         // depth per tile
constexpr int kGWarps = kGT / 32;
constexpr int kPtsPerWarp = kBlockPts / kGWarps;
// slab planes
constexpr int kPhi = 0, kGrad = 1, kHess = 4, kPsi = 10, kT = 12;
constexpr int kGradPlanes = 14;

struct GradSmem {
  double ds[kGRows][kGK];         // density tile
  double ps[kGK][kBlockPts];      // input-plane tile
  double coef[8][kBlockPts];      // (w v_rho_a, w u_a, w v_rho_b, w u_b) per point
  double dens[2][4][kBlockPts];   // rho and grad partial sums per half
  double fx[kBlockPts];           // energy density f per point (0: no Becke term)
  double red[kGWarps][32][3];     // warp sums of the row forces
  double hsum[2][3][kBlockPts];   // per point: sum of its row forces (per half)
  int row_atom[kGRows];           // atom of each row of the current tile
  int host[kBlockPts];            // host atom of each point of the batch
  int batch;
};

__device__ __forceinline__ void pow012(double x, int l, double& p, double& d, double& d2) {
  if (l == 0) { p = 1.0; d = 0.0; d2 = 0.0; }
  else if (l == 1) { p = x; d = 1.0; d2 = 0.0; }
  else if (l == 2) { p = x * x; d = 2.0 * x; d2 = 2.0; }
  else { p = x * x * x; d = 3.0 * x * x; d2 = 6.0 * x; }
}

// (A) values, gradients and Hessians (xx, xy, xz, yy, yz, zz) of the batch's AOs.
__device__ void eval_batch_hess(const DevGrid& G, const BatchDesc& bd, double* __restrict__ slab, size_t plane) {
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const bool live = g < bd.n_pts;
  double x = 0, y = 0, z = 0;
  if (live) {
    x = G.px[bd.pt_start + g];
    y = G.py[bd.pt_start + g];
    z = G.pz[bd.pt_start + g];
  }
  for (int ci = tid >> 7; ci < bd.n_cand; ci += kGT / kBlockPts) {
    const AoShellGpu sh = G.shells[G.cand_shells[bd.cand_start + ci]];
    const int loc = G.cand_loc[bd.cand_start + ci];
    double r0 = 0.0, r1 = 0.0, r2r = 0.0, dx = 0, dy = 0, dz = 0;
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
          r2r += 4.0 * pr.exponent * pr.exponent * e;
        }
        on = !(fabs(r0) < 1e-18 && fabs(r1) < 1e-18 && fabs(r2r) < 1e-18);
      }
    }
    for (int c = 0; c < sh.n_funcs; ++c) {
      double o[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) o[k] = 0.0;
      if (on) {
        const AoCompGpu cp = G.comps[sh.comp_start + c];
        double px, dpx, d2px, py, dpy, d2py, pz, dpz, d2pz;
        pow012(dx, cp.lx, px, dpx, d2px);
        pow012(dy, cp.ly, py, dpy, d2py);
        pow012(dz, cp.lz, pz, dpz, d2pz);
        const double s = cp.scale;
        const double mm = px * py * pz;
        const double m0 = dpx * py * pz, m1 = px * dpy * pz, m2 = px * py * dpz;
        o[0] = s * mm * r0;
        o[1] = s * (m0 * r0 + mm * dx * r1);
        o[2] = s * (m1 * r0 + mm * dy * r1);
        o[3] = s * (m2 * r0 + mm * dz * r1);
        o[4] = s * (d2px * py * pz * r0 + (2.0 * m0 * dx + mm) * r1 + mm * dx * dx * r2r);
        o[5] = s * (dpx * dpy * pz * r0 + (m0 * dy + m1 * dx) * r1 + mm * dx * dy * r2r);
        o[6] = s * (dpx * py * dpz * r0 + (m0 * dz + m2 * dx) * r1 + mm * dx * dz * r2r);
        o[7] = s * (px * d2py * pz * r0 + (2.0 * m1 * dy + mm) * r1 + mm * dy * dy * r2r);
        o[8] = s * (px * dpy * dpz * r0 + (m1 * dz + m2 * dy) * r1 + mm * dy * dz * r2r);
        o[9] = s * (px * py * d2pz * r0 + (2.0 * m2 * dz + mm) * r1 + mm * dz * dz * r2r);
      }
      const size_t off = (size_t)(loc + c) * kBlockPts + g;
#pragma unroll
      for (int k = 0; k < 10; ++k) slab[k * plane + off] = o[k];
    }
  }
}

struct ForceCtx {
  int spin;       // coefficient set (0: alpha, 1: beta)
  int t_plane;    // plane of T_s = P_s Phi
  double scale;   // -2, or -4 when the beta spin is the same as the alpha spin
  const int* ao_atom;
  double* acc;    // shared per-atom sums [3 n_atoms]
};

// OUT = P_sub IN over all rows of the batch.  kForce = false: OUT is stored into plane out_plane.
// kForce = true: OUT is Y_s and the epilogue adds the row forces (see the file comment).
template <bool kForce>
__device__ void contract(const DevGrid& G, const BatchDesc& bd, const double* __restrict__ P, double* __restrict__ slab,
                         size_t plane, int in_plane, int out_plane, GradSmem& S, const ForceCtx& F,
                         double (&hs)[3]) {
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const int h = tid >> 7;
  const int warp = tid >> 5, lane = tid & 31;
  const int m = bd.m;
  const int n = mol_nao(G, bd.mol);
  const int* __restrict__ ao = G.batch_ao + bd.ao_start;
  const double* __restrict__ in = slab + in_plane * plane;
  for (int I = 0; I < m; I += kGRows) {
    double acc[32];
#pragma unroll
    for (int r = 0; r < 32; ++r) acc[r] = 0.0;
    if (kForce) {
      __syncthreads();  // the previous tile's row sums have been added
      if (tid < kGRows) S.row_atom[tid] = I + tid < m ? F.ao_atom[ao[I + tid]] : 0;
    }
    for (int K = 0; K < m; K += kGK) {
      __syncthreads();
      for (int e = tid; e < kGRows * kGK; e += kGT) {
        const int r = e / kGK, kk = e % kGK;
        const int i = I + r, k = K + kk;
        S.ds[r][kk] = (i < m && k < m) ? P[(size_t)ao[i] * n + ao[k]] : 0.0;
      }
      for (int e = tid; e < kGK * kBlockPts; e += kGT) {
        const int kk = e / kBlockPts, gg = e % kBlockPts;
        const int k = K + kk;
        S.ps[kk][gg] = k < m ? in[(size_t)k * kBlockPts + gg] : 0.0;
      }
      __syncthreads();
#pragma unroll 4
      for (int kk = 0; kk < kGK; ++kk) {
        const double ph = S.ps[kk][g];
#pragma unroll
        for (int r = 0; r < 32; ++r) acc[r] = fma(S.ds[h * 32 + r][kk], ph, acc[r]);
      }
    }
    if (!kForce) {
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        const int i = I + h * 32 + r;
        if (i < m) slab[out_plane * plane + (size_t)i * kBlockPts + g] = acc[r];
      }
    } else {
      const double c0 = S.coef[4 * F.spin][g];
      const double u0 = S.coef[4 * F.spin + 1][g], u1 = S.coef[4 * F.spin + 2][g], u2 = S.coef[4 * F.spin + 3][g];
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        const int i = I + h * 32 + r;
        double v0 = 0, v1 = 0, v2 = 0;
        if (i < m) {
          const size_t o = (size_t)i * kBlockPts + g;
          const double t = slab[F.t_plane * plane + o];
          const double d0 = slab[(kGrad + 0) * plane + o], d1 = slab[(kGrad + 1) * plane + o],
                       d2 = slab[(kGrad + 2) * plane + o];
          const double hxx = slab[(kHess + 0) * plane + o], hxy = slab[(kHess + 1) * plane + o],
                       hxz = slab[(kHess + 2) * plane + o], hyy = slab[(kHess + 3) * plane + o],
                       hyz = slab[(kHess + 4) * plane + o], hzz = slab[(kHess + 5) * plane + o];
          const double uh0 = u0 * hxx + u1 * hxy + u2 * hxz;
          const double uh1 = u0 * hxy + u1 * hyy + u2 * hyz;
          const double uh2 = u0 * hxz + u1 * hyz + u2 * hzz;
          const double y = acc[r];
          v0 = F.scale * ((c0 * d0 + uh0) * t + d0 * y);
          v1 = F.scale * ((c0 * d1 + uh1) * t + d1 * y);
          v2 = F.scale * ((c0 * d2 + uh2) * t + d2 * y);
          hs[0] += v0;
          hs[1] += v1;
          hs[2] += v2;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          v0 += __shfl_xor_sync(0xffffffffu, v0, o);
          v1 += __shfl_xor_sync(0xffffffffu, v1, o);
          v2 += __shfl_xor_sync(0xffffffffu, v2, o);
        }
        if (lane == 0) {
          S.red[warp][r][0] = v0;
          S.red[warp][r][1] = v1;
          S.red[warp][r][2] = v2;
        }
      }
      __syncthreads();
      if (tid < 3) {
        for (int r = 0; r < kGRows && I + r < m; ++r) {
          const int hh = r >> 5, rr = r & 31;
          const double v = S.red[4 * hh][rr][tid] + S.red[4 * hh + 1][rr][tid] + S.red[4 * hh + 2][rr][tid] +
                           S.red[4 * hh + 3][rr][tid];
          F.acc[3 * S.row_atom[r] + tid] += v;
        }
      }
    }
  }
}

// (B) rho and the sum of grad phi T (half of grad rho) of spin plane t_plane into dens[0][..][g].
__device__ void density_from_t(const BatchDesc& bd, const double* __restrict__ slab, size_t plane, int t_plane,
                               GradSmem& S) {
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const int h = tid >> 7;
  double rho = 0, sx = 0, sy = 0, sz = 0;
  for (int i = h; i < bd.m; i += 2) {
    const size_t o = (size_t)i * kBlockPts + g;
    const double t = slab[t_plane * plane + o];
    rho += slab[o] * t;
    sx += slab[plane + o] * t;
    sy += slab[2 * plane + o] * t;
    sz += slab[3 * plane + o] * t;
  }
  __syncthreads();
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

__global__ void __launch_bounds__(kGT, 1) xc_grad_kernel(DevGrid G, GradArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GradSmem& S = *reinterpret_cast<GradSmem*>(smem_raw);
  double* acc = reinterpret_cast<double*>(smem_raw + sizeof(GradSmem));
  const int tid = threadIdx.x;
  const int g = tid & (kBlockPts - 1);
  const int h = tid >> 7;
  const int warp = tid >> 5, lane = tid & 31;
  const int na3 = 3 * A.n_atoms;
  const int m_pad = (A.max_m + kGRows - 1) / kGRows * kGRows;
  const size_t plane = (size_t)m_pad * kBlockPts;
  double* slab = A.slab + (size_t)blockIdx.x * A.slab_stride;
  // Becke scratch of each warp behind the planes: dist[n], cell[n], wacc[3n], s, e, l [n x n]
  double* wscr = slab + (size_t)kGradPlanes * plane;
  const int n_at = A.n_atoms;
  const size_t per_warp = becke_scratch_doubles(n_at);
  BeckeScratch W;
  W.dist = wscr + (size_t)warp * per_warp;
  W.cell = W.dist + n_at;
  W.wacc = W.cell + n_at;
  W.s = W.wacc + 3 * n_at;
  W.e = W.s + (size_t)n_at * n_at;
  W.l = W.e + (size_t)n_at * n_at;
  const bool fused = A.xc >= 0;
  for (int k = tid; k < na3; k += kGT) acc[k] = 0.0;
  if (fused)
    for (size_t k = tid; k < (size_t)kGWarps * per_warp; k += kGT) wscr[k] = 0.0;
  __syncthreads();

  while (true) {
    if (tid == 0) S.batch = atomicAdd(A.counter, 1);
    __syncthreads();
    const int q = S.batch;
    __syncthreads();
    if (q >= G.n_batches) break;
    const int b = G.order[q];
    const BatchDesc bd = G.batches[b];
    const bool live = g < bd.n_pts;
    const size_t pt = (size_t)bd.pt_start + g;
    eval_batch_hess(G, bd, slab, plane);
    if (tid < kBlockPts) S.host[g] = live ? A.host[pt] : 0;
    __syncthreads();
    double hs[3] = {0, 0, 0};
    const ForceCtx none{0, 0, 0.0, nullptr, nullptr};
    const bool two = !fused || !A.closed;  // beta pass needed
    if (fused) {
      contract<false>(G, bd, A.Pa, slab, plane, kPhi, kT, S, none, hs);
      __syncthreads();
      density_from_t(bd, slab, plane, kT, S);
      double ra = 0, gax = 0, gay = 0, gaz = 0;
      if (tid < kBlockPts) {
        ra = S.dens[0][0][g];
        gax = 2.0 * S.dens[0][1][g];
        gay = 2.0 * S.dens[0][2][g];
        gaz = 2.0 * S.dens[0][3][g];
      }
      __syncthreads();
      if (!A.closed) {
        contract<false>(G, bd, A.Pb, slab, plane, kPhi, kT + 1, S, none, hs);
        __syncthreads();
        density_from_t(bd, slab, plane, kT + 1, S);
      }
      if (tid < kBlockPts) {
        double rb = ra, gbx = gax, gby = gay, gbz = gaz;
        if (!A.closed) {
          rb = S.dens[0][0][g];
          gbx = 2.0 * S.dens[0][1][g];
          gby = 2.0 * S.dens[0][2][g];
          gbz = 2.0 * S.dens[0][3][g];
        }
        for (int k = 0; k < 8; ++k) S.coef[k][g] = 0.0;
        S.fx[g] = 0.0;
        const double rpa = fmax(ra, 0.0), rpb = fmax(rb, 0.0);
        if (live && !(rpa + rpb < 1e-18)) {
          const double gaa = gax * gax + gay * gay + gaz * gaz;
          const double gab = gax * gbx + gay * gby + gaz * gbz;
          const double gbb = gbx * gbx + gby * gby + gbz * gbz;
          const XcVal o = xc_eval(A.xc, rpa, rpb, gaa, gab, gbb);
          const double w = G.pw[pt];
          if (fabs(w) > 1e-24) {
            S.coef[0][g] = w * o.vra;
            S.coef[1][g] = w * (2.0 * o.vgaa * gax + o.vgab * gbx);
            S.coef[2][g] = w * (2.0 * o.vgaa * gay + o.vgab * gby);
            S.coef[3][g] = w * (2.0 * o.vgaa * gaz + o.vgab * gbz);
            S.coef[4][g] = w * o.vrb;
            S.coef[5][g] = w * (2.0 * o.vgbb * gbx + o.vgab * gax);
            S.coef[6][g] = w * (2.0 * o.vgbb * gby + o.vgab * gay);
            S.coef[7][g] = w * (2.0 * o.vgbb * gbz + o.vgab * gaz);
          }
          S.fx[g] = o.f;
        }
      }
    } else if (tid < kBlockPts) {
#pragma unroll
      for (int k = 0; k < 8; ++k) S.coef[k][g] = live ? A.wxc[8 * pt + k] : 0.0;
      S.fx[g] = 0.0;
    }
    __syncthreads();
    if (!fused) {
      // T_a (and T_b) for the caller's coefficients
      contract<false>(G, bd, A.Pa, slab, plane, kPhi, kT, S, none, hs);
      if (!A.closed) {
        __syncthreads();
        contract<false>(G, bd, A.Pb, slab, plane, kPhi, kT + 1, S, none, hs);
      }
      __syncthreads();
    }
    // (D) psi planes, then the force tiles per spin
    for (int s = 0; s < (two ? 2 : 1); ++s) {
      const double u0 = S.coef[4 * s + 1][g], u1 = S.coef[4 * s + 2][g], u2 = S.coef[4 * s + 3][g];
      for (int i = h; i < bd.m; i += 2) {
        const size_t o = (size_t)i * kBlockPts + g;
        slab[(kPsi + s) * plane + o] = u0 * slab[plane + o] + u1 * slab[2 * plane + o] + u2 * slab[3 * plane + o];
      }
    }
    __syncthreads();
    {
      const ForceCtx fa{0, kT, two ? -2.0 : -4.0, A.ao_atom, acc};
      contract<true>(G, bd, A.Pa, slab, plane, kPsi, 0, S, fa, hs);
      if (two) {
        __syncthreads();
        const ForceCtx fb{1, A.closed ? kT : kT + 1, -2.0, A.ao_atom, acc};
        contract<true>(G, bd, A.closed ? A.Pa : A.Pb, slab, plane, kPsi + 1, 0, S, fb, hs);
      }
    }
    __syncthreads();
    S.hsum[h][0][g] = hs[0];
    S.hsum[h][1][g] = hs[1];
    S.hsum[h][2][g] = hs[2];
    __syncthreads();
    if (tid < 3) {
      for (int gg = 0; gg < bd.n_pts; ++gg) {
        acc[3 * S.host[gg] + tid] -= S.hsum[0][tid][gg] + S.hsum[1][tid][gg];
      }
    }
    // (E) Becke weight derivative, one warp per point
    if (fused && n_at > 1) {
      for (int k = 0; k < kPtsPerWarp; ++k) {
        const int gg = warp * kPtsPerWarp + k;
        if (gg >= bd.n_pts) break;
        const double f = S.fx[gg];
        const size_t p = (size_t)bd.pt_start + gg;
        const double rw = A.raw_w[p];
        if (fabs(f) < 1e-18 || rw == 0.0) continue;
        becke_point(n_at, A.xyz, A.inv_r, A.a_ij, A.pairs, A.n_pairs, S.host[gg], G.px[p], G.py[p], G.pz[p], rw * f,
                    W);
      }
    }
    __syncthreads();
    // (F) the batch's row of per-atom sums
    double* out = A.part + (size_t)b * na3;
    for (int k = tid; k < na3; k += kGT) {
      double v = acc[k];
      acc[k] = 0.0;
      if (fused) {
        for (int w = 0; w < kGWarps; ++w) {
          double* wa = wscr + (size_t)w * per_warp + 2 * n_at;
          v += wa[k];
          wa[k] = 0.0;
        }
      }
      out[k] = v;
    }
    __syncthreads();
  }
  (void)lane;
}

// grad[k] = sum over batches b (in order) of part[b][k]; one CTA per entry k.
__global__ void __launch_bounds__(256) grad_reduce_kernel(const double* __restrict__ part, int n_batches, int na3,
                                                          double* __restrict__ grad, int accumulate) {
  __shared__ double s[256];
  const int k = blockIdx.x, t = threadIdx.x;
  double v = 0.0;
  for (int b = t; b < n_batches; b += 256) v += part[(size_t)b * na3 + k];
  s[t] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (t < o) s[t] += s[t + o];
    __syncthreads();
  }
  if (t == 0) grad[k] = accumulate ? grad[k] + s[0] : s[0];
}

}  // namespace

size_t grad_smem_bytes(int n_atoms) { return sizeof(GradSmem) + (size_t)3 * n_atoms * sizeof(double); }

size_t grad_slab_doubles(int max_m, int n_atoms) {
  const size_t m_pad = (size_t)(max_m + kGRows - 1) / kGRows * kGRows;
  return (size_t)kGradPlanes * m_pad * kBlockPts + (size_t)kGWarps * becke_scratch_doubles(n_atoms);
}

int grad_max_atoms() { return kMaxGradAtoms; }

cudaError_t launch_xc_grad(const DevGrid& G, const GradArgs& A, int n_ctas, cudaStream_t st) {
  const size_t smem = grad_smem_bytes(A.n_atoms);
  const cudaError_t e = cudaFuncSetAttribute(xc_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  xc_grad_kernel<<<n_ctas, kGT, smem, st>>>(G, A);
  return cudaGetLastError();
}

cudaError_t launch_grad_reduce(const double* part, int n_batches, int n_atoms, double* grad, cudaStream_t st) {
  grad_reduce_kernel<<<3 * n_atoms, 256, 0, st>>>(part, n_batches, 3 * n_atoms, grad, 0);
  return cudaGetLastError();
}

cudaError_t launch_grad_accumulate(const double* part, int n_rows, int n_atoms, double* grad, cudaStream_t st) {
  grad_reduce_kernel<<<3 * n_atoms, 256, 0, st>>>(part, n_rows, 3 * n_atoms, grad, 1);
  return cudaGetLastError();
}

}  // namespace cxc
