// xc_grad_mixed.cu -- XC nuclear gradient with its density contractions on the tensor cores.
//
// The same quantity as xc_grad.cu (xc_nuclear_gradient, vxc.rs:1769-1912):
//   dExc/dR_A = -2 sum_g sum_s sum_{i on A, A != host(g)} [ A_s,iq T_s,i + dphi_iq Y_s,i ] + ...
// with A_s,iq = w v_rho_s dphi_iq + (w u_s) . Hphi_i,q, T_s = P_s Phi, Y_s = P_s Psi_s and
// Psi_s = (w u_s) . grad Phi, plus the Becke weight derivative.  A row's term goes to its own atom
// and, with the opposite sign, to the point's host atom (the reference adds both), so rows on the
// host atom cancel exactly and are skipped here.
//
// Two persistent CTAs of 256 threads per SM (256 TMEM columns and ~107 KB of shared memory each), as
// the tensor-core Vxc kernel.  For each 128-point batch of m candidate AOs:
//   (A) phi, grad phi and the six second derivatives in double-float on the FP32 pipe (error-free
//       transformations, the table-driven exp), FP32 high and BF16 low halves, in ten planes;
//       the Hessian form's screening (shell cutoff; radial value, slope and curvature below 1e-18);
//   (B) per spin, T_s = Phi P_s on tcgen05 with the exact fixed-point split of vxc_mixed.cu (Phi rows
//       scaled by 2^-e_g, D rows by 2^-f_nu, four BF16 pieces each, ten products, hh products summed
//       exactly); the epilogue keeps T as a double-float plane and forms rho_s, grad rho_s by
//       compensated sums;
//   (C) the FP64 functional per point (the one-spin form for a closed shell): (w v_rho_s, w u_s), f;
//   (D) per spin, Psi_s = (w u_s) . grad Phi in double-float, split the same way (scale 2^-e'_g) and
//       Y_s = Psi_s P_s on tcgen05; the epilogue forms each row's force from T, Y, grad phi and the
//       Hessian in double-float, sums consecutive rows of one atom per point, reduces those sums
//       over the points with warp shuffles and adds them, in a fixed order, to the batch's row of
//       per-atom sums; every point's total goes to its host atom with the opposite sign;
//   (E) the Becke weight derivative in double-float (becke_grad.cuh): teams of 1-8 warps, one point
//       per team, with the pair tables in the idle operand stage (up to 87 atoms), else one warp
//       per point with the tables in the scratch slab;
//   (F) a second kernel adds the batches' rows in batch order (deterministic).
// Every mbarrier wait is bounded; on expiry the kernel sets the status word, waits (bounded) for its
// own MMAs and bulk copies in flight, frees TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "becke_grad.cuh"
#include "common.cuh"
#include "dfloat.cuh"
#include "launch.h"
#include "mixed_ops.cuh"
#include "tc_ptx.cuh"
#include "xc_device.cuh"
#include "xc_df.cuh"

namespace cxc {

namespace {

using namespace mix;
using becke::BeckeScratchDf;
using becke::becke_point_df;
using becke::becke_scratch_doubles;

constexpr int kGM = kThreads;         // threads per CTA (two CTAs per SM)
constexpr int kGWarpsM = kGM / 32;
constexpr int kMaxGM = 2048;          // AOs per batch held in shared memory
constexpr uint32_t kWaitG = 1u << 26;
constexpr uint32_t kTmemColsG = 256;
constexpr int kStageG = 98304;        // GEMM operands: A 4 x 16 KB + B 4 x 8 KB
constexpr int kOffAoG = kStageG;                 // int [kMaxGM]
constexpr int kOffEgG = kOffAoG + kMaxGM * 4;    // int [128]: Phi row scale
constexpr int kOffEpG = kOffEgG + 512;           // int [128]: Psi row scale
constexpr int kOffTabG = kOffEpG + 512;          // df32 [64]: 2^(-j/64)
constexpr int kOffFxG = kOffTabG + 512;          // int [kNc]: density row exponents of the chunk
constexpr int kOffHostG = kOffFxG + kNc * 4;     // int [128]: host atom per point
constexpr int kOffMiscG = kOffHostG + 512;       // mbarriers, TMEM slot, batch index
constexpr int kSmemG = kOffMiscG + 32 + 1024;    // + alignment slack
// stage-resident scratch while no operands are in flight
constexpr int kOffDensS = 65536;                 // double [2][4][128]
constexpr int kOffRedS = 0;                      // per-warp runs of the row forces (7.2 KB)
constexpr int kOffHsumS = 8192;                  // double [2][3][128]: per-point host sums
static_assert(2 * (kSmemG + 1024) <= 233472, "two CTAs must fit in one SM's shared memory");
constexpr int kPlanesG = 10;                     // phi, grad (3), Hessian (xx xy xz yy yz zz)

// double-float from an FP32 high half and a BF16 low half
__device__ __forceinline__ df32 ld_df(const float* hi, const __nv_bfloat16* lo, size_t o) {
  return df32{hi[o], __bfloat162float(lo[o])};
}

__device__ __forceinline__ df32 df_fma(df32 a, df32 b, df32 c) { return df_add(df_mul(a, b), c); }

// (A) values, gradients and Hessians of the batch's AOs in double-float (rows [m, m_k) of the last
// 64-row K block zeroed).
// Returns the largest |phi| hi part this thread wrote.
__device__ float ao_eval_df_hess(const DevGrid& G, const BatchDesc& bd, float* __restrict__ hi,
                                 __nv_bfloat16* __restrict__ lo, size_t P, int m_k, const df32* tab) {
  float vmax = 0.f;
  const int tid = threadIdx.x;
  const int g = tid & 127;
  const bool live = g < bd.n_pts;
  df32 X = {0.f, 0.f}, Y = {0.f, 0.f}, Zc = {0.f, 0.f};
  if (live) {
    X = df_from_double(G.px[bd.pt_start + g]);
    Y = df_from_double(G.py[bd.pt_start + g]);
    Zc = df_from_double(G.pz[bd.pt_start + g]);
  }
  for (int ci = tid >> 7; ci < bd.n_cand; ci += kGM / 128) {
    const int si = G.cand_shells[bd.cand_start + ci];
    const AoShellGpu sh = G.shells[si];
    const int loc = G.cand_loc[bd.cand_start + ci];
    df32 dx = {0.f, 0.f}, dy = {0.f, 0.f}, dz = {0.f, 0.f}, r0 = {0.f, 0.f}, r1 = {0.f, 0.f}, r2r = {0.f, 0.f};
    bool on = false;
    if (live) {
      const float2 cx = G.shell_cf[3 * si], cy = G.shell_cf[3 * si + 1], cz = G.shell_cf[3 * si + 2];
      dx = df_sub(X, df32{cx.x, cx.y});
      dy = df_sub(Y, df32{cy.x, cy.y});
      dz = df_sub(Zc, df32{cz.x, cz.y});
      const df32 r2 = df_add(df_add(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz));
      if (!(r2.hi > (float)sh.r2_cutoff)) {
        for (int p = 0; p < sh.n_prims; ++p) {
          const float4 pf = G.prim_f[sh.prim_start + p];  // (a_hi, a_lo, w_hi, w_lo)
          const df32 a = {pf.x, pf.y};
          const df32 e = df_mul(df32{pf.z, pf.w}, df_exp_neg(df_mul(a, r2), tab));
          r0 = df_add(r0, e);
          const df32 ae = df_mul(a, e);
          r1 = df_sub(r1, df_mul_f(ae, 2.f));
          r2r = df_add(r2r, df_mul_f(df_mul(a, ae), 4.f));
        }
        on = !(fabsf(r0.hi) < 1e-18f && fabsf(r1.hi) < 1e-18f && fabsf(r2r.hi) < 1e-18f);
      }
    }
    for (int c = 0; c < sh.n_funcs; ++c) {
      df32 o[kPlanesG];
#pragma unroll
      for (int k = 0; k < kPlanesG; ++k) o[k] = df32{0.f, 0.f};
      if (on) {
        const AoCompGpu cp = G.comps[sh.comp_start + c];
        const float2 sc = G.comp_f[sh.comp_start + c];
        const df32 s = {sc.x, sc.y};
        // x^l, l x^(l-1), l (l-1) x^(l-2)
        df32 px = {1.f, 0.f}, dpx = {0.f, 0.f}, qx = {0.f, 0.f};
        df32 py = {1.f, 0.f}, dpy = {0.f, 0.f}, qy = {0.f, 0.f};
        df32 pz = {1.f, 0.f}, dpz = {0.f, 0.f}, qz = {0.f, 0.f};
        if (cp.lx == 1) { px = dx; dpx = df32{1.f, 0.f}; }
        if (cp.lx == 2) { px = df_mul(dx, dx); dpx = df_mul_f(dx, 2.f); qx = df32{2.f, 0.f}; }
        if (cp.lx == 3) { const df32 x2 = df_mul(dx, dx); px = df_mul(x2, dx); dpx = df_mul_f(x2, 3.f); qx = df_mul_f(dx, 6.f); }
        if (cp.ly == 1) { py = dy; dpy = df32{1.f, 0.f}; }
        if (cp.ly == 2) { py = df_mul(dy, dy); dpy = df_mul_f(dy, 2.f); qy = df32{2.f, 0.f}; }
        if (cp.ly == 3) { const df32 y2 = df_mul(dy, dy); py = df_mul(y2, dy); dpy = df_mul_f(y2, 3.f); qy = df_mul_f(dy, 6.f); }
        if (cp.lz == 1) { pz = dz; dpz = df32{1.f, 0.f}; }
        if (cp.lz == 2) { pz = df_mul(dz, dz); dpz = df_mul_f(dz, 2.f); qz = df32{2.f, 0.f}; }
        if (cp.lz == 3) { const df32 z2 = df_mul(dz, dz); pz = df_mul(z2, dz); dpz = df_mul_f(z2, 3.f); qz = df_mul_f(dz, 6.f); }
        const df32 yz = df_mul(py, pz), xz = df_mul(px, pz), xy = df_mul(px, py);
        const df32 mm = df_mul(px, yz);
        const df32 m0 = df_mul(dpx, yz), m1 = df_mul(dpy, xz), m2 = df_mul(dpz, xy);
        const df32 mr1 = df_mul(mm, r1), mr2 = df_mul(mm, r2r);
        o[0] = df_mul(s, df_mul(mm, r0));
        o[1] = df_mul(s, df_fma(m0, r0, df_mul(mr1, dx)));
        o[2] = df_mul(s, df_fma(m1, r0, df_mul(mr1, dy)));
        o[3] = df_mul(s, df_fma(m2, r0, df_mul(mr1, dz)));
        // Hxx = s (qx py pz r0 + (2 m0 dx + mm) r1 + mm dx^2 r2r), and so on
        o[4] = df_mul(s, df_add(df_add(df_mul(df_mul(qx, yz), r0), df_mul(df_fma(df_mul_f(m0, 2.f), dx, mm), r1)),
                                df_mul(mr2, df_mul(dx, dx))));
        o[5] = df_mul(s, df_add(df_add(df_mul(df_mul(df_mul(dpx, dpy), pz), r0),
                                       df_mul(df_fma(m0, dy, df_mul(m1, dx)), r1)),
                                df_mul(mr2, df_mul(dx, dy))));
        o[6] = df_mul(s, df_add(df_add(df_mul(df_mul(df_mul(dpx, py), dpz), r0),
                                       df_mul(df_fma(m0, dz, df_mul(m2, dx)), r1)),
                                df_mul(mr2, df_mul(dx, dz))));
        o[7] = df_mul(s, df_add(df_add(df_mul(df_mul(qy, xz), r0), df_mul(df_fma(df_mul_f(m1, 2.f), dy, mm), r1)),
                                df_mul(mr2, df_mul(dy, dy))));
        o[8] = df_mul(s, df_add(df_add(df_mul(df_mul(df_mul(px, dpy), dpz), r0),
                                       df_mul(df_fma(m1, dz, df_mul(m2, dy)), r1)),
                                df_mul(mr2, df_mul(dy, dz))));
        o[9] = df_mul(s, df_add(df_add(df_mul(df_mul(qz, xy), r0), df_mul(df_fma(df_mul_f(m2, 2.f), dz, mm), r1)),
                                df_mul(mr2, df_mul(dz, dz))));
      }
      const size_t off = (size_t)(loc + c) * 128 + g;
      vmax = fmaxf(vmax, fabsf(o[0].hi));
#pragma unroll
      for (int k = 0; k < kPlanesG; ++k) {
        hi[k * P + off] = o[k].hi;
        lo[k * P + off] = __float2bfloat16_rn(o[k].lo);
      }
    }
  }
  const int pad = (m_k - bd.m) * 128;
  for (int e = tid; e < pad; e += kGM) {
    const size_t o = (size_t)bd.m * 128 + e;
#pragma unroll
    for (int k = 0; k < kPlanesG; ++k) {
      hi[k * P + o] = 0.f;
      lo[k * P + o] = __float2bfloat16_rn(0.f);
    }
  }
  return vmax;
}

// Psi = u . grad phi at row mu, point g (double-float).
__device__ __forceinline__ df32 psi_at(const float* __restrict__ hi, const __nv_bfloat16* __restrict__ lo, size_t P,
                                       size_t o, df32 ux, df32 uy, df32 uz) {
  const df32 gx = ld_df(hi + P, lo + P, o), gy = ld_df(hi + 2 * P, lo + 2 * P, o), gz = ld_df(hi + 3 * P, lo + 3 * P, o);
  return df_add(df_add(df_mul(ux, gx), df_mul(uy, gy)), df_mul(uz, gz));
}

// GEMM1 A operand of the batch, tile (kb, piece q) at apack + (4 kb + q) * 16 KB: the rows of the
// source (the Phi planes, or the double-float Psi plane psi_hi / psi_lo when given) scaled by 2^-e_g
// and cut into four fixed-point pieces.
__device__ void pack_rows(unsigned char* __restrict__ apack, const float* __restrict__ hi,
                          const __nv_bfloat16* __restrict__ lo, const int* s_e, int nkb,
                          const float* __restrict__ psi_hi, const float* __restrict__ psi_lo) {
  for (int e = threadIdx.x; e < nkb * 128 * 8; e += kGM) {
    const int kb = e >> 10, g = e & 127, c = (e >> 7) & 7;
    const int mu0 = kb * 64 + c * 8;
    const int eg = s_e[g];
    __nv_bfloat16 h[8], md[8], l[8], q[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const size_t o = (size_t)(mu0 + k) * 128 + g;
      const df32 v = psi_hi ? df32{psi_hi[o], psi_lo[o]} : ld_df(hi, lo, o);
      fixsplit4(ldexpf(v.hi, -eg), ldexpf(v.lo, -eg), h[k], md[k], l[k], q[k]);
    }
    unsigned char* t = apack + (size_t)kb * 65536 + sw128(g, c);
    *reinterpret_cast<uint4*>(t) = pack8v(h);
    *reinterpret_cast<uint4*>(t + 16384) = pack8v(md);
    *reinterpret_cast<uint4*>(t + 32768) = pack8v(l);
    *reinterpret_cast<uint4*>(t + 49152) = pack8v(q);
  }
}

}  // namespace

__global__ void __launch_bounds__(kGM, 2) xc_grad_mixed_kernel(DevGrid G, GradArgs A, int* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* stage = base;
  int* s_ao = reinterpret_cast<int*>(base + kOffAoG);
  int* s_eg = reinterpret_cast<int*>(base + kOffEgG);
  int* s_ep = reinterpret_cast<int*>(base + kOffEpG);
  df32* s_tab = reinterpret_cast<df32*>(base + kOffTabG);
  int* s_fx = reinterpret_cast<int*>(base + kOffFxG);
  int* s_host = reinterpret_cast<int*>(base + kOffHostG);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(base + kOffMiscG);
  uint64_t* tbar = reinterpret_cast<uint64_t*>(base + kOffMiscG + 8);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(base + kOffMiscG + 16);
  int* s_batch = reinterpret_cast<int*>(base + kOffMiscG + 20);
  double(*dens)[4][128] = reinterpret_cast<double(*)[4][128]>(stage + kOffDensS);
  double(*run_v)[32][3] = reinterpret_cast<double(*)[32][3]>(stage + kOffRedS);  // per warp: run sums
  int(*run_at)[32] = reinterpret_cast<int(*)[32]>(stage + kOffRedS + 6144);        // per warp: run atoms
  int* run_n = reinterpret_cast<int*>(stage + kOffRedS + 7168);                     // per warp: runs

  double(*hsum)[3][128] = reinterpret_cast<double(*)[3][128]>(stage + kOffHsumS);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = tid & 127, h = tid >> 7;
  const int nspin = A.closed ? 1 : 2;
  const int na3 = 3 * A.n_atoms;

  if (tid == 0) {
    mbar_init(mbar, 1);
    mbar_init(tbar, 1);
    fence_mbar_init();
  }
  if (tid < 64) s_tab[tid] = df_from_double(exp2(-(double)tid / 64.0));
  if (warp == 0) {
    tmem_alloc(tmem_slot, kTmemColsG);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
  const uint32_t tH = tmem, tC1 = tmem + 64, tC2 = tmem + 128, tS = tmem + 192;
  uint32_t phase = 0, tphase = 0;
  bool tma_busy = false;
  bool failed = false;

  const int m_pad_all = (A.max_m + 127) / 128 * 128;
  const size_t P = (size_t)m_pad_all * 128;
  float* hi = reinterpret_cast<float*>(A.slab + (size_t)blockIdx.x * A.slab_stride);
  __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(hi + kPlanesG * P);
  float* t_hi = reinterpret_cast<float*>(lo + kPlanesG * P);  // [2][P]
  float* t_lo = t_hi + 2 * P;                                 // [2][P]
  float* p_hi = t_lo + 2 * P;                                  // Psi of the current spin
  float* p_lo = p_hi + P;
  unsigned char* apack = reinterpret_cast<unsigned char*>(p_lo + P);  // m_pad_all / 64 x 64 KB
  double* coef = reinterpret_cast<double*>(apack + (size_t)m_pad_all * 1024);  // [9][128]
  double* bscr = coef + 9 * 128;
  const size_t per_warp = becke_scratch_doubles(A.n_atoms);
  BeckeScratchDf W;
  W.dist = reinterpret_cast<df32*>(bscr + (size_t)warp * per_warp);
  W.cell = reinterpret_cast<double*>(W.dist + A.n_atoms);
  W.wacc = W.cell + A.n_atoms;
  W.s = reinterpret_cast<df32*>(W.wacc + na3);
  W.e = W.s + (size_t)A.n_atoms * A.n_atoms;
  W.l = W.e + (size_t)A.n_atoms * A.n_atoms;
  for (size_t k = tid; k < (size_t)kGWarpsM * per_warp; k += kGM) bscr[k] = 0.0;

  const uint2* Dhl_a0 = reinterpret_cast<const uint2*>(A.Pa);
  const uint2* Dhl_b0 = Dhl_a0 + G.nn_total;
  const int* fexp_a0 = reinterpret_cast<const int*>(Dhl_a0 + 2 * G.nn_total);
  const int* fexp_b0 = fexp_a0 + G.n_total;
  const uint32_t sb = smem_addr(stage);
  const uint32_t idesc = idesc_bf16_f32(128, kNc);
  const double scale = A.closed ? -4.0 : -2.0;

  auto wait_mma = [&]() -> bool {
    const bool ok = mbar_wait_bounded(mbar, phase, kWaitG);
    phase ^= 1u;
    tc_fence_after();
    return __syncthreads_or(!ok) == 0;
  };
  auto wait_tma = [&]() -> bool {
    const bool ok = mbar_wait_bounded(tbar, tphase, kWaitG);
    if (ok) {
      tphase ^= 1u;
      tma_busy = false;
    }
    return __syncthreads_or(!ok) == 0;
  };
  // One N chunk [nc, nc + 64) of X P_s (A operand already packed in apack): the K loop, then
  // epi(first_group) with the accumulators in TMEM (the chunk's value is hh + corrections, plus the
  // running sum of earlier 16-block groups when the contraction is longer than 1024 AOs).
  auto chunk = [&](int nc, int m, int nkb, int n, const uint2* Dhl, auto&& epi) {
    for (int kb = 0; kb < nkb; ++kb) {
      if (tid == 0) {
        mbar_arrive_expect_tx(tbar, 65536);
#pragma unroll
        for (int t = 0; t < 4; ++t) bulk_g2s(sb + t * 16384, apack + (size_t)kb * 65536 + t * 16384, 16384, tbar);
        tma_busy = true;
      }
      gather_b(stage, Dhl, s_ao, n, m, kb, nc);
      fence_proxy_async_smem();
      if (!wait_tma()) { failed = true; return; }
      if (tid == 0) {
        tc_fence_after();
        const uint64_t ah = sdesc_sw128(sb), am = sdesc_sw128(sb + 16384), al = sdesc_sw128(sb + 32768);
        const uint64_t aq = sdesc_sw128(sb + 49152);
        const uint64_t bh = sdesc_sw128(sb + 65536), bm = sdesc_sw128(sb + 73728), bl = sdesc_sw128(sb + 81920);
        const uint64_t bq = sdesc_sw128(sb + 90112);
        const bool group_start = (kb & 15) == 0;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          const uint64_t o = (uint64_t)(ks * 2);
          const uint32_t acc0 = (!group_start || ks > 0) ? 1u : 0u;
          mma_bf16_ss(tH, ah + o, bh + o, idesc, acc0);   // weight 1
          mma_bf16_ss(tC1, ah + o, bm + o, idesc, acc0);  // weight 2^-8
          mma_bf16_ss(tC1, am + o, bh + o, idesc, 1u);
          mma_bf16_ss(tC2, ah + o, bl + o, idesc, acc0);  // weight 2^-16
          mma_bf16_ss(tC2, am + o, bm + o, idesc, 1u);
          mma_bf16_ss(tC2, al + o, bh + o, idesc, 1u);
          mma_bf16_ss(tC2, ah + o, bq + o, idesc, 1u);    // weight 2^-24
          mma_bf16_ss(tC2, am + o, bl + o, idesc, 1u);
          mma_bf16_ss(tC2, al + o, bm + o, idesc, 1u);
          mma_bf16_ss(tC2, aq + o, bh + o, idesc, 1u);
        }
        mma_commit(mbar);
      }
      if (!wait_mma()) { failed = true; return; }
      const bool group_end = ((kb & 15) == 15) || kb == nkb - 1;
      if (!group_end) continue;
      const bool first_group = kb < 16, last_group = kb == nkb - 1;
      if (!last_group) {
        for (int c0 = h * (kNc / 2); c0 < (h + 1) * (kNc / 2); c0 += 16) {
          float a[16], bb[16], cc[16];
          tmem_ld16(tH + lane_base + (uint32_t)c0, a);
          tmem_ld16(tC1 + lane_base + (uint32_t)c0, bb);
          tmem_ld16(tC2 + lane_base + (uint32_t)c0, cc);
#pragma unroll
          for (int j = 0; j < 16; ++j) bb[j] += cc[j];
          if (!first_group) tmem_ld16(tS + lane_base + (uint32_t)c0, cc);
#pragma unroll
          for (int j = 0; j < 16; ++j) a[j] = (first_group ? 0.f : cc[j]) + a[j] + bb[j];
          tmem_st16(tS + lane_base + (uint32_t)c0, a);
        }
      } else {
        epi(first_group);
      }
      tc_fence_before();
      __syncthreads();
    }
  };
  // four consecutive columns from c0 of the chunk's value, as double-floats (still scaled)
  auto load4 = [&](int c0, bool first_group, df32* t) {
    float a[4], bb[4], c2[4], cc[4];
    tmem_ld4x4(tH + lane_base + (uint32_t)c0, tC1 + lane_base + (uint32_t)c0, tC2 + lane_base + (uint32_t)c0,
               (first_group ? tH : tS) + lane_base + (uint32_t)c0, a, bb, c2, cc);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      bb[j] += c2[j];
      t[j] = first_group ? two_sum(a[j], bb[j]) : df_add_f(two_sum(cc[j], a[j]), bb[j]);
    }
  };

  while (!failed) {
    if (tid == 0) *s_batch = atomicAdd(A.counter, 1);
    __syncthreads();
    const int q = *s_batch;
    __syncthreads();
    if (q >= G.n_batches) break;
    const int b = G.order[q];
    const BatchDesc bd = G.batches[b];
    const int m = bd.m;
    const int n = mol_nao(G, bd.mol);
    const int nkb = (m + 63) / 64;
    const int m_k = nkb * 64;  // rows read by the packed operand and the chunked epilogues
    const bool live = g < bd.n_pts;
    const size_t pt = (size_t)bd.pt_start + g;
    double* out = A.part + (size_t)b * na3;
    for (int i = tid; i < m; i += kGM) s_ao[i] = G.batch_ao[bd.ao_start + i];
    if (tid < 128) s_host[g] = live ? A.host[pt] : -1;
    const float vmax = ao_eval_df_hess(G, bd, hi, lo, P, m_k, s_tab);
    {  // e_g: power-of-two exponent with max_mu |Phi[g][mu]| 2^-e_g < 1
      dens[0][0][g + 128 * h] = (double)vmax;  // scratch: the stage is idle
      __syncthreads();
      if (h == 0) {
        int ex = 0;
        frexpf(fmaxf((float)dens[0][0][g], (float)dens[0][0][g + 128]), &ex);
        s_eg[g] = ex;
      }
      __syncthreads();
    }
    pack_rows(apack, hi, lo, s_eg, nkb, nullptr, nullptr);
    fence_proxy_async_global();  // the packed tiles are read by bulk copies
    __syncthreads();

    // (B) T_s = Phi P_s, kept as a double-float plane; rho_s and grad rho_s
    double spin_rho[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int s = 0; s < nspin && !failed; ++s) {
      const uint2* Dhl = s ? Dhl_b0 : Dhl_a0;
      const int* fexp = s ? fexp_b0 : fexp_a0;
      const int eg = s_eg[g];
      float* th = t_hi + s * P;
      float* tl = t_lo + s * P;
      CompSum sr, sgx, sgy, sgz;
      for (int nc = 0; nc < m && !failed; nc += kNc) {
        if (tid < kNc) s_fx[tid] = nc + tid < m ? fexp[s_ao[nc + tid]] : 0;
        chunk(nc, m, nkb, n, Dhl, [&](bool first_group) {
          for (int c0 = h * (kNc / 2); c0 < (h + 1) * (kNc / 2); c0 += 4) {
            df32 t[4];
            load4(c0, first_group, t);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int nu = nc + c0 + j;
              if (nu < m) {
                const df32 tv = df_ldexp(t[j], eg + s_fx[c0 + j]);
                const size_t o = (size_t)nu * 128 + g;
                th[o] = tv.hi;
                tl[o] = tv.lo;
                acc_prod(sr, ld_df(hi, lo, o), tv);
                acc_prod(sgx, ld_df(hi + P, lo + P, o), tv);
                acc_prod(sgy, ld_df(hi + 2 * P, lo + 2 * P, o), tv);
                acc_prod(sgz, ld_df(hi + 3 * P, lo + 3 * P, o), tv);
              }
            }
          }
        });
      }
      if (failed) break;
      const double acc[4] = {sr.value(), sgx.value(), sgy.value(), sgz.value()};
      for (int k = 0; k < 4; ++k) dens[h][k][g] = acc[k];
      __syncthreads();
      for (int k = 0; k < 4; ++k) spin_rho[s][k] = dens[0][k][g] + dens[1][k][g];
      __syncthreads();
    }
    if (failed) break;

    // (C) functional, one thread per point: coef rows (w v_rho_a, w u_a, w v_rho_b, w u_b, f).  A
    // closed shell's functional is split between the halves: part 0 of xc_eval_cs_df in threads
    // h == 0, part 1 in threads h == 1 (passed through dens), summed as xc_eval_cs_fast sums them.
    XcCs xpart{0.0, 0.0, 0.0};
    if (A.closed) {
      const double rpa = fmax(spin_rho[0][0], 0.0);
      if (live && !(rpa + rpa < 1e-18)) {
        const double gax = 2.0 * spin_rho[0][1], gay = 2.0 * spin_rho[0][2], gaz = 2.0 * spin_rho[0][3];
        xpart = xc_eval_cs_fast_part(A.xc, rpa, gax * gax + gay * gay + gaz * gaz, s_tab, h);
      }
      if (h == 1) {
        dens[1][0][g] = xpart.f;
        dens[1][1][g] = xpart.vr;
        dens[1][2][g] = xpart.vg;
      }
      __syncthreads();
    }
    if (h == 0) {
      double cf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      const double ra = spin_rho[0][0];
      const double gax = 2.0 * spin_rho[0][1], gay = 2.0 * spin_rho[0][2], gaz = 2.0 * spin_rho[0][3];
      const int sb1 = A.closed ? 0 : 1;
      const double rb = spin_rho[sb1][0];
      const double gbx = 2.0 * spin_rho[sb1][1], gby = 2.0 * spin_rho[sb1][2], gbz = 2.0 * spin_rho[sb1][3];
      const double rpa = fmax(ra, 0.0), rpb = fmax(rb, 0.0);
      if (live && A.closed && !(rpa + rpb < 1e-18)) {
        // closed shell: the one-spin form (u_a = (2 v_gamma_aa + v_gamma_ab) grad rho_a = 2 v_g grad rho_a)
        const XcCs o{xpart.f + dens[1][0][g], xpart.vr + dens[1][1][g], xpart.vg + dens[1][2][g]};
        const double w = G.pw[pt];
        if (fabs(w) > 1e-24) {
          const double us = 2.0 * w * o.vg;
          cf[0] = cf[4] = w * o.vr;
          cf[1] = cf[5] = us * gax;
          cf[2] = cf[6] = us * gay;
          cf[3] = cf[7] = us * gaz;
        }
        cf[8] = o.f;
      } else if (live && !(rpa + rpb < 1e-18)) {
        const double gaa = gax * gax + gay * gay + gaz * gaz;
        const double gab = gax * gbx + gay * gby + gaz * gbz;
        const double gbb = gbx * gbx + gby * gby + gbz * gbz;
        const XcVal o = xc_eval(A.xc, rpa, rpb, gaa, gab, gbb);
        const double w = G.pw[pt];
        if (fabs(w) > 1e-24) {
          cf[0] = w * o.vra;
          cf[1] = w * (2.0 * o.vgaa * gax + o.vgab * gbx);
          cf[2] = w * (2.0 * o.vgaa * gay + o.vgab * gby);
          cf[3] = w * (2.0 * o.vgaa * gaz + o.vgab * gbz);
          cf[4] = w * o.vrb;
          cf[5] = w * (2.0 * o.vgbb * gbx + o.vgab * gax);
          cf[6] = w * (2.0 * o.vgbb * gby + o.vgab * gay);
          cf[7] = w * (2.0 * o.vgbb * gbz + o.vgab * gaz);
        }
        cf[8] = o.f;
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) coef[k * 128 + g] = cf[k];
      if (A.fx_out && live) A.fx_out[pt] = cf[8];
    }
    __syncthreads();

    // (D) per spin: Psi_s, Y_s = Psi_s P_s, and the row forces
    df32 hs0 = {0.f, 0.f}, hs1 = hs0, hs2 = hs0;  // this thread's point: sum of its row terms
    for (int s = 0; s < nspin && !failed; ++s) {
      const uint2* Dhl = s ? Dhl_b0 : Dhl_a0;
      const int* fexp = s ? fexp_b0 : fexp_a0;
      const float* th = t_hi + s * P;
      const float* tl = t_lo + s * P;
      const df32 c0 = df_from_double(coef[(4 * s) * 128 + g]);
      const df32 ux = df_from_double(coef[(4 * s + 1) * 128 + g]);
      const df32 uy = df_from_double(coef[(4 * s + 2) * 128 + g]);
      const df32 uz = df_from_double(coef[(4 * s + 3) * 128 + g]);
      {  // Psi into its plane (rows up to m_k: the padding rows give zeros), and e'_g
        float mx = 0.f;
        for (int i = h; i < m_k; i += 2) {
          const size_t o = (size_t)i * 128 + g;
          const df32 ps = psi_at(hi, lo, P, o, ux, uy, uz);
          p_hi[o] = ps.hi;
          p_lo[o] = ps.lo;
          mx = fmaxf(mx, fabsf(ps.hi));
        }
        dens[0][0][g + 128 * h] = (double)mx;
        __syncthreads();
        if (h == 0) {
          int ex = 0;
          frexpf(fmaxf((float)dens[0][0][g], (float)dens[0][0][g + 128]), &ex);
          s_ep[g] = ex;
        }
        __syncthreads();
      }
      pack_rows(apack, hi, lo, s_ep, nkb, p_hi, p_lo);
      fence_proxy_async_global();
      __syncthreads();
      const int ep = s_ep[g];
      const int hg = s_host[g];
      for (int nc = 0; nc < m && !failed; nc += kNc) {
        if (tid < kNc) s_fx[tid] = nc + tid < m ? fexp[s_ao[nc + tid]] : 0;
        chunk(nc, m, nkb, n, Dhl, [&](bool first_group) {
          // the group's 32 columns in runs of one atom: each thread sums its point's terms per run,
          // and a finished run's sum over the warp's 32 points goes to the warp's run list
          df32 r0 = {0.f, 0.f}, r1 = r0, r2 = r0;
          int cur = -1, nrun = 0;
          auto flush = [&]() {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
              r0 = df_add(r0, df32{__shfl_xor_sync(0xffffffffu, r0.hi, off), __shfl_xor_sync(0xffffffffu, r0.lo, off)});
              r1 = df_add(r1, df32{__shfl_xor_sync(0xffffffffu, r1.hi, off), __shfl_xor_sync(0xffffffffu, r1.lo, off)});
              r2 = df_add(r2, df32{__shfl_xor_sync(0xffffffffu, r2.hi, off), __shfl_xor_sync(0xffffffffu, r2.lo, off)});
            }
            if (lane == 0) {
              run_v[warp][nrun][0] = df_to_double(r0);
              run_v[warp][nrun][1] = df_to_double(r1);
              run_v[warp][nrun][2] = df_to_double(r2);
              run_at[warp][nrun] = cur;
            }
            ++nrun;
          };
          for (int c0c = h * (kNc / 2); c0c < (h + 1) * (kNc / 2); c0c += 4) {
            df32 y[4];
            load4(c0c, first_group, y);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int col = c0c + j;
              const int i = nc + col;
              const int at = i < m ? A.ao_atom[s_ao[i]] : -1;  // the same for the whole warp
              if (at != cur) {
                if (cur >= 0) flush();
                cur = at;
                r0 = r1 = r2 = df32{0.f, 0.f};
              }
              if (i < m && live && at != hg) {
                const df32 yv = df_ldexp(y[j], ep + s_fx[col]);
                const size_t o = (size_t)i * 128 + g;
                const df32 t = df32{th[o], tl[o]};
                const df32 d0 = ld_df(hi + P, lo + P, o), d1 = ld_df(hi + 2 * P, lo + 2 * P, o),
                           d2 = ld_df(hi + 3 * P, lo + 3 * P, o);
                const df32 hxx = ld_df(hi + 4 * P, lo + 4 * P, o), hxy = ld_df(hi + 5 * P, lo + 5 * P, o),
                           hxz = ld_df(hi + 6 * P, lo + 6 * P, o), hyy = ld_df(hi + 7 * P, lo + 7 * P, o),
                           hyz = ld_df(hi + 8 * P, lo + 8 * P, o), hzz = ld_df(hi + 9 * P, lo + 9 * P, o);
                const df32 a0 = df_add(df_add(df_mul(c0, d0), df_mul(ux, hxx)), df_add(df_mul(uy, hxy), df_mul(uz, hxz)));
                const df32 a1 = df_add(df_add(df_mul(c0, d1), df_mul(ux, hxy)), df_add(df_mul(uy, hyy), df_mul(uz, hyz)));
                const df32 a2 = df_add(df_add(df_mul(c0, d2), df_mul(ux, hxz)), df_add(df_mul(uy, hyz), df_mul(uz, hzz)));
                const df32 v0 = df_add(df_mul(a0, t), df_mul(d0, yv));
                const df32 v1 = df_add(df_mul(a1, t), df_mul(d1, yv));
                const df32 v2 = df_add(df_mul(a2, t), df_mul(d2, yv));
                r0 = df_add(r0, v0);
                r1 = df_add(r1, v1);
                r2 = df_add(r2, v2);
                hs0 = df_add(hs0, v0);
                hs1 = df_add(hs1, v1);
                hs2 = df_add(hs2, v2);
              }
            }
          }
          if (cur >= 0) flush();
          if (lane == 0) run_n[warp] = nrun;
        });
        if (failed) break;
        // the runs' sums, group by group in column order, into the batch's per-atom row
        if (tid < 3) {
          for (int grp = 0; grp < 2; ++grp) {
            const int w0 = 4 * grp;
            for (int r = 0; r < run_n[w0]; ++r) {
              const double v = run_v[w0][r][tid] + run_v[w0 + 1][r][tid] + run_v[w0 + 2][r][tid] + run_v[w0 + 3][r][tid];
              out[3 * run_at[w0][r] + tid] += scale * v;
            }
          }
        }
        __syncthreads();
      }
    }
    if (failed) break;
    // host-atom term: minus every point's total
    hsum[h][0][g] = df_to_double(hs0);
    hsum[h][1][g] = df_to_double(hs1);
    hsum[h][2][g] = df_to_double(hs2);
    __syncthreads();
    if (tid < 3) {
      double run = 0.0;
      int cur = -1;
      for (int gg = 0; gg < bd.n_pts; ++gg) {
        const int at = s_host[gg];
        if (at != cur) {
          if (cur >= 0) out[3 * cur + tid] -= scale * run;
          cur = at;
          run = 0.0;
        }
        run += hsum[0][tid][gg] + hsum[1][tid][gg];
      }
      if (cur >= 0) out[3 * cur + tid] -= scale * run;
    }
    // (E) Becke weight derivative: teams of 1-8 warps per point with the pair tables in the (idle)
    // stage when one team's tables fit, else one warp per point with tables in the scratch slab
    __syncthreads();
    const size_t team_bytes = becke::becke_cta_bytes(A.n_atoms);
    const bool cta_becke = team_bytes + (size_t)24 * A.n_atoms <= (size_t)kStageG;
    if (A.fx_out) {
      // the weight derivative runs as becke_mixed_kernel
    } else if (A.n_atoms > 1 && cta_becke) {
      int n_teams = 1;
      while (n_teams < kGWarpsM && (size_t)(2 * n_teams) * team_bytes + (size_t)24 * A.n_atoms <= (size_t)kStageG)
        n_teams *= 2;
      const int nt = kGM / n_teams, team = tid / nt, tt = tid % nt;
      df32* xyz_df = reinterpret_cast<df32*>(stage + (size_t)n_teams * team_bytes);
      for (int k = tid; k < 3 * A.n_atoms; k += kGM) xyz_df[k] = df_from_double(A.xyz[k]);
      becke::BeckeCta T;
      T.carve(stage + (size_t)team * team_bytes, A.n_atoms);
      for (int k = tt; k < na3; k += nt) T.wacc[k] = df32{0.f, 0.f};
      __syncthreads();
      for (int gg = team; gg < bd.n_pts; gg += n_teams) {
        const double f = coef[8 * 128 + gg];
        const size_t p = (size_t)bd.pt_start + gg;
        const double rw = A.raw_w[p];
        if (fabs(f) < 1e-18 || rw == 0.0) continue;
        becke::becke_point_team(A.n_atoms, xyz_df, reinterpret_cast<const df32*>(A.pair_df), s_host[gg],
                                df_from_double(G.px[p]), df_from_double(G.py[p]), df_from_double(G.pz[p]),
                                df_from_double(rw * f), T, tt, nt, team);
      }
      __syncthreads();
      for (int k = tid; k < na3; k += kGM) {
        double v = 0.0;
        for (int t = 0; t < n_teams; ++t) {
          becke::BeckeCta Tt;
          Tt.carve(stage + (size_t)t * team_bytes, A.n_atoms);
          v += df_to_double(Tt.wacc[k]);
        }
        out[k] += v;
      }
    } else if (A.n_atoms > 1) {
      for (int k = 0; k < 128 / kGWarpsM; ++k) {
        const int gg = warp * (128 / kGWarpsM) + k;
        if (gg >= bd.n_pts) break;
        const double f = coef[8 * 128 + gg];
        const size_t p = (size_t)bd.pt_start + gg;
        const double rw = A.raw_w[p];
        if (fabs(f) < 1e-18 || rw == 0.0) continue;
        becke_point_df(A.n_atoms, A.xyz, reinterpret_cast<const df32*>(A.pair_df), A.pairs, A.n_pairs, s_host[gg], G.px[p], G.py[p], G.pz[p],
                       rw * f, W);
      }
    }
    __syncthreads();
    if (!A.fx_out && A.n_atoms > 1 && !cta_becke) {
      for (int k = tid; k < na3; k += kGM) {
        double v = 0.0;
        for (int w = 0; w < kGWarpsM; ++w) {
          double* wa = bscr + (size_t)w * per_warp + 2 * A.n_atoms;
          v += wa[k];
          wa[k] = 0.0;
        }
        out[k] += v;
      }
    }
    __syncthreads();
  }

  if (failed) {
    if (tid == 0) atomicExch(status, 1);
    mbar_wait_bounded(mbar, phase ^ 1u, kWaitG);
    if (tma_busy) mbar_wait_bounded(tbar, tphase, kWaitG);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, kTmemColsG);
}

// The Becke weight derivative as its own kernel (atoms whose pair tables fit in shared memory):
// one team of nt threads per CTA (a warp for up to 40 atoms, else the whole 256-thread CTA), the
// team's tables in dynamic shared memory, kBeckePts consecutive points per CTA, and one row of
// per-atom sums per CTA (part[cta][3 n_atoms]).  Separate from the quadrature kernel so that many
// more teams are resident per SM than its two CTAs of eight warps allow.
constexpr int kBeckePts = 16;

__global__ void becke_mixed_kernel(DevGrid G, GradArgs A, const double* __restrict__ fx, double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char bsm[];
  const int na = A.n_atoms, na3 = 3 * na;
  const int tid = threadIdx.x, nt = blockDim.x;
  becke::BeckeCta T;
  T.carve(bsm, na);
  // the nuclei as double-floats behind the team's tables
  df32* xyz_df = reinterpret_cast<df32*>(bsm + becke::becke_cta_bytes(na));
  for (int k = tid; k < 3 * na; k += nt) xyz_df[k] = df_from_double(A.xyz[k]);
  for (int k = tid; k < na3; k += nt) T.wacc[k] = df32{0.f, 0.f};
  becke::team_sync(nt, 0);
  const int p0 = blockIdx.x * kBeckePts;
  for (int k = 0; k < kBeckePts; ++k) {
    const int p = p0 + k;
    if (p >= G.n_pts) break;
    const double f = fx[p], rw = A.raw_w[p];
    if (fabs(f) < 1e-18 || rw == 0.0) continue;
    becke::becke_point_team(na, xyz_df, reinterpret_cast<const df32*>(A.pair_df), A.host[p], df_from_double(G.px[p]),
                            df_from_double(G.py[p]), df_from_double(G.pz[p]), df_from_double(rw * f), T, tid, nt, 0);
  }
  becke::team_sync(nt, 0);
  double* out = part + (size_t)blockIdx.x * na3;
  for (int k = tid; k < na3; k += nt) out[k] = df_to_double(T.wacc[k]);
}

// Whether the separate weight-derivative kernel applies (its team's tables fit in shared memory),
// its launch shape, and the number of CTAs (rows of its partial sums).
int becke_kernel_threads(int n_atoms) { return n_atoms <= 40 ? 32 : 256; }
size_t becke_kernel_smem(int n_atoms) { return becke::becke_cta_bytes(n_atoms) + (size_t)24 * n_atoms; }
bool becke_kernel_fits(int n_atoms) {
  return n_atoms > 1 && becke::becke_cta_bytes(n_atoms) + (size_t)24 * n_atoms <= (size_t)kStageG;
}
int becke_kernel_ctas(int n_pts) { return (n_pts + kBeckePts - 1) / kBeckePts; }

cudaError_t launch_becke_mixed(const DevGrid& G, const GradArgs& A, const double* fx, double* part, cudaStream_t st) {
  const int nt = becke_kernel_threads(A.n_atoms);
  const size_t smem = becke_kernel_smem(A.n_atoms);
  const cudaError_t e = cudaFuncSetAttribute(becke_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  becke_mixed_kernel<<<becke_kernel_ctas(G.n_pts), nt, smem, st>>>(G, A, fx, part);
  return cudaGetLastError();
}

size_t grad_mixed_slab_doubles(int max_m, int n_atoms) {
  const size_t m_pad = (size_t)(max_m + 127) / 128 * 128, P = m_pad * 128;
  // planes: 10 FP32 + 10 BF16; T planes: 2 spins x (FP32 hi + FP32 lo); Psi (FP32 hi + lo); packed A
  const size_t bytes = P * (kPlanesG * 4 + kPlanesG * 2 + 16 + 8 + 8) + 9 * 128 * sizeof(double) +
                       (size_t)kGWarpsM * becke_scratch_doubles(n_atoms) * sizeof(double);
  return (bytes / sizeof(double) + 127) / 128 * 128;  // 1 KB multiples keep every CTA's slab aligned
}

int grad_mixed_max_m() { return kMaxGM; }

cudaError_t launch_xc_grad_mixed(const DevGrid& G, const GradArgs& A, int n_ctas, int* status, cudaStream_t st) {
  if (A.max_m > kMaxGM) return cudaErrorInvalidValue;
  static bool attr = false;
  if (!attr) {
    const cudaError_t e = cudaFuncSetAttribute(xc_grad_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemG);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  xc_grad_mixed_kernel<<<n_ctas, kGM, kSmemG, st>>>(G, A, status);
  return cudaGetLastError();
}

}  // namespace cxc
