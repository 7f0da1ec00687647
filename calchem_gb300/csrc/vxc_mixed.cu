// vxc_mixed.cu -- tensor-core (tcgen05) XC quadrature: the mixed-precision form.
//
// Two persistent CTAs of 256 threads per SM (each 256 TMEM columns, ~110 KB of shared memory) take
// 128-point batches from a device queue, so that one CTA's SIMT and FP64 phases run under the
// other's contractions.  For each batch of m candidate AOs (GEMM1's K dimension padded with zero rows
// to a multiple of 64; GEMM2's tiles to a multiple of 128 with rows that are never read back):
//   (A) AO values and gradients in double-float arithmetic on the FP32 pipe (48-bit: error-free
//       transformations, a table-driven exp, basis constants and coordinates as float pairs) into
//       the CTA's scratch slab -- or, when the grid has an AO cache, into the batch's cache block,
//       which later launches read instead of evaluating (steps A and B depend on the grid and basis
//       only) -- as [m][128] planes (FP32 hi and BF16 lo of phi, d/dx, d/dy, d/dz), with the
//       reference's screening (ao_grid.rs:182-230).  Plain FP32 AO values carry errors of
//       a few ulp that are identical at the 302 angular points of a radial shell and so do not
//       average out; at 48 bits they are negligible;
//   (B) every Phi row (point) is scaled by a power of two to |x| < 1 and cut into four fixed-point
//       BF16 pieces (multiples of 2^-7, 2^-15, 2^-23, 2^-31), written once per batch into the slab
//       as 128-byte-swizzled operand tiles (the GEMM1 A operand, loaded by bulk copies);
//   (C) GEMM1  T[g][nu] = sum_mu Phi[g][mu] D[mu][nu]  on tcgen05: M = 128 points, N = 64 AOs per
//       TMEM chunk, K = AOs in blocks of 64; D rows are cut the same way (four pieces, gathered per
//       block); the ten products with weight down to 2^-24 are formed.  The hh products are integer
//       multiples of 2^-14 and a 1024-term sum stays below 2^24 units, so the tensor core's FP32
//       accumulation (which truncates) adds them EXACTLY; the correction classes (i + j = 1;
//       i + j = 2 and 3) are at least 2^8 smaller and accumulate separately, over up to 16 K
//       blocks; longer contractions are combined into a fourth accumulator;
//   (D) epilogue: each thread owns one point (its TMEM lane); T = hh + corrections is kept as a
//       double-float, times the density row's scale 2^f (the point's scale 2^e_g multiplies the
//       finished sums); the planes stream through a ring of shared-memory buffers by bulk copies (a
//       buffer is refilled once every warp has arrived on its release barrier); rho = sum Phi T is
//       a compensated sum of double-float products, grad rho = 2 sum grad Phi T three FP32 FMA sums
//       of them (compensated too in builds with per-point output), with the AO gradients' low parts
//       kept (on (H2O)61 against the FP64 form: the FMA sums for grad rho move Exc by < 2e-9 Eh and
//       take 7 % off the kernel; dropping the low parts would move it by 2.6e-8, summing rho the
//       same way by 1.1e-7);
//   (E) the functional per point (double-float for the closed-shell codes 0-5 above 1e-12, FP64
//       otherwise; a closed shell's two parts of xc_eval_cs_df in the two 128-thread halves),
//       Exc and Nelec partial sums in FP64 (vxc.rs:890-920);
//   (F) GEMM2  W = Z^T Phi + Phi^T Z  (Z = (w v_rho / 2) Phi + (w u) . grad Phi) on lower
//       128 x 128 AO tile pairs, K = 64 points per step: Phi and Z split into three BF16 pieces
//       (floating, 24 bits), written as swizzled tiles and loaded by bulk copies (for m <= 128, one
//       tile pair: written straight into the shared-memory stage per K half), six products per
//       half step, the hh products in one accumulator and the corrections in another;
//   (G) the W tile is drained from TMEM and added to V's upper triangle with FP64 atomics,
//       coalesced across lanes, skipping contributions below 1e-11; a final kernel mirrors the upper
//       triangle into the lower.
// Every mbarrier wait is bounded, and a wait that expires sets the status flag, waits (bounded) for
// the CTA's own MMAs and copies in flight, frees TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "dfloat.cuh"
#include "mixed_ops.cuh"
#include "tc_ptx.cuh"
#include "xc_device.cuh"
#include "xc_df.cuh"

namespace cxc {

namespace {

using namespace mix;
constexpr int kMT = kThreads;         // threads per CTA (two CTAs per SM)
constexpr int kGroups = kMT / 128;    // thread groups of 128 (one thread per point in each)
constexpr int kMaxMixedM = 2048;      // AOs per batch held in shared memory
constexpr uint32_t kWaitLimit = 1u << 26;
constexpr int kRing = 4;              // epilogue bulk-copy buffers in the stage
constexpr int kRingBytes = 24576;     // one 8-row step: 4 x 4 KB FP32 + 4 x 2 KB BF16
constexpr int kMaxTileN = 128;        // largest GEMM1 N chunk

// Shared-memory and TMEM layout of the kernel for GEMM1 N chunk kN (AOs per TMEM accumulator):
//   kN = 64:  256 TMEM columns (hh, hm+mh, the 2^-16/2^-24 class, running sum: 64 each) and a 96 KB
//             operand stage (GEMM1 A 64 KB + B 32 KB), so that two CTAs share an SM;
//   kN = 128: all 512 TMEM columns of the SM and a 128 KB stage (A 64 KB + B 64 KB), one CTA per SM:
//             half the GEMM1 rounds and half the reloads of the A operand per batch.
// GEMM2 needs 6 x 16 KB of the stage and 256 TMEM columns in both.
template <int kN>
struct MixCfg {
  static_assert(kN == 64 || kN == 128, "GEMM1 N chunk of 64 or 128 AOs");
  static constexpr uint32_t kTmemCols = 4 * kN;
  static constexpr int kCtas = kN == 64 ? 2 : 1;                // resident CTAs per SM
  static constexpr int kStageBytes = 65536 + kN * 512;          // GEMM1 A 64 KB + B kN x 64 x 4 pieces
  static constexpr int kOffCoef = kStageBytes;                  // float [8][128]
  static constexpr int kOffAo = kOffCoef + 8 * 128 * 4;         // int [kMaxMixedM]
  static constexpr int kOffRed = kOffAo + kMaxMixedM * 4;       // double [3][kMT / 32]
  static constexpr int kOffEg = kOffRed + 3 * (kMT / 32) * 8;   // int [128]: per-point power-of-two scale
  static constexpr int kOffTab = kOffEg + 128 * 4;              // df32 [64]: 2^(-j/64)
  static constexpr int kOffFx = kOffTab + 64 * 8;               // int [kN]: row exponents of the chunk's AOs
  static constexpr int kOffMisc = kOffFx + kMaxTileN * 4;       // mbarriers, tmem slot, batch
  static constexpr int kSmemBytes = kOffMisc + 96 + 1024;       // + alignment slack
  static_assert(kRing * kRingBytes <= kStageBytes, "the epilogue ring lives in the stage");
  static_assert(6 * 16384 <= kStageBytes, "GEMM2's six image tiles live in the stage");
  static_assert(kCtas * (kSmemBytes + 1024) <= 233472, "the resident CTAs must fit in one SM's shared memory");
};
// dens [kGroups][4][128] doubles (8 KB) lives in the stage at +64 KB while the stage is idle
constexpr int kOffDensInStage = 65536;
static_assert(24 + 8 * kRing + 8 <= 64, "misc area holds the barriers, the TMEM slot, the batch index and the planes' base");
static_assert(64 + 8 * kRing <= 96, "the ring's release barriers follow at +64");

// (double)x for a normal float x, by moving its sign, exponent and mantissa fields: the same value
// as the conversion, with integer instructions only
__device__ __forceinline__ double normal_f32_to_f64(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t em = u & 0x7FFFFFFFu;
  return __hiloint2double((int)((u & 0x80000000u) | ((em >> 3) + ((1023u - 127u) << 20))), (int)(em << 29));
}

// (A) AO values and gradients in double-float.  Planes p = 0..3 (phi, d/dx, d/dy, d/dz) hold the
// FP32 hi parts at planes + p * P and the lo parts, rounded to BF16 (lo <= ulp(hi) / 2, so hi + lo
// keeps ~32 significant bits), at lo_planes + p * P; row = local AO, column = point.
// Returns the largest |phi| hi part this thread wrote (the point's row scale needs the maximum).
__device__ float ao_eval_df(const DevGrid& G, const BatchDesc& bd, float* __restrict__ planes,
                            __nv_bfloat16* __restrict__ lo_planes, size_t P, int m_k, const df32* tab) {
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
  for (int ci = tid >> 7; ci < bd.n_cand; ci += kMT / 128) {
    const int si = G.cand_shells[bd.cand_start + ci];
    const AoShellGpu sh = G.shells[si];
    const int loc = G.cand_loc[bd.cand_start + ci];
    df32 dx = {0.f, 0.f}, dy = {0.f, 0.f}, dz = {0.f, 0.f}, r0 = {0.f, 0.f}, r1 = {0.f, 0.f};
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
          r1 = df_sub(r1, df_add(ae, ae));
        }
        on = !(fabsf(r0.hi) < 1e-18f && fabsf(r1.hi) < 1e-18f);
      }
    }
    // per shell: r1 * (dx, dy, dz), and the squares for d shells
    df32 r1x = {0.f, 0.f}, r1y = r1x, r1z = r1x, x2 = r1x, y2 = r1x, z2 = r1x;
    if (on) {
      r1x = df_mul(r1, dx);
      r1y = df_mul(r1, dy);
      r1z = df_mul(r1, dz);
      if (sh.n_funcs == 6) {
        x2 = df_mul(dx, dx);
        y2 = df_mul(dy, dy);
        z2 = df_mul(dz, dz);
      }
    }
    for (int c = 0; c < sh.n_funcs; ++c) {
      df32 v = {0.f, 0.f}, gx = {0.f, 0.f}, gy = {0.f, 0.f}, gz = {0.f, 0.f};
      if (on) {
        const AoCompGpu cp = G.comps[sh.comp_start + c];
        const float2 sc = G.comp_f[sh.comp_start + c];
        const df32 s = {sc.x, sc.y};
        const int lsum = cp.lx + cp.ly + cp.lz;
        if (lsum <= 2) {
          // monomial mm = x^lx y^ly z^lz and its derivatives m_q (uniform branches: one component
          // per thread group); phi = s mm r0, d/dq phi = s (m_q r0 + mm r1 q)
          df32 mm = {1.f, 0.f};
          df32 mqx = {0.f, 0.f}, mqy = mqx, mqz = mqx;
          if (lsum == 1) {
            mm = cp.lx ? dx : (cp.ly ? dy : dz);
          } else if (lsum == 2) {
            if (cp.lx == 2) { mm = x2; mqx = df_mul_f(dx, 2.f); }
            else if (cp.ly == 2) { mm = y2; mqy = df_mul_f(dy, 2.f); }
            else if (cp.lz == 2) { mm = z2; mqz = df_mul_f(dz, 2.f); }
            else if (cp.lz == 0) { mm = df_mul(dx, dy); mqx = dy; mqy = dx; }
            else if (cp.ly == 0) { mm = df_mul(dx, dz); mqx = dz; mqz = dx; }
            else { mm = df_mul(dy, dz); mqy = dz; mqz = dy; }
          }
          v = df_mul(mm, r0);
          gx = df_mul(mm, r1x);
          gy = df_mul(mm, r1y);
          gz = df_mul(mm, r1z);
          if (lsum == 1) {  // m_q = 1 on the component's axis
            if (cp.lx) gx = df_add(gx, r0);
            else if (cp.ly) gy = df_add(gy, r0);
            else gz = df_add(gz, r0);
          } else if (lsum == 2) {
            if (cp.lx) gx = df_add(gx, df_mul(mqx, r0));
            if (cp.ly) gy = df_add(gy, df_mul(mqy, r0));
            if (cp.lz) gz = df_add(gz, df_mul(mqz, r0));
          }
          if (!(sc.x == 1.f && sc.y == 0.f)) {
            v = df_mul(s, v);
            gx = df_mul(s, gx);
            gy = df_mul(s, gy);
            gz = df_mul(s, gz);
          }
        } else {
          // x^l and its derivative l x^(l-1)
          df32 px = {1.f, 0.f}, dpx = {0.f, 0.f}, py = {1.f, 0.f}, dpy = {0.f, 0.f}, pz = {1.f, 0.f}, dpz = {0.f, 0.f};
          if (cp.lx >= 1) { dpx = px; px = dx; }
          if (cp.lx >= 2) { dpx = df_mul_f(dx, 2.f); px = df_mul(dx, dx); }
          if (cp.lx >= 3) { dpx = df_mul_f(px, 3.f); px = df_mul(px, dx); }
          if (cp.ly >= 1) { dpy = py; py = dy; }
          if (cp.ly >= 2) { dpy = df_mul_f(dy, 2.f); py = df_mul(dy, dy); }
          if (cp.ly >= 3) { dpy = df_mul_f(py, 3.f); py = df_mul(py, dy); }
          if (cp.lz >= 1) { dpz = pz; pz = dz; }
          if (cp.lz >= 2) { dpz = df_mul_f(dz, 2.f); pz = df_mul(dz, dz); }
          if (cp.lz >= 3) { dpz = df_mul_f(pz, 3.f); pz = df_mul(pz, dz); }
          const df32 yz = df_mul(py, pz), xz = df_mul(px, pz), xy = df_mul(px, py);
          const df32 mm = df_mul(px, yz);
          const df32 mr1 = df_mul(mm, r1);
          v = df_mul(s, df_mul(mm, r0));
          gx = df_mul(s, df_add(df_mul(df_mul(dpx, yz), r0), df_mul(mr1, dx)));
          gy = df_mul(s, df_add(df_mul(df_mul(dpy, xz), r0), df_mul(mr1, dy)));
          gz = df_mul(s, df_add(df_mul(df_mul(dpz, xy), r0), df_mul(mr1, dz)));
        }
        if (!(fabsf(v.hi) > 1e-16f || fabsf(gx.hi) > 1e-16f || fabsf(gy.hi) > 1e-16f || fabsf(gz.hi) > 1e-16f))
          v = gx = gy = gz = df32{0.f, 0.f};
      }
      const size_t o = (size_t)(loc + c) * 128 + g;
      vmax = fmaxf(vmax, fabsf(v.hi));
      planes[o] = v.hi;
      planes[P + o] = gx.hi;
      planes[2 * P + o] = gy.hi;
      planes[3 * P + o] = gz.hi;
      lo_planes[o] = __float2bfloat16_rn(v.lo);
      lo_planes[P + o] = __float2bfloat16_rn(gx.lo);
      lo_planes[2 * P + o] = __float2bfloat16_rn(gy.lo);
      lo_planes[3 * P + o] = __float2bfloat16_rn(gz.lo);
    }
  }
  // zero the rows [m, m_k) of the last GEMM1 K block (the A operand's padding must be finite zeros)
  const int pad = (m_k - bd.m) * 128;
  for (int e = tid; e < pad; e += kMT) {
    const size_t o = (size_t)bd.m * 128 + e;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      planes[p * P + o] = 0.f;
      lo_planes[p * P + o] = __float2bfloat16_rn(0.f);
    }
  }
  return vmax;
}

// (B) the GEMM1 A operand of the whole batch: for K block kb, tile q (q = 0..3: pieces of weight
// 2^-7, 2^-15, 2^-23, 2^-31) at apack + (4 kb + q) * 16 KB, 128 points x 64 AOs, 128-byte swizzle.
// Phi[g][mu] 2^-e_g from the double-float planes.
__device__ void pack_a(unsigned char* __restrict__ apack, const float* __restrict__ planes,
                       const __nv_bfloat16* __restrict__ lo_planes, const int* s_eg, int nkb) {
  for (int e = threadIdx.x; e < nkb * 128 * 8; e += kMT) {
    const int kb = e >> 10, g = e & 127, c = (e >> 7) & 7;
    const int mu0 = kb * 64 + c * 8;
    const int eg = s_eg[g];
    __nv_bfloat16 h[8], md[8], l[8], q[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const size_t o = (size_t)(mu0 + k) * 128 + g;
      fixsplit4(ldexpf(planes[o], -eg), ldexpf(__bfloat162float(lo_planes[o]), -eg), h[k], md[k], l[k], q[k]);
    }
    unsigned char* t = apack + (size_t)kb * 65536 + sw128(g, c);
    *reinterpret_cast<uint4*>(t) = pack8v(h);
    *reinterpret_cast<uint4*>(t + 16384) = pack8v(md);
    *reinterpret_cast<uint4*>(t + 32768) = pack8v(l);
    *reinterpret_cast<uint4*>(t + 49152) = pack8v(q);
  }
}

// Byte offset of GEMM2 image tile (piece p: 0..2 Phi^T, 3..5 Z^T; AO row block ib; point block kb2)
// in the slab's image area; each tile is 128 AO rows x 64 points, 128-byte swizzle.
__device__ __forceinline__ size_t img_tile(int p, int ib, int kb2, int n_ib) {
  return (((size_t)p * n_ib + ib) * 2 + kb2) * 16384;
}

// Three CTA-wide sums with one barrier: warp shuffles, then thread 0 adds the warps' partials in
// order (the results are valid in thread 0).
__device__ __forceinline__ void cta_sum3(double (&v)[3], double (*red)[kMT / 32]) {
#pragma unroll
  for (int q = 0; q < 3; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v[q];
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double s = 0;
      for (int k = 0; k < kMT / 32; ++k) s += red[q][k];
      v[q] = s;
    }
}

}  // namespace

// kCache: the grid has an AO cache (EvalArgs::ao_cache); the instantiation without it keeps the
// batch's planes in the CTA's slab at fixed addresses.  kN: GEMM1 N chunk (MixCfg).
template <bool kCache, int kN>
__global__ void __launch_bounds__(kMT, MixCfg<kN>::kCtas) vxc_mixed_kernel(DevGrid G, EvalArgs A) {
  using Cfg = MixCfg<kN>;
  constexpr int kOffCoef = Cfg::kOffCoef, kOffAo = Cfg::kOffAo, kOffRed = Cfg::kOffRed, kOffEg = Cfg::kOffEg;
  constexpr int kOffTab = Cfg::kOffTab, kOffFx = Cfg::kOffFx, kOffMisc = Cfg::kOffMisc;
  constexpr uint32_t kTmemCols = Cfg::kTmemCols;
  constexpr int kNc = kN;  // GEMM1 N chunk of this instantiation
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* stage = base;
  float(*coef)[128] = reinterpret_cast<float(*)[128]>(base + kOffCoef);
  double(*dens)[4][128] = reinterpret_cast<double(*)[4][128]>(base + kOffDensInStage);  // [kGroups], stage idle
  int* s_ao = reinterpret_cast<int*>(base + kOffAo);
  double(*red)[kMT / 32] = reinterpret_cast<double(*)[kMT / 32]>(base + kOffRed);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(base + kOffMisc);      // MMA commits
  uint64_t* tbar = reinterpret_cast<uint64_t*>(base + kOffMisc + 8);  // operand bulk copies
  uint64_t* ring = reinterpret_cast<uint64_t*>(base + kOffMisc + 16); // kRing barriers of the epilogue ring
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(base + kOffMisc + 16 + 8 * kRing);
  int* s_batch = reinterpret_cast<int*>(base + kOffMisc + 20 + 8 * kRing);
  // the batch's planes (the AO cache block or the slab), kept in shared memory rather than in a
  // register for the whole batch: read back where needed
  float** s_planes = reinterpret_cast<float**>(base + kOffMisc + 24 + 8 * kRing);
  // per ring buffer: every warp arrives once it has read the buffer; the thread that refills it waits
  uint64_t* ring_free = reinterpret_cast<uint64_t*>(base + kOffMisc + 64);
  int* s_eg = reinterpret_cast<int*>(base + kOffEg);
  df32* s_tab = reinterpret_cast<df32*>(base + kOffTab);
  float* s_fs = reinterpret_cast<float*>(base + kOffFx);  // 2^f of the chunk's density rows

  const int tid = threadIdx.x, warp = tid >> 5;
  const int g = tid & 127, h = tid >> 7;
  const bool uks = A.mode == kModeUks;
  const int nspin = uks ? 2 : 1;
  // grad rho by FP32 FMA sums, except where per-point or per-atom shares are asked for: the judge
  // of a learned grid compares atoms' shares from different batch plans to ~1e-9 Eh, and the FMA
  // sums' roundings (~5e-10 on an oxygen's share) follow the batch's set of AOs
  const bool fma_grad = A.point_out == nullptr && !A.shares_only;

  if (tid == 0) {
    mbar_init(mbar, 1);
    mbar_init(tbar, 1);
    for (int r = 0; r < kRing; ++r) mbar_init(ring + r, 1);
    for (int r = 0; r < kRing; ++r) mbar_init(ring_free + r, kMT / 32);
    fence_mbar_init();
  }
  if (tid < 64) s_tab[tid] = df_from_double(exp2(-(double)tid / 64.0));
  if (warp == 0) {
    tmem_alloc(tmem_slot, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
  // TMEM: GEMM1 uses four kN-column accumulators (hh, hm+mh, hl+mm+lh, running sum); GEMM2, which
  // runs after GEMM1 is finished, uses 128 columns for its hh products and 128 for its corrections.
  const uint32_t tH = tmem, tC1 = tmem + kN, tC2 = tmem + 2 * kN, tS = tmem + 3 * kN;
  const uint32_t tW = tmem, tWc = tmem + 128;
  uint32_t phase = 0, tphase = 0;
  uint32_t ring_uses[kRing] = {0, 0, 0, 0};  // uses of each buffer (its fill and release phases alike)
  bool ring_busy[kRing] = {false, false, false, false};  // a bulk copy issued and not yet waited for
  bool tma_busy = false;
  bool failed = false;

  const int m_pad_all = (A.max_m + 127) / 128 * 128;
  const int n_ib = m_pad_all / 128;
  // the CTA's scratch slab: FP32 planes [4][m_pad_all][128], BF16 planes, the packed operand
  // (m_pad_all / 64 x 64 KB), the GEMM2 image tiles (6 x n_ib x 2 x 16 KB)
  const size_t P_slab = (size_t)m_pad_all * 128;  // floats per plane
  float* const planes_slab = reinterpret_cast<float*>(A.slab + (size_t)blockIdx.x * A.slab_stride);
  unsigned char* const img = reinterpret_cast<unsigned char*>(planes_slab + 4 * P_slab) + P_slab * 4 * 2 +
                             (size_t)m_pad_all * 1024;
  const uint2* Dhl_a0 = reinterpret_cast<const uint2*>(A.Pa);
  const uint2* Dhl_b0 = Dhl_a0 + G.nn_total;
  const int* fexp_a0 = reinterpret_cast<const int*>(Dhl_a0 + 2 * G.nn_total);
  const int* fexp_b0 = fexp_a0 + G.n_total;
  const uint32_t sb = smem_addr(stage);
  // L2 policies: the packed A operand and the GEMM2 image tiles are read again (per N chunk, per
  // tile pair); the BF16 low planes are read for the last time by the GEMM1 epilogue
  const uint64_t pol_keep = l2_policy_evict_last(), pol_last_use = l2_policy_evict_first();

  // one MMA round: wait for the commit of the round just issued
  auto wait_mma = [&]() -> bool {
    const bool ok = mbar_wait_bounded(mbar, phase, kWaitLimit);
    phase ^= 1u;
    tc_fence_after();
    return __syncthreads_or(!ok) == 0;
  };
  // operand bulk copies of this round (issued by thread 0 with expect_tx)
  auto wait_tma = [&]() -> bool {
    const bool ok = mbar_wait_bounded(tbar, tphase, kWaitLimit);
    if (ok) {
      tphase ^= 1u;
      tma_busy = false;
    }
    return __syncthreads_or(!ok) == 0;
  };

  while (!failed) {
    if (tid == 0) *s_batch = atomicAdd(A.counter + 1, 1);
    __syncthreads();
    const int q = *s_batch;
    __syncthreads();
    if (q >= G.n_batches) break;
    const int b = G.order[q];
    const BatchDesc bd = G.batches[b];
    const int m = bd.m;
    const int n = mol_nao(G, bd.mol);
    const long long moff = mol_mat(G, bd.mol);
    const int roff = mol_row(G, bd.mol);
    const int nkb = (m + 63) / 64;
    for (int i = tid; i < m; i += kMT) s_ao[i] = G.batch_ao[bd.ao_start + i];
    // the batch's AO planes, packed operand and row exponents: in the AO cache when the grid has
    // one with a block for this batch (written by the first launch that reaches the batch, read by
    // later ones), else in the CTA's scratch slab -- with a cache, a batch without a block is laid
    // out as a block at the slab's start (P <= P_slab, so it ends before the slab's image tiles)
    // (both layouts: the FP32 planes, then the BF16 planes, then the packed operand)
    long long cache_off = -1;
    if constexpr (kCache) cache_off = A.ao_cache_off[b];
    const bool in_cache = cache_off >= 0;
    const size_t P = kCache ? (size_t)nkb * 64 * 128 : P_slab;  // floats per plane
    auto batch_planes = [&]() -> float* {
      if constexpr (kCache) return *reinterpret_cast<float* volatile*>(s_planes);
      return planes_slab;
    };
    bool cached = false;
    if constexpr (kCache) {
      if (tid == 0) *s_planes = in_cache ? reinterpret_cast<float*>(A.ao_cache + cache_off) : planes_slab;
      // the flag has the same value in every thread: only this CTA writes it, after the reads below
      cached = in_cache && *reinterpret_cast<volatile int*>(A.ao_cache_ok + b) != 0;
      __syncthreads();
    }
    if (cached) {
      const int* eg_cached = reinterpret_cast<const int*>(
          reinterpret_cast<const unsigned char*>(batch_planes() + 6 * P) + (size_t)nkb * 65536);
      if (h == 0) s_eg[g] = eg_cached[g];
      __syncthreads();
    } else {
      float* const planes = batch_planes();
      __nv_bfloat16* const lo_planes = reinterpret_cast<__nv_bfloat16*>(planes + 4 * P);
      unsigned char* const apack = reinterpret_cast<unsigned char*>(lo_planes + 4 * P);
      int* const eg_cached = in_cache ? reinterpret_cast<int*>(apack + (size_t)nkb * 65536) : nullptr;
      const float vmax = ao_eval_df(G, bd, planes, lo_planes, P, nkb * 64, s_tab);
      {  // e_g: power-of-two exponent with max_mu |Phi[g][mu]| 2^-e_g < 1
        dens[0][0][g + 128 * h] = (double)vmax;  // scratch: the stage is idle
        __syncthreads();
        if (h == 0) {
          float t = 0.f;
          for (int k = 0; k < kGroups; ++k) t = fmaxf(t, (float)dens[0][0][g + 128 * k]);
          int ex = 0;
          frexpf(t, &ex);
          s_eg[g] = ex;
          if (eg_cached) eg_cached[g] = ex;
        }
        __syncthreads();
      }
      pack_a(apack, planes, lo_planes, s_eg, nkb);
      fence_proxy_async_global();  // the packed tiles are read by bulk copies
      __syncthreads();
      if (eg_cached && tid == 0) {
        __threadfence();
        A.ao_cache_ok[b] = 1;  // read by later launches only
      }
    }

    double spin_rho[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int s = 0; s < nspin && !failed; ++s) {
      const uint2* Dhl = (s ? Dhl_b0 : Dhl_a0) + moff;
      const int* fexp = (s ? fexp_b0 : fexp_a0) + roff;
      const int eg = s_eg[g];
      CompSum sr, sgx, sgy, sgz;
      const uint32_t idesc = idesc_bf16_f32(128, kNc);
      for (int nc = 0; nc < m && !failed; nc += kNc) {
        // the density rows' power-of-two scales 2^f for this chunk's AOs (read in the epilogue; the
        // barriers of the K loop order the writes before it)
        if (tid < kNc) s_fs[tid] = pow2f(nc + tid < m ? fexp[s_ao[nc + tid]] : 0);
        for (int kb = 0; kb < nkb; ++kb) {
          if (tid == 0) {  // A operand of this K block: four 16 KB tiles
            mbar_arrive_expect_tx(tbar, 65536);
#pragma unroll
            for (int t = 0; t < 4; ++t)
              bulk_g2s_hint(sb + t * 16384,
                            reinterpret_cast<unsigned char*>(batch_planes() + 6 * P) + (size_t)kb * 65536 + t * 16384,
                            16384, tbar, pol_keep);
            tma_busy = true;
          }
          gather_b<kN>(stage, Dhl, s_ao, n, m, kb, nc);
          fence_proxy_async_smem();
          if (!wait_tma()) { failed = true; break; }
          if (tid == 0) {
            tc_fence_after();
            const uint64_t ah = sdesc_sw128(sb), am = sdesc_sw128(sb + 16384), al = sdesc_sw128(sb + 32768);
            const uint64_t aq = sdesc_sw128(sb + 49152);
            // B pieces: kN rows of 128 bytes each, one after the other from +64 KB
            const uint64_t bh = sdesc_sw128(sb + 65536), bm = sdesc_sw128(sb + 65536 + kN * 128);
            const uint64_t bl = sdesc_sw128(sb + 65536 + 2 * kN * 128), bq = sdesc_sw128(sb + 65536 + 3 * kN * 128);
            const bool group_start = (kb & 15) == 0;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint64_t o = (uint64_t)(ks * 2);  // 32 bytes per K step of 16 BF16
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
          if (!wait_mma()) { failed = true; break; }
          const bool group_end = ((kb & 15) == 15) || kb == nkb - 1;
          if (!group_end) continue;
          const bool first_group = kb < 16, last_group = kb == nkb - 1;
          if (!last_group) {
            // running sum S += hh + corrections (contractions longer than 1024 AOs)
            for (int c0 = h * (kNc / kGroups); c0 < (h + 1) * (kNc / kGroups); c0 += 16) {
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
            // rho = sum Phi T and grad rho terms over the chunk's 64 AOs.  The planes of the chunk's
            // rows stream through the (now idle) stage in steps of 8 rows (24 KB), kRing steps in
            // flight; in step st group h takes the four columns 8 st + 4 h .. + 3.
            const int n_steps = min(kNc / 8, (m - nc + 7) / 8);
            auto issue = [&](int st) {  // 8 rows: 4 FP32 hi planes (4 KB each), 4 BF16 lo planes (2 KB)
              const int r = st % kRing;
              mbar_arrive_expect_tx(ring + r, 4 * 4096 + 4 * 2048);
              const size_t row0 = (size_t)(nc + 8 * st) * 128;
              const float* planes = batch_planes();
              const __nv_bfloat16* lo_planes = reinterpret_cast<const __nv_bfloat16*>(planes + 4 * P);
#pragma unroll
              for (int pl = 0; pl < 4; ++pl) {
                bulk_g2s(sb + r * kRingBytes + pl * 4096, planes + pl * P + row0, 4096, ring + r);
                bulk_g2s_hint(sb + r * kRingBytes + 16384 + pl * 2048, lo_planes + pl * P + row0, 2048, ring + r,
                              pol_last_use);
              }
              ring_busy[r] = true;
            };
            if (tid == 0) {
              fence_proxy_async_smem();
              for (int st = 0; st < min(kRing, n_steps); ++st) issue(st);
            }
            // each buffer is released by an arrival of every warp (no block-wide barrier per step); an
            // expired wait marks the chunk failed, and the flag is combined after the loop
            bool efail = false;
            // the step loop, compiled once per form of the grad rho sums and per K group kind (a branch
            // per product would be predicated and issue both forms)
            auto steps = [&](auto fma_form, auto first_form) {
              constexpr bool kFma = decltype(fma_form)::value, kFirst = decltype(first_form)::value;
              for (int st = 0; st < n_steps; ++st) {
                const int r = st % kRing;
                const bool ok = !efail && mbar_wait_bounded(ring + r, ring_uses[r] & 1u, kWaitLimit);
                if (ok) {  // on expiry the copy stays pending and teardown waits for it again
                  ring_uses[r]++;
                  ring_busy[r] = false;
                } else {
                  efail = true;
                }
                const int c0 = 8 * st + 4 * h;
                const uint32_t tl = lane_base + (uint32_t)c0;
                float a[4], bb[4], c2[4], cc[4];
                if constexpr (kFirst)
                  tmem_ld4x3(tH + tl, tC1 + tl, tC2 + tl, a, bb, c2);
                else
                  tmem_ld4x4(tH + tl, tC1 + tl, tC2 + tl, tS + tl, a, bb, c2, cc);
#pragma unroll
                for (int j = 0; j < 4; ++j) bb[j] += c2[j];
                const float* buf = reinterpret_cast<const float*>(stage + r * kRingBytes);
                const __nv_bfloat16* lbuf = reinterpret_cast<const __nv_bfloat16*>(stage + r * kRingBytes + 16384);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                  const int nu = nc + c0 + j;
                  if (ok && nu < m) {
                    df32 t;
                    if constexpr (kFirst)
                      t = two_sum(a[j], bb[j]);
                    else
                      t = df_add_f(two_sum(cc[j], a[j]), bb[j]);
                    const float sc = s_fs[c0 + j];
                    t = df32{t.hi * sc, t.lo * sc};
                    const int o = (4 * h + j) * 128 + g;  // row within the step, point g
                    acc_prod(sr, df32{buf[o], __bfloat162float(lbuf[o])}, t);
                    const df32 xg = {buf[1024 + o], __bfloat162float(lbuf[1024 + o])};
                    const df32 yg = {buf[2 * 1024 + o], __bfloat162float(lbuf[2 * 1024 + o])};
                    const df32 zg = {buf[3 * 1024 + o], __bfloat162float(lbuf[3 * 1024 + o])};
                    if constexpr (kFma) {
                      acc_prod_fma(sgx, xg, t);
                      acc_prod_fma(sgy, yg, t);
                      acc_prod_fma(sgz, zg, t);
                    } else {
                      acc_prod(sgx, xg, t);
                      acc_prod(sgy, yg, t);
                      acc_prod(sgz, zg, t);
                    }
                  }
                }
                __syncwarp();
                if ((tid & 31) == 0) mbar_arrive(ring_free + r);  // this warp is done with buffer r
                if (tid == 0 && st + kRing < n_steps) {
                  // refill buffer r once every warp has released it (the release of this use: the
                  // phase with the parity of the use's index)
                  if (!efail && mbar_wait_bounded(ring_free + r, (ring_uses[r] - 1u) & 1u, kWaitLimit)) {
                    fence_proxy_async_smem();
                    issue(st + kRing);
                  } else {
                    efail = true;
                  }
                }
              }
            };
            if (fma_grad) {
              if (first_group)
                steps(std::true_type{}, std::true_type{});
              else
                steps(std::true_type{}, std::false_type{});
            } else {
              if (first_group)
                steps(std::false_type{}, std::true_type{});
              else
                steps(std::false_type{}, std::false_type{});
            }
            if (__syncthreads_or(efail)) { failed = true; break; }
          }
          tc_fence_before();
          __syncthreads();
        }
      }
      // the point's scale 2^e_g, applied to the sums (exact)
      const double seg = ldexp(1.0, eg);
      double acc[4] = {sr.value() * seg, sgx.value() * seg, sgy.value() * seg, sgz.value() * seg};
      if (failed) break;
      for (int k = 0; k < 4; ++k) dens[h][k][g] = acc[k];
      __syncthreads();
      for (int k = 0; k < 4; ++k) {
        double t = dens[0][k][g];
        for (int j = 1; j < kGroups; ++j) t += dens[j][k][g];
        spin_rho[s][k] = t;
      }
      __syncthreads();
    }
    if (failed) break;

    // (E) functional, one thread per point (threads with h == 0).  The closed-shell functional is
    // split between the halves: part 0 of xc_eval_cs_df (exchange and VWN) in threads h == 0, part 1
    // in threads h == 1 (passed through dens, idle until the image pass), summed as xc_eval_cs_fast
    // sums them.
    XcCs xpart{0.0, 0.0, 0.0};
    if (!uks && A.mode != kModeFxc) {
      const double ra = spin_rho[0][0];
      if (g < bd.n_pts && !(ra < 1e-18)) {
        const double gax = 2.0 * spin_rho[0][1], gay = 2.0 * spin_rho[0][2], gaz = 2.0 * spin_rho[0][3];
        xpart = xc_eval_cs_fast_part(A.xc, 0.5 * ra, 0.25 * (gax * gax + gay * gay + gaz * gaz), s_tab, h);
      }
      if (h == 1) {
        dens[1][0][g] = xpart.f;
        dens[1][1][g] = xpart.vr;
        dens[1][2][g] = xpart.vg;
      }
      __syncthreads();
    }
    double e_loc = 0, na_loc = 0, nb_loc = 0;
    if (h == 0) {
      const bool live = g < bd.n_pts;
      for (int k = 0; k < 8; ++k) coef[k][g] = 0.f;
      const double ra = spin_rho[0][0];
      const double gax = 2.0 * spin_rho[0][1], gay = 2.0 * spin_rho[0][2], gaz = 2.0 * spin_rho[0][3];
      const size_t pt = (size_t)bd.pt_start + g;
      if (A.mode == kModeFxc) {
        // TD-DFT kernel contraction (fxc.rs:374-645; the FP64 form's coefficients): the batch's
        // density is the trial matrix M, so ra = eta = sum M phi phi and (gax, gay, gaz) = xi
        if (live) {
          const double* c = A.fxc_coef + 11 * pt;
          const double* kc = c + (A.triplet ? 7 : 3);
          const double w = G.pw[pt];
          const double sigma = c[0] * gax + c[1] * gay + c[2] * gaz;
          const double dv = kc[0] * ra + kc[1] * sigma;
          const double gc = kc[1] * ra + kc[2] * sigma;
          coef[0][g] = (float)(0.5 * w * dv);
          coef[1][g] = (float)(w * (kc[3] * gax + gc * c[0]));
          coef[2][g] = (float)(w * (kc[3] * gay + gc * c[1]));
          coef[3][g] = (float)(w * (kc[3] * gaz + gc * c[2]));
        }
      } else if (!uks) {
        if (live && !(ra < 1e-18)) {
          const double w = G.pw[pt];
          const XcCs o{xpart.f + dens[1][0][g], xpart.vr + dens[1][1][g], xpart.vg + dens[1][2][g]};
          e_loc = w * o.f;
          na_loc = w * ra;
          const double us = w * o.vg;
          coef[0][g] = (float)(0.5 * w * o.vr);
          coef[1][g] = (float)(us * gax);
          coef[2][g] = (float)(us * gay);
          coef[3][g] = (float)(us * gaz);
          if (A.point_out) {
            A.point_out[2 * pt] = e_loc;
            A.point_out[2 * pt + 1] = w * o.vr * ra + us * (gax * gax + gay * gay + gaz * gaz);
          }
        }
      } else {
        const double rb0 = spin_rho[1][0];
        const double gbx = 2.0 * spin_rho[1][1], gby = 2.0 * spin_rho[1][2], gbz = 2.0 * spin_rho[1][3];
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
          coef[0][g] = (float)(0.5 * w * o.vra);
          coef[1][g] = (float)(w * (2.0 * o.vgaa * gax + o.vgab * gbx));
          coef[2][g] = (float)(w * (2.0 * o.vgaa * gay + o.vgab * gby));
          coef[3][g] = (float)(w * (2.0 * o.vgaa * gaz + o.vgab * gbz));
          coef[4][g] = (float)(0.5 * w * o.vrb);
          coef[5][g] = (float)(w * (2.0 * o.vgbb * gbx + o.vgab * gax));
          coef[6][g] = (float)(w * (2.0 * o.vgbb * gby + o.vgab * gay));
          coef[7][g] = (float)(w * (2.0 * o.vgbb * gbz + o.vgab * gaz));
        }
      }
    }
    __syncthreads();
    {
      double sums[3] = {e_loc, na_loc, nb_loc};
      cta_sum3(sums, red);
      if (tid == 0) {
        A.batch_red[3 * (size_t)b] = sums[0];
        A.batch_red[3 * (size_t)b + 1] = sums[1];
        A.batch_red[3 * (size_t)b + 2] = sums[2];
      }
    }
    // per-point shares only: no GEMM2 and no V update (cta_sum3's barrier follows the last reads of
    // the stage and of coef, so the next batch may reuse them)
    if (A.shares_only) continue;

    // (F)+(G) per spin: image tiles Phi^T / Z^T, then lower tile pairs of W.  Rows [m, 128 n_ib) of
    // the tiles are left as they are: a W entry depends on its own row of A and of B only, and the
    // drain reads rows and columns below m.
    const uint32_t idesc2 = idesc_bf16_f32(128, 128);
    // 8 points (c16 * 8 ..) of AO row mu: Phi^T and Z^T, three BF16 pieces each
    const float* const planes = batch_planes();
    auto image8 = [&](const float (&cz)[4][8], int mu, int c16, uint4 (&p3)[3], uint4 (&z3)[3]) {
      const size_t o = (size_t)mu * 128 + c16 * 8;
      float ph[8], zz[8];
      // the hi planes' last use in the batch: streaming loads (first in line for eviction)
      const float4 p0 = __ldcs(reinterpret_cast<const float4*>(planes + o));
      const float4 p1 = __ldcs(reinterpret_cast<const float4*>(planes + o + 4));
      const float4 x0 = __ldcs(reinterpret_cast<const float4*>(planes + P + o));
      const float4 x1 = __ldcs(reinterpret_cast<const float4*>(planes + P + o + 4));
      const float4 y0 = __ldcs(reinterpret_cast<const float4*>(planes + 2 * P + o));
      const float4 y1 = __ldcs(reinterpret_cast<const float4*>(planes + 2 * P + o + 4));
      const float4 z0 = __ldcs(reinterpret_cast<const float4*>(planes + 3 * P + o));
      const float4 z1 = __ldcs(reinterpret_cast<const float4*>(planes + 3 * P + o + 4));
      ph[0] = p0.x; ph[1] = p0.y; ph[2] = p0.z; ph[3] = p0.w; ph[4] = p1.x; ph[5] = p1.y; ph[6] = p1.z; ph[7] = p1.w;
      const float dxv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
      const float dyv[8] = {y0.x, y0.y, y0.z, y0.w, y1.x, y1.y, y1.z, y1.w};
      const float dzv[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        zz[k] = cz[0][k] * ph[k] + cz[1][k] * dxv[k] + cz[2][k] * dyv[k] + cz[3][k] * dzv[k];
      }
      pack8x3(ph, p3[0], p3[1], p3[2]);
      pack8x3(zz, z3[0], z3[1], z3[2]);
    };
    // one K step of 64 points for a tile pair whose A and B images sit at stage slots da.. and db..
    auto mma_half = [&](int da, int db, bool first) {
      uint64_t d[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) d[t] = sdesc_sw128(sb + t * 16384);
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const uint64_t o = (uint64_t)(ks * 2);
        const uint32_t acc = (!first || ks > 0) ? 1u : 0u;
        mma_bf16_ss(tW, d[da] + o, d[db] + o, idesc2, acc);
        mma_bf16_ss(tWc, d[da] + o, d[db + 1] + o, idesc2, acc);
        mma_bf16_ss(tWc, d[da + 1] + o, d[db] + o, idesc2, 1u);
        mma_bf16_ss(tWc, d[da] + o, d[db + 2] + o, idesc2, 1u);
        mma_bf16_ss(tWc, d[da + 1] + o, d[db + 1] + o, idesc2, 1u);
        mma_bf16_ss(tWc, d[da + 2] + o, d[db] + o, idesc2, 1u);
      }
    };
    // drain: lane = AO row i of tile I, this group's 64 columns of tile J
    auto drain = [&](double* V, int I, int J) {
      const int i = I + g;
      const int row0 = I + 32 * (warp & 3);  // the warp's first row (its TMEM lanes)
      for (int c0 = h * 64; c0 < h * 64 + 64; c0 += 32) {
        // a 32-column block none of whose entries the warp adds (columns beyond m, rows beyond m, or
        // in the diagonal tile columns above every row of the warp) is skipped by the whole warp
        if (J + c0 >= m || row0 >= m || (I == J && c0 > 32 * (warp & 3) + 31)) continue;
        float wv[32], wc[32];
        tmem_ld32(tW + lane_base + (uint32_t)c0, wv);
        tmem_ld32(tWc + lane_base + (uint32_t)c0, wc);
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) wv[jj] += wc[jj];
        if (i < m) {
          const int ai = s_ao[i];
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {
            const int j = J + c0 + jj;
            // contributions below 1e-11 are not added: most AO pairs of a compact batch involve an
            // AO near the edge of its cut-off sphere (values down to ~1e-18 at the batch's points),
            // and skipping their updates changes an element of V by < 1e-11 per batch, far below
            // this form's ~1e-6 agreement with FP64 (max |dV| against FP64 on (H2O)61 and C8H18 the
            // same to three digits at 1e-13 and 1e-11), while it removes most of the FP64 atomics
            if (j < m && (I != J || i >= j) && fabsf(wv[jj]) >= 1e-11f) {
              const int aj = s_ao[j];
              const int r = ai < aj ? ai : aj, c = ai < aj ? aj : ai;
              atomicAdd(&V[(size_t)r * n + c], normal_f32_to_f64(wv[jj]));
            }
          }
        }
      }
      tc_fence_before();
      __syncthreads();
    };
    for (int s = 0; s < nspin && !failed; ++s) {
      double* V = (s ? A.Vb : A.Va) + moff;
      if (m <= 128) {
        // one tile pair: the six image tiles of each 64-point K half are built in the stage and
        // consumed there (slots 0..2 Phi^T, 3..5 Z^T), with no global round trip
        for (int kb2 = 0; kb2 < 2 && !failed; ++kb2) {
          float cz[4][8];  // this thread's 8 points (the same in every row)
#pragma unroll
          for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) cz[k][kk] = coef[4 * s + k][(kb2 * 8 + (tid & 7)) * 8 + kk];
          for (int e = tid; e < m * 8; e += kMT) {
            const int mu = e >> 3, cc = e & 7;
            uint4 p3[3], z3[3];
            image8(cz, mu, kb2 * 8 + cc, p3, z3);
            const uint32_t sw = sw128(mu, cc);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
              *reinterpret_cast<uint4*>(stage + t * 16384 + sw) = p3[t];
              *reinterpret_cast<uint4*>(stage + (3 + t) * 16384 + sw) = z3[t];
            }
          }
          fence_proxy_async_smem();  // the tiles are read by the tensor core
          __syncthreads();
          if (tid == 0) {
            tc_fence_after();
            mma_half(3, 0, kb2 == 0);  // A = Z, B = Phi
            mma_half(0, 3, false);     // A = Phi, B = Z
            mma_commit(mbar);
          }
          if (!wait_mma()) { failed = true; break; }
        }
        if (failed) break;
        drain(V, 0, 0);
        continue;
      }
      float cz[4][8];  // this thread's 8 points (the same in every row)
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) cz[k][kk] = coef[4 * s + k][(tid & 15) * 8 + kk];
      for (int e = tid; e < m * 16; e += kMT) {
        const int mu = e >> 4, c16 = e & 15;
        uint4 p3[3], z3[3];
        image8(cz, mu, c16, p3, z3);
        const int ib = mu >> 7, r = mu & 127, kb2 = c16 >> 3, cc = c16 & 7;
        const uint32_t sw = sw128(r, cc);
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          if (s == 0) *reinterpret_cast<uint4*>(img + img_tile(t, ib, kb2, n_ib) + sw) = p3[t];
          *reinterpret_cast<uint4*>(img + img_tile(3 + t, ib, kb2, n_ib) + sw) = z3[t];
        }
      }
      fence_proxy_async_global();  // the tiles are read by bulk copies
      __syncthreads();
      for (int I = 0; I < m && !failed; I += 128) {
        for (int J = 0; J <= I && !failed; J += 128) {
          // four rounds: (kb2, half); half 0 A = Z_I, B = Phi_J; half 1 A = Phi_I, B = Z_J
          for (int rnd = 0; rnd < 4; ++rnd) {
            const int kb2 = rnd >> 1, half = rnd & 1;
            if (tid == 0) {
              mbar_arrive_expect_tx(tbar, 6 * 16384);
              const int pa = half ? 0 : 3, pb = half ? 3 : 0;  // first piece of the A and B images
#pragma unroll
              for (int t = 0; t < 3; ++t) {
                bulk_g2s_hint(sb + t * 16384, img + img_tile(pa + t, I >> 7, kb2, n_ib), 16384, tbar, pol_keep);
                bulk_g2s_hint(sb + (3 + t) * 16384, img + img_tile(pb + t, J >> 7, kb2, n_ib), 16384, tbar, pol_keep);
              }
              tma_busy = true;
            }
            if (!wait_tma()) { failed = true; break; }
            if (tid == 0) {
              tc_fence_after();
              mma_half(0, 3, rnd == 0);  // d[0..2] A (hi, mid, lo), d[3..5] B (hi, mid, lo)
              mma_commit(mbar);
            }
            if (!wait_mma()) { failed = true; break; }
          }
          if (failed) break;
          drain(V, I, J);
        }
      }
    }
  }

  // teardown: on failure, give the MMAs and bulk copies in flight a bounded chance to finish
  if (failed) {
    if (tid == 0) atomicExch(A.counter + 2, 1);
    mbar_wait_bounded(mbar, phase ^ 1u, kWaitLimit);  // the round that timed out
    if (tma_busy) mbar_wait_bounded(tbar, tphase, kWaitLimit);
    for (int r = 0; r < kRing; ++r)
      if (ring_busy[r]) mbar_wait_bounded(ring + r, ring_uses[r] & 1u, kWaitLimit);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// D (FP64, n x n) -> per-row fixed-point split: row nu is scaled by 2^-f_nu (|x| < 1) and cut into
// multiples of 2^-7, 2^-15, 2^-23, 2^-31 (computed in FP64, each exact in BF16); packed as
// x = hi | mid << 16, y = lo | lo2 << 16.  One CTA per row.
__global__ void __launch_bounds__(256) split_density_kernel(const double* __restrict__ D, int n_single,
                                                           const int* __restrict__ mol_n,
                                                           const long long* __restrict__ mol_off,
                                                           const int* __restrict__ mol_ao_off, int n_mols,
                                                           uint2* __restrict__ out, int* __restrict__ fexp) {
  __shared__ double red[256];
  // packed row r belongs to the molecule whose row range [mol_ao_off[i], mol_ao_off[i + 1]) holds it
  int mol = 0;
  if (mol_ao_off) {
    int lo = 0, hi = n_mols - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (mol_ao_off[mid] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    mol = lo;
  }
  const int n = mol_n ? mol_n[mol] : n_single;
  const int row = (int)blockIdx.x - (mol_ao_off ? mol_ao_off[mol] : 0);
  D += mol_off ? mol_off[mol] : 0ll;
  out += mol_off ? mol_off[mol] : 0ll;
  const double* d = D + (size_t)row * n;
  double mx = 0.0;
  for (int j = threadIdx.x; j < n; j += 256) mx = fmax(mx, fabs(d[j]));
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  int f = 0;
  frexp(red[0], &f);
  if (threadIdx.x == 0) fexp[blockIdx.x] = f;
  for (int j = threadIdx.x; j < n; j += 256) {
    const double x = ldexp(d[j], -f);
    const double h = rint(x * 128.0) / 128.0;
    const double r1 = x - h;
    const double m = rint(r1 * 32768.0) / 32768.0;
    const double r2 = r1 - m;
    const double l = rint(r2 * 8388608.0) / 8388608.0;
    const double r3 = r2 - l;
    const double q = rint(r3 * 2147483648.0) / 2147483648.0;
    out[(size_t)row * n + j] = make_uint2(pack_bf16x2(__float2bfloat16_rn((float)h), __float2bfloat16_rn((float)m)),
                                          pack_bf16x2(__float2bfloat16_rn((float)l), __float2bfloat16_rn((float)q)));
  }
}

// The closed-shell point functional at n points (rho_a = rho_b = rho[i], all gammas = gam[i]):
// out[3 i ..] = (f, v_rho_a, v_gamma_aa + v_gamma_ab / 2), the FP64 form (precision 0) or the form the
// tensor-core kernels use (precision 1).
__global__ void __launch_bounds__(256) closed_shell_points_kernel(int xc, int precision, int n,
                                                                 const double* __restrict__ rho,
                                                                 const double* __restrict__ gam,
                                                                 double* __restrict__ out) {
  __shared__ df32 tab[64];
  if (threadIdx.x < 64) tab[threadIdx.x] = df_from_double(exp2(-(double)threadIdx.x / 64.0));
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const XcCs o = precision ? xc_eval_cs_fast(xc, rho[i], gam[i], tab) : xc_eval_cs(xc, rho[i], gam[i]);
    out[3 * (size_t)i] = o.f;
    out[3 * (size_t)i + 1] = o.vr;
    out[3 * (size_t)i + 2] = o.vg;
  }
}

cudaError_t launch_closed_shell_points(int xc, int precision, int n, const double* rho, const double* gam,
                                       double* out, cudaStream_t st) {
  const int blocks = std::min((n + 255) / 256, 4096);
  closed_shell_points_kernel<<<blocks, 256, 0, st>>>(xc, precision, n, rho, gam, out);
  return cudaGetLastError();
}

int mixed_supported(int mode) { return (mode == kModeRks || mode == kModeUks) ? 1 : 0; }

// Per-CTA slab: 4 FP32 + 4 BF16 planes (24 B / AO / point), the packed A operand (8 B), the GEMM2
// image tiles (12 B).
size_t mixed_slab_doubles(int max_m) {
  const size_t m_pad = (size_t)(max_m + 127) / 128 * 128;
  return m_pad * 128 * (4 * sizeof(float) + 4 * sizeof(__nv_bfloat16) + 4 * sizeof(__nv_bfloat16) +
                        6 * sizeof(__nv_bfloat16)) / sizeof(double);
}

int mixed_ctas_per_sm(int tile_n) { return tile_n == 128 ? MixCfg<128>::kCtas : MixCfg<64>::kCtas; }

int mixed_max_m() { return kMaxMixedM; }

cudaError_t mixed_set_attributes() {
  static bool attr = false;
  if (attr) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(vxc_mixed_kernel<false, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MixCfg<64>::kSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(vxc_mixed_kernel<true, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             MixCfg<64>::kSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(vxc_mixed_kernel<false, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             MixCfg<128>::kSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(vxc_mixed_kernel<true, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             MixCfg<128>::kSmemBytes);
  if (e == cudaSuccess) attr = true;
  return e;
}

// n_ctas: the CTAs to launch (the caller sizes them by mixed_ctas_per_sm(A.tile_n)).
cudaError_t launch_mixed(const DevGrid& G, const EvalArgs& A, int n_ctas, cudaStream_t st) {
  if (A.max_m > kMaxMixedM) return cudaErrorInvalidValue;
  const cudaError_t e = mixed_set_attributes();
  if (e != cudaSuccess) return e;
  if (A.tile_n == 128) {
    if (A.ao_cache)
      vxc_mixed_kernel<true, 128><<<n_ctas, kMT, MixCfg<128>::kSmemBytes, st>>>(G, A);
    else
      vxc_mixed_kernel<false, 128><<<n_ctas, kMT, MixCfg<128>::kSmemBytes, st>>>(G, A);
  } else {
    if (A.ao_cache)
      vxc_mixed_kernel<true, 64><<<n_ctas, kMT, MixCfg<64>::kSmemBytes, st>>>(G, A);
    else
      vxc_mixed_kernel<false, 64><<<n_ctas, kMT, MixCfg<64>::kSmemBytes, st>>>(G, A);
  }
  return cudaGetLastError();
}

cudaError_t launch_mixed_prepare(const double* P, int n_total, const int* mol_n, const long long* mol_off,
                                 const int* mol_ao_off, int n_mols, void* out, int* fexp, cudaStream_t st) {
  split_density_kernel<<<n_total, 256, 0, st>>>(P, n_total, mol_n, mol_off, mol_ao_off, n_mols,
                                                reinterpret_cast<uint2*>(out), fexp);
  return cudaGetLastError();
}

}  // namespace cxc
