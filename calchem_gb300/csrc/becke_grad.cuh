// becke_grad.cuh -- derivative of the Becke partition weight of one grid point with respect to the
// nuclei (grid.rs:423-584), one warp per point; shared by the FP64 and tensor-core gradient kernels.
#pragma once

#include <cuda_runtime.h>

#include "dfloat.cuh"

namespace cxc {
namespace becke {

// Becke step s(nu) and ds/dnu (grid.rs:129-140).
__device__ __forceinline__ void step_d(double nu, double& s, double& ds) {
  const double x = nu < -1.0 ? -1.0 : (nu > 1.0 ? 1.0 : nu);
  const double f1 = 1.5 * x - 0.5 * x * x * x, d1 = 1.5 - 1.5 * x * x;
  const double f2 = 1.5 * f1 - 0.5 * f1 * f1 * f1, d2 = 1.5 - 1.5 * f1 * f1;
  const double f3 = 1.5 * f2 - 0.5 * f2 * f2 * f2, d3 = 1.5 - 1.5 * f2 * f2;
  s = 0.5 * (1.0 - f3);
  ds = -0.5 * d3 * d2 * d1;
}

__device__ __forceinline__ double clamp_unit(double v) { return v < -1.0 ? -1.0 : (v > 1.0 ? 1.0 : v); }

__host__ __device__ __forceinline__ size_t becke_scratch_doubles(int n) { return 5 * (size_t)n + 3 * (size_t)n * n; }

// Per-point pair tables of one warp (n x n, row-major), behind dist[n], cell[n] and wacc[3 n].
struct BeckeScratch {
  double* dist;  // |r - R_c|
  double* cell;  // P_c = prod_{d != c} s_cd
  double* wacc;  // [3 n] the warp's weight-derivative sums
  double* s;     // s_cd (s_dc = 1 - s_cd, both stored; 1 for coincident atoms)
  double* e;     // prod_{d != c, k} s_cd at [c][k]
  double* l;     // ds_cd/dmu_cd (the same for both orientations)
};

// (E) raw_w f dW/dR for one point, one warp; wacc[3a + q] is owned by lane a % 32.
//   1. lanes over the unordered pairs (c < d): s_cd from mu_cd = (r_c - r_d) / R_cd and the size
//      adjustment, and its slope (grid.rs:447-476);
//   2. lanes over atoms c: the cell function P_c (factors multiplied in increasing d, as the
//      reference accumulates them) and every "product but one" prod_{d != c, k} s_cd as a prefix
//      times a suffix product -- the reference's cell[c] / s_ck, or the explicit product when
//      s_ck <= 1e-12 (grid.rs:500-515), without a division;
//   3. lanes over atoms a != host: d(P_host / Z)/dR_a from the pairs (a, b) (grid.rs:517-583);
//      the host atom gets minus their sum.
static __device__ void becke_point(int n, const double* __restrict__ xyz, const double* __restrict__ inv_r,
                            const double* __restrict__ a_ij, const int2* __restrict__ pairs, int n_pairs, int host,
                            double x, double y, double z, double pref_in, const BeckeScratch& W) {
  const int lane = threadIdx.x & 31;
  for (int c = lane; c < n; c += 32) {
    const double dx = x - xyz[3 * c], dy = y - xyz[3 * c + 1], dz = z - xyz[3 * c + 2];
    W.dist[c] = sqrt(dx * dx + dy * dy + dz * dz);
  }
  __syncwarp();
  for (int p = lane; p < n_pairs; p += 32) {
    const int c = pairs[p].x, d = pairs[p].y;
    const size_t cd = (size_t)c * n + d, dc = (size_t)d * n + c;
    const double inv = inv_r[cd];
    double sv = 1.0, sl = 0.0;
    if (inv != 0.0) {
      const double mu = clamp_unit((W.dist[c] - W.dist[d]) * inv);
      const double a = a_ij[cd];
      double dsdnu;
      step_d(mu + a * (1.0 - mu * mu), sv, dsdnu);
      sl = dsdnu * (1.0 - 2.0 * a * mu);
    }
    W.s[cd] = sv;
    W.s[dc] = inv != 0.0 ? 1.0 - sv : 1.0;
    W.l[cd] = sl;
    W.l[dc] = sl;
  }
  __syncwarp();
  double zl = 0.0;
  for (int c = lane; c < n; c += 32) {
    const double* __restrict__ sr = W.s + (size_t)c * n;
    double* __restrict__ er = W.e + (size_t)c * n;
    double pre = 1.0;
    for (int k = 0; k < n; ++k) {
      er[k] = pre;
      if (k != c) pre *= sr[k];
    }
    W.cell[c] = pre;
    zl += pre;
    double suf = 1.0;
    for (int k = n - 1; k >= 0; --k) {
      er[k] *= suf;
      if (k != c) suf *= sr[k];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) zl += __shfl_xor_sync(0xffffffffu, zl, o);
  __syncwarp();
  const double zs = zl;
  if (zs <= 1e-30) return;
  const double wn = W.cell[host] / zs, pref = pref_in / zs;
  double h0 = 0, h1 = 0, h2 = 0;
  for (int a = lane; a < n; a += 32) {
    if (a == host) continue;
    const double ra = W.dist[a];
    if (ra < 1e-14) continue;
    const double ax = xyz[3 * a], ay = xyz[3 * a + 1], az = xyz[3 * a + 2];
    const double ir = 1.0 / ra;
    const double dr0 = -(x - ax) * ir, dr1 = -(y - ay) * ir, dr2 = -(z - az) * ir;
    double ph0 = 0, ph1 = 0, ph2 = 0, zz0 = 0, zz1 = 0, zz2 = 0;
    const size_t row = (size_t)a * n;
    for (int b = 0; b < n; ++b) {
      if (b == a) continue;
      const double inv = inv_r[row + b];
      const double slope = W.l[row + b];
      if (inv == 0.0 || fabs(slope) < 1e-30) continue;
      const double mu = clamp_unit((ra - W.dist[b]) * inv);
      const double v0 = ax - xyz[3 * b], v1 = ay - xyz[3 * b + 1], v2 = az - xyz[3 * b + 2];
      const double pa = W.e[row + b], pb = W.e[(size_t)b * n + a];
      const double k = slope * inv;
      const double ds0 = k * (dr0 - mu * v0 * inv), ds1 = k * (dr1 - mu * v1 * inv), ds2 = k * (dr2 - mu * v2 * inv);
      zz0 += pa * ds0 - pb * ds0;
      zz1 += pa * ds1 - pb * ds1;
      zz2 += pa * ds2 - pb * ds2;
      if (b == host) {
        ph0 -= pb * ds0;
        ph1 -= pb * ds1;
        ph2 -= pb * ds2;
      }
    }
    const double w0 = pref * (ph0 - wn * zz0), w1 = pref * (ph1 - wn * zz1), w2 = pref * (ph2 - wn * zz2);
    W.wacc[3 * a] += w0;
    W.wacc[3 * a + 1] += w1;
    W.wacc[3 * a + 2] += w2;
    h0 -= w0;
    h1 -= w1;
    h2 -= w2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    h0 += __shfl_xor_sync(0xffffffffu, h0, o);
    h1 += __shfl_xor_sync(0xffffffffu, h1, o);
    h2 += __shfl_xor_sync(0xffffffffu, h2, o);
  }
  __syncwarp();
  if (lane == 0) {
    W.wacc[3 * host] += h0;
    W.wacc[3 * host + 1] += h1;
    W.wacc[3 * host + 2] += h2;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------------------------
// Double-float form of becke_point for the tensor-core gradient: the same quantity to ~1e-14
// relative on the FP32 pipe.
//
// The step polynomial p(y) = (3 y - y^3) / 2 is iterated through t = 1 - |y|, which obeys
// t' = t^2 (3 - t) / 2 exactly (1 - p(y) = (1 - y)^2 (2 + y) / 2 and p is odd), so s and 1 - s keep
// their relative precision when one of them is tiny, and p'(y) = 3 t (2 - t) / 2.  1 - nu and
// 1 + nu come from (1 - mu)(1 - a (1 + mu)) and (1 + mu)(1 + a (1 - mu)).  Pairs whose terms are
// below 1e-20 (|E_ab - E_ba| |slope| / R_ab, and E_ba |slope| / R_ab for b = host) are skipped: their
// sum over a whole grid stays below 1e-16 Eh/Bohr.

__device__ __forceinline__ df32 df_clamp_unit(df32 v) {
  if (v.hi >= 1.f) return df32{1.f, 0.f};
  if (v.hi <= -1.f) return df32{-1.f, 0.f};
  return v;
}

// s_{lo hi}, 1 - s_{lo hi} and ds/dmu for mu = mu_{lo hi}, a = a_{lo hi}.
__device__ __forceinline__ void step_df(df32 mu, df32 a, df32& s, df32& sc, df32& slope) {
  const df32 one = {1.f, 0.f};
  const df32 om = df_sub(one, mu), op = df_add(one, mu);
  const df32 um = df_mul(om, df_sub(one, df_mul(a, op)));  // 1 - nu
  const df32 vp = df_mul(op, df_add(one, df_mul(a, om)));  // 1 + nu
  const bool upper = um.hi <= vp.hi;                        // nu >= 0
  df32 t = upper ? um : vp;
  df32 d = one;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const df32 dk = df_mul_f(df_mul(t, df_sub(df32{2.f, 0.f}, t)), 1.5f);
    t = df_mul_f(df_mul(df_mul(t, t), df_sub(df32{3.f, 0.f}, t)), 0.5f);
    d = df_mul(d, dk);
  }
  const df32 half_t = df_mul_f(t, 0.5f);
  const df32 rest = df_sub(one, half_t);
  s = upper ? half_t : rest;
  sc = upper ? rest : half_t;
  // ds/dnu = -p'(f2) p'(f1) p'(nu) / 2, dnu/dmu = 1 - 2 a mu
  slope = df_mul(df_mul_f(d, -0.5f), df_sub(one, df_mul_f(df_mul(a, mu), 2.f)));
}

// Per-warp tables of becke_point_df: dist[n] (double-float), cell[n] (double), wacc[3 n] (double),
// then the pair tables s, e, l as double-floats (n x n each); the same size as BeckeScratch.
struct BeckeScratchDf {
  df32* dist;
  double* cell;
  double* wacc;
  df32* s;
  df32* e;
  df32* l;
};

// pdf: per ordered atom pair (a, b), 5 double-floats: 1 / R_ab (0 for a == b or coincident atoms),
// the size adjustment a_ab, and (R_a - R_b) / R_ab.  Only the O(n) per-point work is FP64.
static __device__ void becke_point_df(int n, const double* __restrict__ xyz, const df32* __restrict__ pdf,
                                      const int2* __restrict__ pairs, int n_pairs, int host, double x, double y,
                                      double z, double pref_in, const BeckeScratchDf& W) {
  const int lane = threadIdx.x & 31;
  for (int c = lane; c < n; c += 32) {
    const double dx = x - xyz[3 * c], dy = y - xyz[3 * c + 1], dz = z - xyz[3 * c + 2];
    W.dist[c] = df_from_double(sqrt(dx * dx + dy * dy + dz * dz));
  }
  __syncwarp();
  for (int p = lane; p < n_pairs; p += 32) {
    const int c = pairs[p].x, d = pairs[p].y;
    const size_t cd = (size_t)c * n + d, dc = (size_t)d * n + c;
    const df32 inv = pdf[5 * cd];
    df32 sv = {1.f, 0.f}, sc = {1.f, 0.f}, sl = {0.f, 0.f};
    if (inv.hi != 0.f) {
      const df32 mu = df_clamp_unit(df_mul(df_sub(W.dist[c], W.dist[d]), inv));
      step_df(mu, pdf[5 * cd + 1], sv, sc, sl);
    }
    W.s[cd] = sv;
    W.s[dc] = sc;
    W.l[cd] = sl;
    W.l[dc] = sl;
  }
  __syncwarp();
  double zl = 0.0;
  for (int c = lane; c < n; c += 32) {
    const df32* __restrict__ sr = W.s + (size_t)c * n;
    df32* __restrict__ er = W.e + (size_t)c * n;
    df32 pre = {1.f, 0.f};
    for (int k = 0; k < n; ++k) {
      er[k] = pre;
      if (k != c) pre = df_mul(pre, sr[k]);
    }
    const double cv = df_to_double(pre);
    W.cell[c] = cv;
    zl += cv;
    df32 suf = {1.f, 0.f};
    for (int k = n - 1; k >= 0; --k) {
      er[k] = df_mul(er[k], suf);
      if (k != c) suf = df_mul(suf, sr[k]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) zl += __shfl_xor_sync(0xffffffffu, zl, o);
  __syncwarp();
  const double zs = zl;
  if (zs <= 1e-30) return;
  const double wn = W.cell[host] / zs, pref = pref_in / zs;
  double h0 = 0, h1 = 0, h2 = 0;
  for (int a = lane; a < n; a += 32) {
    if (a == host) continue;
    const df32 dra = W.dist[a];
    const double ra = df_to_double(dra);
    if (ra < 1e-14) continue;
    const double ir = 1.0 / ra;
    const df32 dr0 = df_from_double(-(x - xyz[3 * a]) * ir), dr1 = df_from_double(-(y - xyz[3 * a + 1]) * ir),
               dr2 = df_from_double(-(z - xyz[3 * a + 2]) * ir);
    df32 ph0 = {0.f, 0.f}, ph1 = ph0, ph2 = ph0, zz0 = ph0, zz1 = ph0, zz2 = ph0;
    const size_t row = (size_t)a * n;
    for (int b = 0; b < n; ++b) {
      const df32* t = pdf + 5 * (row + b);
      const df32 inv = t[0];
      if (b == a || inv.hi == 0.f) continue;
      const df32 sl = W.l[row + b];
      const df32 ea = W.e[row + b], eb = W.e[(size_t)b * n + a];
      const df32 diff = df_sub(ea, eb);
      const float scl = fabsf(sl.hi) * inv.hi;
      if (fabsf(diff.hi) * scl < 1e-20f && (b != host || fabsf(eb.hi) * scl < 1e-20f)) continue;
      const df32 mu = df_clamp_unit(df_mul(df_sub(dra, W.dist[b]), inv));
      const df32 k = df_mul(sl, inv);
      const df32 ds0 = df_mul(k, df_sub(dr0, df_mul(mu, t[2])));
      const df32 ds1 = df_mul(k, df_sub(dr1, df_mul(mu, t[3])));
      const df32 ds2 = df_mul(k, df_sub(dr2, df_mul(mu, t[4])));
      zz0 = df_add(zz0, df_mul(diff, ds0));
      zz1 = df_add(zz1, df_mul(diff, ds1));
      zz2 = df_add(zz2, df_mul(diff, ds2));
      if (b == host) {
        ph0 = df_sub(ph0, df_mul(eb, ds0));
        ph1 = df_sub(ph1, df_mul(eb, ds1));
        ph2 = df_sub(ph2, df_mul(eb, ds2));
      }
    }
    const double w0 = pref * (df_to_double(ph0) - wn * df_to_double(zz0));
    const double w1 = pref * (df_to_double(ph1) - wn * df_to_double(zz1));
    const double w2 = pref * (df_to_double(ph2) - wn * df_to_double(zz2));
    W.wacc[3 * a] += w0;
    W.wacc[3 * a + 1] += w1;
    W.wacc[3 * a + 2] += w2;
    h0 -= w0;
    h1 -= w1;
    h2 -= w2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    h0 += __shfl_xor_sync(0xffffffffu, h0, o);
    h1 += __shfl_xor_sync(0xffffffffu, h1, o);
    h2 += __shfl_xor_sync(0xffffffffu, h2, o);
  }
  __syncwarp();
  if (lane == 0) {
    W.wacc[3 * host] += h0;
    W.wacc[3 * host + 1] += h1;
    W.wacc[3 * host + 2] += h2;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------------------------
// The same derivative by a team of threads (a warp, or 2-8 warps) per point, with the pair tables in
// shared memory (the operand stage of the tensor-core kernel is idle at that time).  Each team's
// block holds:
//   dist[n] (double-float), cell[n], tmp[3n], wacc[3n], hq[4] (double); pp[n] (double-float);
//   cnt[n] (int); su, scu, lu [n (n - 1) / 2] (double-float): s_cd, 1 - s_cd and ds_cd/dmu_cd, c < d.
// The "product but one" E_ab = prod_{d != a, b} s_ad comes from the row's product of its factors
// above 1e-30 (pp) and the count of the others (cnt): pp / s_ab when none is below, pp when s_ab
// is the only one, and 0 otherwise (then E_ab < 1e-30).  Pairs whose terms are below 1e-18
// (|E_ab - E_ba| |slope| / R_ab, and E_ba |slope| / R_ab for b = host; first tested on FP32 estimates)
// are skipped: with every E, slope and R^-1 of order one at most, the dropped sum over a grid stays
// below ~1e-12 Eh/Bohr.  The pass-2 sums over b are reduced by xor shuffles inside fixed lane groups,
// so results are deterministic.

// dist, cell, tmp[3], wacc[3], ph[4] (n each), hq[4], pp (n); cnt (n ints); su, scu, lu, cres (n(n-1)/2)
__host__ __device__ constexpr size_t becke_cta_bytes(int n) {
  return (8 * (13 * (size_t)n + 4) + 8 * (size_t)n + 4 * (size_t)(n + (n & 1)) + 16 * (size_t)n * (size_t)(n - 1) + 15) /
         16 * 16;
}

struct BeckeCta {
  df32 *dist, *cell, *tmp, *wacc, *ph, *hq;
  df32* pp;
  int* cnt;
  df32 *su, *scu, *lu, *cres;
  __device__ void carve(unsigned char* base, int n) {
    dist = reinterpret_cast<df32*>(base);
    cell = dist + n;
    tmp = cell + n;
    wacc = tmp + 3 * n;
    ph = wacc + 3 * n;  // per atom a: E_{host a} slope / R and mu e of the pair (a, host)
    hq = ph + 4 * n;
    pp = hq + 4;
    cnt = reinterpret_cast<int*>(pp + n);
    su = reinterpret_cast<df32*>(cnt + n + (n & 1));  // 8-byte aligned
    const size_t np = (size_t)n * (n - 1) / 2;
    scu = su + np;
    lu = scu + np;
    cres = lu + np;
  }
};

__device__ __forceinline__ int pair_id(int c, int d, int n) { return c * n - c * (c + 1) / 2 + (d - c - 1); }

// FP32 estimate of |E_ab| (relative error ~1e-6)
__device__ __forceinline__ float est_but_one(const BeckeCta& T, int a, float s_ab) {
  const int c = T.cnt[a];
  if (c == 0) return fabsf(__fdividef(T.pp[a].hi, s_ab));
  if (c == 1 && !(s_ab > 1e-30f)) return fabsf(T.pp[a].hi);
  return 0.f;
}

// E_ab for the row a (see above)
__device__ __forceinline__ df32 prod_but_one(const BeckeCta& T, int a, df32 s_ab) {
  const int c = T.cnt[a];
  if (c == 0) return df_div(T.pp[a], s_ab);
  if (c == 1 && !(s_ab.hi > 1e-30f)) return T.pp[a];
  return df32{0.f, 0.f};
}

// Barrier of a team of nt threads (whole warps): the warp itself, or named barrier 1 + team id.
__device__ __forceinline__ void team_sync(int nt, int team) {
  if (nt == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + team), "r"(nt) : "memory");
  }
}

// Called by every thread of a team (threads tid = 0..nt-1 of the team, team index `team`) for one
// point (uniform arguments within the team).  T.wacc collects the weight-derivative sums of the
// team's points and must be zeroed by the caller.
static __device__ void becke_point_team(int n, const df32* __restrict__ xyz_df, const df32* __restrict__ pdf, int host,
                                        df32 x, df32 y, df32 z, df32 pref_in, const BeckeCta& T, int tid, int nth,
                                        int team) {
  // everything below is double-float arithmetic on the FP32 pipe (GB300's FP64 rate is 1/64 of it)
  for (int c = tid; c < n; c += nth) {
    const df32 dx = df_sub(x, xyz_df[3 * c]), dy = df_sub(y, xyz_df[3 * c + 1]), dz = df_sub(z, xyz_df[3 * c + 2]);
    T.dist[c] = df_sqrt(df_add(df_add(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz)));
  }
  team_sync(nth, team);
  const int np = n * (n - 1) / 2;
  {
    // pair p = pair_id(c, d): rows of n - 1, n - 2, ... entries; walk the rows once per thread
    int c = 0, rem = tid;
    while (c < n - 1 && rem >= n - 1 - c) { rem -= n - 1 - c; ++c; }
    for (int p = tid; p < np; p += nth) {
      const int d = c + 1 + rem;
      const size_t cd = (size_t)c * n + d;
      const df32 inv = pdf[5 * cd];
      df32 sv = {1.f, 0.f}, sc = {1.f, 0.f}, sl = {0.f, 0.f};
      if (inv.hi != 0.f) {
        const df32 mu = df_clamp_unit(df_mul(df_sub(T.dist[c], T.dist[d]), inv));
        step_df(mu, pdf[5 * cd + 1], sv, sc, sl);
      }
      T.su[p] = sv;
      T.scu[p] = sc;
      T.lu[p] = sl;
      rem += nth;  // advance to pair p + nth
      while (c < n - 1 && rem >= n - 1 - c) { rem -= n - 1 - c; ++c; }
    }
  }
  team_sync(nth, team);
  for (int c = tid; c < n; c += nth) {
    df32 pr = {1.f, 0.f};
    int k = 0;
    for (int d = 0; d < n; ++d) {
      if (d == c) continue;
      const df32 f = c < d ? T.su[pair_id(c, d, n)] : T.scu[pair_id(d, c, n)];
      if (f.hi > 1e-30f) pr = df_mul(pr, f);
      else ++k;
    }
    T.pp[c] = pr;
    T.cnt[c] = k;
    T.cell[c] = k == 0 ? pr : df32{0.f, 0.f};
  }
  team_sync(nth, team);
  if (tid == 0) {
    df32 zs = {0.f, 0.f};
    for (int c = 0; c < n; ++c) zs = df_add(zs, T.cell[c]);
    T.hq[3] = zs;
  }
  team_sync(nth, team);
  const df32 zs = T.hq[3];
  if (zs.hi <= 1e-30f) return;  // uniform: every thread read the same value
  const df32 wn = df_div(T.cell[host], zs), pref = df_div(pref_in, zs);
  // dZ/dR_a = sum_b (E_ab - E_ba) k_ab (dr_a - mu_ab e_ab) with k = slope / R_ab.  Each unordered
  // pair (c < d) is evaluated once, lanes over pairs: c_cd = (E_cd - E_dc) k and c_cd mu_cd e_cd
  // go to atom c with a plus sign and to atom d with a minus sign (mu, e and the difference of E
  // change sign with the orientation).  The results overwrite the pair's s, 1 - s and slope slots
  // (only this lane reads them) plus cres; the pair with the host also leaves E_{host a} k and
  // mu e for the host term of atom a.
  for (int k = tid; k < 4 * n; k += nth) T.ph[k] = df32{0.f, 0.f};
  team_sync(nth, team);
  {
    int c = 0, rem = tid;
    while (c < n - 1 && rem >= n - 1 - c) { rem -= n - 1 - c; ++c; }
    for (int p = tid; p < np; p += nth) {
      const int d = c + 1 + rem;
      const df32* t = pdf + 5 * ((size_t)c * n + d);
      const df32 inv = t[0];
      const df32 zero = {0.f, 0.f};
      df32 cc = zero, w0 = zero, w1 = zero, w2 = zero;
      if (inv.hi != 0.f) {
        const df32 sl = T.lu[p], s_cd = T.su[p], s_dc = T.scu[p];
        const float scl = fabsf(sl.hi) * inv.hi;
        const bool host_pair = c == host || d == host;
        // FP32 estimates first: skip when both products but one are below the threshold
        if (!(est_but_one(T, c, s_cd.hi) * scl < 5e-19f && est_but_one(T, d, s_dc.hi) * scl < 5e-19f)) {
          const df32 ec = prod_but_one(T, c, s_cd), ed = prod_but_one(T, d, s_dc);
          const df32 diff = df_sub(ec, ed);
          const bool use_diff = !(fabsf(diff.hi) * scl < 1e-18f);
          const df32 eh = c == host ? ec : ed;  // E_{host a}
          const bool use_host = host_pair && !(fabsf(eh.hi) * scl < 1e-18f);
          if (use_diff || use_host) {
            const df32 mu = df_clamp_unit(df_mul(df_sub(T.dist[c], T.dist[d]), inv));  // mu_cd
            const df32 k = df_mul(sl, inv);
            if (use_diff) {
              cc = df_mul(diff, k);
              const df32 cm = df_mul(cc, mu);
              w0 = df_mul(cm, t[2]);
              w1 = df_mul(cm, t[3]);
              w2 = df_mul(cm, t[4]);
            }
            if (use_host) {
              // atom a = the other one; mu_{a host} e_{a host} = mu_cd e_cd in either orientation
              const int a = c == host ? d : c;
              T.ph[4 * a] = df_mul(eh, k);
              T.ph[4 * a + 1] = df_mul(mu, t[2]);
              T.ph[4 * a + 2] = df_mul(mu, t[3]);
              T.ph[4 * a + 3] = df_mul(mu, t[4]);
            }
          }
        }
      }
      T.su[p] = cc;
      T.scu[p] = w0;
      T.lu[p] = w1;
      T.cres[p] = w2;
      rem += nth;
      while (c < n - 1 && rem >= n - 1 - c) { rem -= n - 1 - c; ++c; }
    }
  }
  team_sync(nth, team);
  for (int a = tid; a < n; a += nth) {
    const df32 zero = {0.f, 0.f};
    df32 tq0 = zero, tq1 = zero, tq2 = zero;
    const df32 dra = T.dist[a];
    if (a != host && dra.hi >= 1e-14f) {
      df32 cs = zero, w0 = zero, w1 = zero, w2 = zero;
      for (int b = 0; b < n; ++b) {
        if (b == a) continue;
        const int p = a < b ? pair_id(a, b, n) : pair_id(b, a, n);
        if (a < b) {
          cs = df_add(cs, T.su[p]);
          w0 = df_add(w0, T.scu[p]);
          w1 = df_add(w1, T.lu[p]);
          w2 = df_add(w2, T.cres[p]);
        } else {
          cs = df_sub(cs, T.su[p]);
          w0 = df_sub(w0, T.scu[p]);
          w1 = df_sub(w1, T.lu[p]);
          w2 = df_sub(w2, T.cres[p]);
        }
      }
      const df32 ir = df_div(df32{1.f, 0.f}, dra);
      const df32 dr0 = df_mul(df_sub(xyz_df[3 * a], x), ir);
      const df32 dr1 = df_mul(df_sub(xyz_df[3 * a + 1], y), ir);
      const df32 dr2 = df_mul(df_sub(xyz_df[3 * a + 2], z), ir);
      const df32 zz0 = df_sub(df_mul(dr0, cs), w0), zz1 = df_sub(df_mul(dr1, cs), w1), zz2 = df_sub(df_mul(dr2, cs), w2);
      // d P_host / dR_a = -E_{host a} k (dr_a - mu e): mu e was stored for the pair's (lower, higher)
      // orientation, and both factors change sign with it, so it is also the (a, host) value
      const df32 kb = T.ph[4 * a];
      const df32 ph0 = df_mul(kb, df_sub(T.ph[4 * a + 1], dr0)), ph1 = df_mul(kb, df_sub(T.ph[4 * a + 2], dr1)),
                 ph2 = df_mul(kb, df_sub(T.ph[4 * a + 3], dr2));
      tq0 = df_mul(pref, df_sub(ph0, df_mul(wn, zz0)));
      tq1 = df_mul(pref, df_sub(ph1, df_mul(wn, zz1)));
      tq2 = df_mul(pref, df_sub(ph2, df_mul(wn, zz2)));
    }
    T.tmp[3 * a] = tq0;
    T.tmp[3 * a + 1] = tq1;
    T.tmp[3 * a + 2] = tq2;
  }
  team_sync(nth, team);
  if (tid < 3) {
    df32 h = {0.f, 0.f};
    for (int a = 0; a < n; ++a)
      if (a != host) h = df_sub(h, T.tmp[3 * a + tid]);
    T.hq[tid] = h;
  }
  team_sync(nth, team);
  for (int k = tid; k < 3 * n; k += nth) T.wacc[k] = df_add(T.wacc[k], (k / 3 == host) ? T.hq[k % 3] : T.tmp[k]);
  team_sync(nth, team);
}

}  // namespace becke
}  // namespace cxc
