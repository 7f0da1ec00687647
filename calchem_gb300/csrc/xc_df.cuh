// xc_df.cuh -- the closed-shell point functionals in double-float arithmetic (FP32 pipe).
//
// GB300 runs FP64 at about 1/64 of its FP32 rate, and a B3LYP point in FP64 costs ~1000 FP64
// instructions (cube roots, logarithms, an arctangent, an exponential and a dozen divisions), so
// in the tensor-core quadrature the functional was the one phase bound by the FP64 pipe.  Here
// the same formulas as xc_eval_cs (xc_device.cuh; CalChem's eval_xc_spin at rho_a = rho_b,
// crates/calchem-dft/src/xc.rs:159-555) run on double-floats (~48 significant bits).  The
// elementary functions are the FP32 library value refined by one Newton step evaluated in
// double-float (cube root, logarithm), Tang's table-driven exponential (df_exp_neg), and a
// table-plus-series arctangent; each is accurate to ~1e-13 relative or better, so the energy
// density and its partials agree with the FP64 form to ~1e-12 relative.
//
// Range: FP32 carries the double-floats, so the caller keeps the FP64 form for rho < kDfRhoMin
// (1e-12 total density), where rho^(8/3) (B88, PBE) would leave the FP32 range.  Above it every
// intermediate stays inside [1e-37, 1e38] for densities up to 1e6 and any gradient that does not
// overflow FP32 (a lo part may be subnormal near the lower end, ~40 bits left).  The LYP terms in
// omega = exp(-C rho^(-1/3)) rho^(-11/3) / (1 + D rho^(-1/3)) are dropped where C rho^(-1/3) > 80
// (rho < 3.2e-8): there they are below 1e-30 of the t0 term, and rho^3 would leave the FP32 range.
#pragma once

#include <cuda_runtime.h>

#include "dfloat.cuh"
#include "xc_device.cuh"

namespace cxc {

constexpr double kDfRhoMin = 1e-12;  // total density below which the FP64 form is used

// A double constant as a double-float (folded at compile time).
__host__ __device__ constexpr df32 dfc(double c) { return df32{(float)c, (float)(c - (double)(float)c)}; }

namespace dfo {
__device__ __forceinline__ df32 operator+(df32 a, df32 b) { return df_add(a, b); }
__device__ __forceinline__ df32 operator-(df32 a, df32 b) { return df_sub(a, b); }
__device__ __forceinline__ df32 operator-(df32 a) { return df_neg(a); }
__device__ __forceinline__ df32 operator*(df32 a, df32 b) { return df_mul(a, b); }
__device__ __forceinline__ df32 operator/(df32 a, df32 b) { return df_div(a, b); }
// with a float that is exact (small integers, halves): no rounding of the constant
__device__ __forceinline__ df32 operator+(df32 a, float b) { return df_add_f(a, b); }
__device__ __forceinline__ df32 operator+(float b, df32 a) { return df_add_f(a, b); }
__device__ __forceinline__ df32 operator-(df32 a, float b) { return df_add_f(a, -b); }
__device__ __forceinline__ df32 operator-(float b, df32 a) { return df_add_f(df_neg(a), b); }
__device__ __forceinline__ df32 operator*(df32 a, float b) { return df_mul_f(a, b); }
__device__ __forceinline__ df32 operator*(float b, df32 a) { return df_mul_f(a, b); }
__device__ __forceinline__ df32& operator+=(df32& a, df32 b) { a = df_add(a, b); return a; }
}  // namespace dfo

// cube root of x > 0: y = cbrtf(x) (1 ulp) and one Newton step y - (y^3 - x) / (3 y^2), the
// residual formed exactly enough (y^2 by TwoProd) that the step leaves ~eps^2 relative error.
__device__ __forceinline__ df32 df_cbrt(df32 x) {
  const float y = cbrtf(x.hi);
  const df32 y2 = two_prod(y, y);
  const df32 res = df_sub(df_mul_f(y2, y), x);
  return fast_two_sum(y, -__fdividef(res.hi, __fmul_rn(3.f, y2.hi)));
}

// exp(x) for x < 88 (tab: the 2^(-j/64) table of df_exp_neg)
__device__ __forceinline__ df32 df_exp(df32 x, const df32* tab) { return df_exp_neg(df_neg(x), tab); }

// log(x) for 1e-37 < x < 1e38: y = logf(x) and one Newton step on exp, y + log1p(d) with
// d = x exp(-y) - 1 (|d| ~ 1e-7, so log1p(d) = d - d^2 / 2 to 1e-21).
__device__ __forceinline__ df32 df_log(df32 x, const df32* tab) {
  const float y = logf(x.hi);
  const df32 d = df_add_f(df_mul(x, df_exp_neg(df32{y, 0.f}, tab)), -1.f);
  return df_add(df32{y, 0.f}, df_add_f(d, -0.5f * d.hi * d.hi));
}

// log(1 + u) for u >= 0: below 2^-10 the series u - u^2/2 + u^3 (1/3 - u/4 + u^2/5 - u^3/6) (the
// u^2 term in double-float, the tail in FP32, truncation < u^7/7); above, the Newton step of
// df_log on 1 + u formed in double-float.
__device__ __forceinline__ df32 df_log1p(df32 u, const df32* tab) {
  if (u.hi < 0.0009765625f) {
    const float uf = u.hi;
    const float tail = uf * uf * uf * (0.33333334f - uf * (0.25f - uf * (0.2f - uf * 0.16666667f)));
    return df_add_f(df_add(u, df_mul_f(df_mul(u, u), -0.5f)), tail);
  }
  const df32 x = df_add_f(u, 1.f);
  const float y = log1pf(u.hi);
  const df32 d = df_add_f(df_mul(x, df_exp_neg(df32{y, 0.f}, tab)), -1.f);
  return df_add(df32{y, 0.f}, df_add_f(d, -0.5f * d.hi * d.hi));
}

// exp(w) - 1 for w >= 0 (w < 88): the series w + w^2/2 + w^3/6 + w^4/24 + w^5/120 below 2^-10,
// else exp(w) - 1 (relative error ~1e-13 / (1 - exp(-w)) < 1e-10 at w = 2^-10).
__device__ __forceinline__ df32 df_expm1(df32 w, const df32* tab) {
  if (w.hi < 0.0009765625f) {
    const float wf = w.hi;
    const float tail = wf * wf * wf * (0.16666667f + wf * (0.041666668f + wf * 0.008333334f));
    return df_add_f(df_add(w, df_mul_f(df_mul(w, w), 0.5f)), tail);
  }
  return df_add_f(df_exp(w, tab), -1.f);
}

// atan(t) for t >= 0: t > 1 by atan(t) = pi/2 - atan(1/t); then t = c + (the rest) with c = j/8,
// atan(t) = atan(c) + atan(d), d = (t - c) / (1 + t c), |d| <= 1/16, and
// atan(d) = d (1 - z/3 + z^2/5 - z^3 (1/7 - z/9 + z^2/11)), z = d^2 <= 2^-8 (truncation
// < z^6/13 ~ 3e-16; the z^3 tail in FP32).  atan(j/8), j = 0..8, are double constants.
__device__ __forceinline__ df32 df_atan(df32 t) {
  using namespace dfo;
  const bool inv = t.hi > 1.f;
  if (inv) t = df_div(df32{1.f, 0.f}, t);
  const int j = (int)rintf(t.hi * 8.f);
  const float c = (float)j * 0.125f;
  const df32 d = df_div(df_add_f(t, -c), df_add_f(df_mul_f(t, c), 1.f));
  const df32 z = d * d;
  const float zf = z.hi;
  const float tail = zf * zf * zf * (0.14285715f - zf * (0.11111111f - zf * 0.09090909f));
  const df32 p = df_add_f(1.f - z * dfc(1.0 / 3.0) + (z * z) * dfc(0.2), -tail);
  df32 base = df32{0.f, 0.f};
  switch (j) {  // atan(j / 8)
    case 1: base = dfc(0.12435499454676144); break;
    case 2: base = dfc(0.24497866312686414); break;
    case 3: base = dfc(0.35877067027057225); break;
    case 4: base = dfc(0.4636476090008061); break;
    case 5: base = dfc(0.5585993153435624); break;
    case 6: base = dfc(0.6435011087932844); break;
    case 7: base = dfc(0.7188299996216245); break;
    case 8: base = dfc(0.7853981633974483); break;
    default: break;
  }
  const df32 a = base + d * p;
  return inv ? dfc(1.5707963267948966) - a : a;
}

// VWN channel constants as double-floats
struct VwnDf { df32 a, x0, b, c, q, c1, c2, c3, bx0; };
__host__ __device__ constexpr VwnDf vwn_df(VwnPara p) {
  return VwnDf{dfc(p.a), dfc(p.x0), dfc(p.b), dfc(p.c), dfc(p.q), dfc(p.c1), dfc(p.c2), dfc(p.c3), dfc(p.b * p.x0)};
}

struct XcCsDf {
  df32 f, vr, vg;  // as XcCs: energy density, dF/drho_a, dF/dgamma_aa + dF/dgamma_ab / 2
};

// PW92 paramagnetic correlation per particle and its rs derivative (pw92 in xc_device.cuh).
__device__ __forceinline__ void pw92_df(df32 rs, const df32* tab, df32& g, df32& dg) {
  using namespace dfo;
  constexpr Pw92Channel c{0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294};
  const df32 x = df_sqrt(rs), x3 = rs * x, x4 = rs * rs;
  const df32 q0 = dfc(-2.0 * c.a) * (1.f + dfc(c.a1) * rs);
  const df32 q1 = dfc(2.0 * c.a) * (dfc(c.b1) * x + dfc(c.b2) * rs + dfc(c.b3) * x3 + dfc(c.b4) * x4);
  const df32 dq1 = dfc(c.a) * (dfc(c.b1) / x + dfc(2.0 * c.b2) + dfc(3.0 * c.b3) * x + dfc(4.0 * c.b4) * rs);
  const df32 ln = df_log1p(df32{1.f, 0.f} / q1, tab);
  g = q0 * ln;
  dg = dfc(-2.0 * c.a * c.a1) * ln - q0 * dq1 / (q1 * (q1 + 1.f));
}

// xc_eval_cs for codes 0-5 (SVWN5, BLYP, PBE, B3LYP, B3LYP5, PBE0) at spin density r and
// gamma_ss g, for r + r >= kDfRhoMin: part 0 the exchange terms (Slater, B88, PBE exchange) and VWN,
// part 1 the other correlation terms (LYP, PBE correlation), which balances the two parts' work for
// B3LYP; the functional is their sum.  tab: the
// 2^(-j/64) table of df_exp_neg.
__device__ __forceinline__ XcCsDf xc_eval_cs_df(int code, df32 r, df32 g, const df32* tab, int part) {
  using namespace dfo;
  XcCsDf o{df32{0.f, 0.f}, df32{0.f, 0.f}, df32{0.f, 0.f}};
  if (g.hi < 0.f) g = df32{0.f, 0.f};
  const df32 rho = r * 2.f;
  const df32 c13 = df_cbrt(r);
  const df32 rho13 = dfc(kCsCbrt2) * c13;
  const bool xpart = part == 0, cpart = !xpart;
  if (xpart && (code == 0 || code == 1 || code == 3 || code == 4)) {  // Slater
    const df32 sc = (code == 3 || code == 4) ? dfc(0.80) : df32{1.f, 0.f};
    o.f += sc * (dfc(-2.0 * kCsCx) * r * c13);
    o.vr += sc * (dfc(-(4.0 / 3.0) * kCsCx) * c13);
  }
  if (xpart && (code == 1 || code == 3 || code == 4)) {  // B88
    const df32 sc = code == 1 ? df32{1.f, 0.f} : dfc(0.72);
    const df32 beta = dfc(0.0042);
    const df32 r43 = r * c13;
    const df32 s2 = g / (r43 * r43);
    const df32 s = df_sqrt(s2);
    const df32 q1 = df_sqrt(s2 + 1.f);
    const df32 ash = df_log1p(s + s2 / (q1 + 1.f), tab);
    const df32 bsa = dfc(6.0 * 0.0042) * s * ash;
    const df32 den = bsa + 1.f;
    const df32 gfun = -(beta * s2) / den;
    const df32 h = -(beta * (bsa + 2.f - dfc(6.0 * 0.0042) * s2 / q1)) / (den * den);
    o.f += sc * (2.f * r43 * gfun);
    o.vr += sc * (dfc(4.0 / 3.0) * c13 * (gfun - s2 * h));
    o.vg += sc * (0.5f * h / r43);
  }
  if (xpart && (code == 2 || code == 5)) {  // PBE exchange (spin scaling: rho_u = rho, gamma_u = 4g)
    const float sc = code == 2 ? 1.f : 0.75f;
    const df32 r43 = rho * rho13;
    const df32 exl = dfc(kCsCxu) * r43;
    const df32 kf = dfc(kCsCbrt3Pi2) * rho13;
    const df32 den_s2 = 4.f * (kf * kf) * (rho * rho);
    const df32 s2 = 4.f * g / den_s2;
    const df32 q = 1.f + dfc(kMu / kKappa) * s2;
    const df32 fx = dfc(1.0 + kKappa) - dfc(kKappa) / q;
    const df32 dfx = dfc(kMu) / (q * q);
    o.f += sc * (exl * fx);
    o.vr += sc * (dfc((4.0 / 3.0) * kCsCxu) * rho13 * fx + exl * dfx * (dfc(-(8.0 / 3.0)) * s2 / rho));
    o.vg += sc * (2.f * (exl * dfx / den_s2));
  }
  if (xpart && (code == 0 || code == 3 || code == 4)) {  // VWN5 / VWN_RPA, paramagnetic channel (part 0)
    const df32 sc = code == 0 ? df32{1.f, 0.f} : dfc(0.19);
    const VwnDf ch = code == 3 ? vwn_df(kVwnRpaPara) : vwn_df(kVwn5Para);
    const df32 x = df_sqrt(dfc(kCsRsK) / rho13);
    const df32 X = x * x + ch.b * x + ch.c;
    const df32 at = df_atan(ch.q / (2.f * x + ch.b));
    const df32 dx0 = x - ch.x0;
    const df32 ep = ch.a * (df_log(x * x / X, tab) + ch.c1 * at - ch.c2 * (df_log(dx0 * dx0 / X, tab) + ch.c3 * at));
    const df32 dp = ch.a * (ch.c * dx0 - ch.bx0 * x) / (dx0 * X);
    o.f += sc * (rho * ep);
    o.vr += sc * (ep - dfc(1.0 / 3.0) * dp);
  }
  if (cpart && (code == 1 || code == 3 || code == 4)) {  // LYP
    const df32 sc = code == 1 ? df32{1.f, 0.f} : dfc(0.81);
    constexpr double A = 0.04918, B = 0.132, C = 0.2533, D = 0.349;
    const df32 rm13 = df32{1.f, 0.f} / rho13;
    const df32 den = 1.f + dfc(D) * rm13;
    const df32 g0 = dfc(-4.0 * A) / (rho * den);
    const df32 dg0 = -g0 * (1.f + dfc((2.0 / 3.0) * D) * rm13) / (rho * den);
    const df32 r2 = r * r;
    const df32 t0 = g0 * r2;
    const df32 dt0 = dg0 * r2 + g0 * r;
    const df32 crm = dfc(C) * rm13;
    if (crm.hi > 80.f) {  // the FP64 form drops them above 500
      o.f += sc * t0;
      o.vr += sc * dt0;
    } else {
      const df32 rho2 = rho * rho;
      const df32 omega = df_exp_neg(crm, tab) / den * (rm13 * rm13 / (rho2 * rho));
      const df32 delta = crm + dfc(D) * rm13 / den;
      const df32 domega = omega * (delta - 11.f) / (3.f * rho);
      const df32 ddelta = dfc(-(1.0 / 3.0)) * (rm13 / rho) * (dfc(C) + dfc(D) / (den * den));
      const df32 r83 = r2 * c13 * c13;
      const df32 stf = dfc(kCsK0) * r2 * (r83 * 2.f);
      const df32 dstf = dfc(kCsK0) * (dfc(11.0 / 3.0) * r83 * r + r * r83);
      const df32 c47 = 47.f - 7.f * delta;
      const df32 cg = r2 * c47 * dfc(1.0 / 18.0) - dfc(2.0 / 3.0) * rho2;
      const df32 dcg = r * c47 * dfc(1.0 / 18.0) + r2 * (ddelta * dfc(-7.0 / 18.0)) - dfc(4.0 / 3.0) * rho;
      const df32 c25 = 2.5f - delta * dfc(1.0 / 18.0), c11 = (delta - 11.f) * dfc(1.0 / 9.0);
      const df32 r3 = r2 * r;
      const df32 qa = r3 / rho;
      const df32 dqa = (2.f * r2 * rho - r3) / rho2;
      const df32 dqb = (r2 * rho - r3) / rho2;
      const df32 ea = -(r2 * c25) - c11 * qa + (dfc(2.0 / 3.0) * rho2 - r2);
      const df32 common = -(r * c25) + r2 * (ddelta * dfc(1.0 / 18.0)) - (ddelta * dfc(1.0 / 9.0)) * qa;
      const df32 dea = common - c11 * dqa + dfc(4.0 / 3.0) * rho;
      const df32 deb = common - c11 * dqb + dfc(4.0 / 3.0) * rho - 2.f * r;
      const df32 aaa = cg + ea, aab = 2.f * cg;
      const df32 sb = stf + (aaa + aab + aaa) * g;
      const df32 ds = dstf + ((dcg + dea) + 2.f * dcg + (dcg + deb)) * g;
      const df32 ab = dfc(A * B);
      o.f += sc * (t0 - ab * omega * sb);
      o.vr += sc * (dt0 - ab * (domega * sb + omega * ds));
      o.vg += sc * (-(ab * omega * (aaa + 0.5f * aab)));
    }
  }
  if (cpart && (code == 2 || code == 5)) {  // PBE correlation on the paramagnetic PW92 channel
    const df32 gt = 4.f * g;
    const df32 rs = dfc(kCsRsK) / rho13;
    const df32 drs = -rs / (3.f * rho);
    df32 ec, de0;
    pw92_df(rs, tab, ec, de0);
    const df32 dec_drho = de0 * drs;
    if (gt.hi < 1e-36f) {
      o.f += rho * ec;
      o.vr += ec + rho * dec_drho;
    } else {
      const df32 b0 = dfc(kBetaPbe / kGammaPbe);
      const df32 gp3 = dfc(kGammaPbe);
      const df32 den_t2 = dfc(kCsCt) * (rho * rho * rho13);
      const df32 t2 = gt / den_t2;
      const df32 w = -ec / gp3;
      df32 af = {0.f, 0.f}, daw = {0.f, 0.f};
      if (!(w.hi > 100.f)) {
        const df32 em1 = df_expm1(w, tab);
        af = b0 / em1;
        daw = -(af * (em1 + 1.f) / em1);
      }
      const df32 u = af * t2;
      const df32 dpol = 1.f + u + u * u;
      const df32 dpol2 = dpol * dpol;
      const df32 za = 1.f + b0 * t2 * ((1.f + u) / dpol);
      const df32 lnz = df_log(za, tab);
      const df32 h = gp3 * lnz;
      const df32 dh_dt2 = gp3 * (b0 * (1.f + 2.f * u) / dpol2) / za;
      const df32 dh_dw = gp3 * ((-(b0 * t2 * t2 * u * (2.f + u)) / dpol2) * daw) / za;
      const df32 dh_drho = dh_dt2 * (dfc(-(7.0 / 3.0)) * t2 / rho) + dh_dw * (-dec_drho / gp3);
      const df32 te = ec + h;
      o.f += rho * te;
      o.vr += te + rho * (dec_drho + dh_drho);
      o.vg += 2.f * (rho * dh_dt2 / den_t2);
    }
  }
  return o;
}

// One part (0 exchange, 1 correlation) of the closed-shell functional for the tensor-core kernels:
// the double-float form for codes 0-5 at total density >= kDfRhoMin; otherwise part 0 is all of
// xc_eval_cs (FP64) and part 1 zero.  Results as doubles.
__device__ __forceinline__ XcCs xc_eval_cs_fast_part(int code, double r, double g, const df32* tab, int part) {
  if (code <= 5 && !(r + r < kDfRhoMin)) {
    const XcCsDf d = xc_eval_cs_df(code, df_from_double(r), df_from_double(fmax(g, 0.0)), tab, part);
    return XcCs{df_to_double(d.f), df_to_double(d.vr), df_to_double(d.vg)};
  }
  if (part != 0) return XcCs{0.0, 0.0, 0.0};
  return xc_eval_cs(code, r, g);
}

// The two parts summed in FP64 (part 0 + part 1), as the Vxc kernel sums them across its halves.
__device__ __forceinline__ XcCs xc_eval_cs_fast(int code, double r, double g, const df32* tab) {
  const XcCs x = xc_eval_cs_fast_part(code, r, g, tab, 0);
  const XcCs c = xc_eval_cs_fast_part(code, r, g, tab, 1);
  return XcCs{x.f + c.f, x.vr + c.vr, x.vg + c.vg};
}

}  // namespace cxc
