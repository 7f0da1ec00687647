// xc_device.cuh -- FP64 spin-polarised point functionals for the device.
//
// Same functional forms and constants as CalChem's eval_xc_spin
// (crates/calchem-dft/src/xc.rs:136-828): Slater exchange, VWN5 / VWN_RPA correlation,
// Becke-88 gradient correction, LYP (Miehlich form), PBE exchange and PBE correlation on PW92,
// and the SVWN5 / BLYP / PBE / B3LYP / B3LYP5 / PBE0 mixtures; the range-separated CAM-B3LYP
// (ITYH-attenuated B88) and wB97X / wB97X-D (attenuated LDA exchange with B97 series) semilocal parts.  Every function returns the
// energy density f (so that Exc = sum_g w_g f) and its partials with respect to
// (rho_a, rho_b, gamma_aa, gamma_ab, gamma_bb).
#pragma once

#include <cuda_runtime.h>

namespace cxc {

struct XcVal {
  double f, vra, vrb, vgaa, vgab, vgbb;
};

__host__ __device__ __forceinline__ XcVal xc_zero() { return XcVal{0, 0, 0, 0, 0, 0}; }

__host__ __device__ __forceinline__ void xc_axpy(XcVal& acc, double s, const XcVal& o) {
  acc.f += s * o.f;
  acc.vra += s * o.vra;
  acc.vrb += s * o.vrb;
  acc.vgaa += s * o.vgaa;
  acc.vgab += s * o.vgab;
  acc.vgbb += s * o.vgbb;
}

constexpr double kPiD = 3.14159265358979323846;
constexpr double kRhoFloor = 1e-18;  // xc.rs:13

// -------------------------------------------------------------------------- Slater (xc.rs:229-251)
__host__ __device__ __forceinline__ void slater_spin(double r, double& f, double& v) {
  if (r < kRhoFloor) { f = 0.0; v = 0.0; return; }
  const double cx = 0.75 * cbrt(6.0 / kPiD);  // 3/4 (6/pi)^(1/3)
  const double r13 = cbrt(r);
  f = -cx * r * r13;
  v = -(4.0 / 3.0) * cx * r13;
}

// -------------------------------------------------------------------------- VWN (xc.rs:270-404)
struct VwnChannel { double a, x0, b, c; };

__host__ __device__ __forceinline__ void vwn_eps(double x, VwnChannel ch, double& eps, double& rs_deps) {
  const double X = x * x + ch.b * x + ch.c;
  const double X0 = ch.x0 * ch.x0 + ch.b * ch.x0 + ch.c;
  const double q = sqrt(4.0 * ch.c - ch.b * ch.b);
  const double at = atan(q / (2.0 * x + ch.b));
  const double dx0 = x - ch.x0;
  eps = ch.a * (log(x * x / X) + (2.0 * ch.b / q) * at -
                (ch.b * ch.x0 / X0) * (log(dx0 * dx0 / X) + (2.0 * (ch.b + 2.0 * ch.x0) / q) * at));
  rs_deps = ch.a * (ch.c * dx0 - ch.b * x * ch.x0) / (dx0 * X);
}

__host__ __device__ __forceinline__ void spin_f(double zeta, double& fz, double& dfz, double& inv_fdd0) {
  const double c2 = cbrt(2.0) - 1.0;
  const double den = 2.0 * c2;
  inv_fdd0 = 1.0 / (4.0 / (9.0 * c2));
  const double zp = fmax(1.0 + zeta, 0.0), zm = fmax(1.0 - zeta, 0.0);
  const double zp13 = cbrt(zp), zm13 = cbrt(zm);
  fz = (zp * zp13 + zm * zm13 - 2.0) / den;
  dfz = (4.0 / (3.0 * den)) * (zp13 - zm13);
}

// rpa = false: VWN5 parameters; rpa = true: VWN_RPA parameters (xc.rs:291-334).
__host__ __device__ __forceinline__ XcVal vwn_corr(double ra, double rb, bool rpa) {
  XcVal o = xc_zero();
  const double rho = ra + rb;
  if (rho < kRhoFloor) return o;
  const VwnChannel para = rpa ? VwnChannel{0.0310907, -0.409286, 13.0720, 42.7198}
                              : VwnChannel{0.0310907, -0.10498, 3.72744, 12.9352};
  const VwnChannel ferro = rpa ? VwnChannel{0.01554535, -0.743294, 20.1231, 101.578}
                               : VwnChannel{0.01554535, -0.32500, 7.06042, 18.0578};
  const VwnChannel stiff = rpa ? VwnChannel{-0.016886863940389905, -0.228344, 1.06835, 11.4813}
                               : VwnChannel{-0.016886863940389905, -0.00475840, 1.13107, 13.0045};
  const double rs = cbrt(3.0 / (4.0 * kPiD * rho));
  const double x = sqrt(rs);
  const double zeta = fmin(fmax((ra - rb) / rho, -1.0), 1.0);
  double ep, dp, ef, df, ac, da;
  vwn_eps(x, para, ep, dp);
  vwn_eps(x, ferro, ef, df);
  vwn_eps(x, stiff, ac, da);
  double fz, dfz, ifdd;
  spin_f(zeta, fz, dfz, ifdd);
  const double z2 = zeta * zeta, z3 = z2 * zeta, z4 = z2 * z2, one_m_z4 = 1.0 - z4;
  const double dec = ef - ep, d_dec = df - dp;
  const double ec = ep + ac * fz * ifdd * one_m_z4 + dec * fz * z4;
  const double rs_dec = dp + da * fz * ifdd * one_m_z4 + d_dec * fz * z4;
  const double dec_dz = ac * ifdd * (dfz * one_m_z4 - 4.0 * z3 * fz) + dec * (dfz * z4 + 4.0 * z3 * fz);
  const double base = ec - (1.0 / 3.0) * rs_dec;
  o.f = rho * ec;
  o.vra = base + (1.0 - zeta) * dec_dz;
  o.vrb = base - (1.0 + zeta) * dec_dz;
  return o;
}

// -------------------------------------------------------------------------- B88 (xc.rs:388-424)
__host__ __device__ __forceinline__ void b88_spin(double r, double g, double& f, double& vr, double& vg) {
  if (r < kRhoFloor) { f = vr = vg = 0.0; return; }
  const double beta = 0.0042;
  const double r13 = cbrt(r), r43 = r * r13;
  const double s2 = fmax(g, 0.0) / (r43 * r43);
  const double s = sqrt(s2);
  const double ash = asinh(s);
  const double den = 1.0 + 6.0 * beta * s * ash;
  const double gfun = -beta * s2 / den;
  const double h = -beta * (2.0 + 6.0 * beta * s * ash - 6.0 * beta * s2 / sqrt(1.0 + s2)) / (den * den);
  f = r43 * gfun;
  vr = (4.0 / 3.0) * r13 * (gfun - s2 * h);
  vg = 0.5 * h / r43;
}

// -------------------------------------------------------------------------- LYP (xc.rs:433-547)
__host__ __device__ __forceinline__ void lyp_bracket_d(double ra, double rb, double delta, double ddelta, double gaa,
                                              double gab, double gbb, double& s, double& ds, double& aaa,
                                              double& aab, double& abb) {
  const double rho = ra + rb, rho2 = rho * rho;
  const double cf = 0.3 * pow(3.0 * kPiD * kPiD, 2.0 / 3.0);
  const double k0 = pow(2.0, 11.0 / 3.0) * cf;
  const double ra83 = ra > 0.0 ? pow(ra, 8.0 / 3.0) : 0.0;
  const double rb83 = rb > 0.0 ? pow(rb, 8.0 / 3.0) : 0.0;
  const double stf = k0 * ra * rb * (ra83 + rb83);
  const double dstf = k0 * ((11.0 / 3.0) * ra83 * rb + rb * rb83);
  const double cg = ra * rb * (47.0 - 7.0 * delta) / 18.0 - (2.0 / 3.0) * rho2;
  const double dcg = rb * (47.0 - 7.0 * delta) / 18.0 + ra * rb * (-7.0 * ddelta) / 18.0 - (4.0 / 3.0) * rho;
  const double c25 = 2.5 - delta / 18.0, c11 = (delta - 11.0) / 9.0;
  const double qa = ra * ra * rb / rho;
  const double dqa = (2.0 * ra * rb * rho - ra * ra * rb) / rho2;
  const double ea = -ra * rb * c25 - c11 * qa + ((2.0 / 3.0) * rho2 - rb * rb);
  const double dea = -rb * c25 + ra * rb * (ddelta / 18.0) - (ddelta / 9.0) * qa - c11 * dqa + (4.0 / 3.0) * rho;
  const double qb = ra * rb * rb / rho;
  const double dqb = (rb * rb * rho - ra * rb * rb) / rho2;
  const double eb = -ra * rb * c25 - c11 * qb + ((2.0 / 3.0) * rho2 - ra * ra);
  const double deb =
      -rb * c25 + ra * rb * (ddelta / 18.0) - (ddelta / 9.0) * qb - c11 * dqb + (4.0 / 3.0) * rho - 2.0 * ra;
  aaa = cg + ea;
  aab = 2.0 * cg;
  abb = cg + eb;
  s = stf + aaa * gaa + aab * gab + abb * gbb;
  ds = dstf + (dcg + dea) * gaa + (2.0 * dcg) * gab + (dcg + deb) * gbb;
}

__host__ __device__ __forceinline__ XcVal lyp_corr(double ra, double rb, double gaa, double gab, double gbb) {
  XcVal o = xc_zero();
  const double rho = ra + rb;
  if (rho < kRhoFloor) return o;
  const double A = 0.04918, B = 0.132, C = 0.2533, D = 0.349;
  const double rm13 = pow(rho, -1.0 / 3.0);
  const double den = 1.0 + D * rm13;
  const double g0 = -4.0 * A / (rho * den);
  const double dg0 = -g0 * (1.0 + (2.0 / 3.0) * D * rm13) / (rho * den);
  if (C * rm13 > 500.0) {  // exp(-C rho^-1/3) underflow guard (xc.rs:515-526)
    o.f = g0 * ra * rb;
    o.vra = dg0 * ra * rb + g0 * rb;
    o.vrb = dg0 * ra * rb + g0 * ra;
    return o;
  }
  const double t0 = g0 * ra * rb;
  const double dt0a = dg0 * ra * rb + g0 * rb;
  const double dt0b = dg0 * ra * rb + g0 * ra;
  const double omega = exp(-C * rm13) / den * pow(rho, -11.0 / 3.0);
  const double delta = C * rm13 + D * rm13 / den;
  const double domega = omega * (delta - 11.0) / (3.0 * rho);
  const double ddelta = -(1.0 / 3.0) * (rm13 / rho) * (C + D / (den * den));
  double s, dsa, aaa, aab, abb, s_b, dsb, u0, u1, u2;
  lyp_bracket_d(ra, rb, delta, ddelta, gaa, gab, gbb, s, dsa, aaa, aab, abb);
  lyp_bracket_d(rb, ra, delta, ddelta, gbb, gab, gaa, s_b, dsb, u0, u1, u2);
  const double ab = A * B;
  o.f = t0 - ab * omega * s;
  o.vra = dt0a - ab * (domega * s + omega * dsa);
  o.vrb = dt0b - ab * (domega * s + omega * dsb);
  o.vgaa = -ab * omega * aaa;
  o.vgab = -ab * omega * aab;
  o.vgbb = -ab * omega * abb;
  return o;
}

// -------------------------------------------------------------------------- PBE (xc.rs:556-828)
// PbeAbParams::CALCHEM_ANALYTIC (xc.rs:566-573)
constexpr double kKappa = 0.804;
constexpr double kMu = 0.2195149727645171;
constexpr double kBetaPbe = 0.06672455060314922;
constexpr double kGammaPbe = 0.0310906908696549;

__host__ __device__ __forceinline__ void pbex_spin(double r, double g, double& f, double& vr, double& vg) {
  if (r < kRhoFloor) { f = vr = vg = 0.0; return; }
  const double ru = 2.0 * r, gu = 4.0 * fmax(g, 0.0);  // spin scaling to the unpolarised form
  const double cxu = -0.75 * cbrt(3.0 / kPiD);
  const double r13 = cbrt(ru), r43 = ru * r13;
  const double exl = cxu * r43;
  const double kf = cbrt(3.0 * kPiD * kPiD * ru);
  const double den_s2 = 4.0 * kf * kf * ru * ru;
  const double s2 = gu / den_s2;
  const double q = 1.0 + (kMu / kKappa) * s2;
  const double fx = 1.0 + kKappa - kKappa / q;
  const double dfx = kMu / (q * q);
  f = 0.5 * exl * fx;
  vr = (4.0 / 3.0) * cxu * r13 * fx + exl * dfx * (-(8.0 / 3.0) * s2 / ru);
  vg = 2.0 * (exl * dfx / den_s2);
}

struct Pw92Channel { double a, a1, b1, b2, b3, b4; };

__host__ __device__ __forceinline__ void pw92(double rs, Pw92Channel c, double& g, double& dg) {
  const double x = sqrt(rs), x3 = rs * x, x4 = rs * rs;
  const double q0 = -2.0 * c.a * (1.0 + c.a1 * rs);
  const double q1 = 2.0 * c.a * (c.b1 * x + c.b2 * rs + c.b3 * x3 + c.b4 * x4);
  const double dq1 = c.a * (c.b1 / x + 2.0 * c.b2 + 3.0 * c.b3 * x + 4.0 * c.b4 * rs);
  const double ln = log(1.0 + 1.0 / q1);
  g = q0 * ln;
  dg = -2.0 * c.a * c.a1 * ln - q0 * dq1 / (q1 * (q1 + 1.0));
}

__host__ __device__ __forceinline__ XcVal pbe_corr(double ra, double rb, double gaa, double gab, double gbb) {
  XcVal o = xc_zero();
  const double rho = ra + rb;
  if (rho < kRhoFloor) return o;
  const double gt = fmax(gaa + 2.0 * gab + gbb, 0.0);
  const double rs = cbrt(3.0 / (4.0 * kPiD * rho));
  const double drs = -rs / (3.0 * rho);
  const double zeta = fmin(fmax((ra - rb) / rho, -1.0), 1.0);
  double e0, de0, e1, de1, mac, dmac;
  pw92(rs, Pw92Channel{0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294}, e0, de0);
  pw92(rs, Pw92Channel{0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517}, e1, de1);
  pw92(rs, Pw92Channel{0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671}, mac, dmac);
  const double ac = -mac, dac = -dmac;
  double fz, dfz, ifdd;
  spin_f(zeta, fz, dfz, ifdd);
  const double z2 = zeta * zeta, z3 = z2 * zeta, z4 = z2 * z2, one_m_z4 = 1.0 - z4;
  const double ec = e0 + ac * fz * ifdd * one_m_z4 + (e1 - e0) * fz * z4;
  const double dec_drs = de0 + dac * fz * ifdd * one_m_z4 + (de1 - de0) * fz * z4;
  const double dec_drho = dec_drs * drs;
  const double dec_dz = ac * ifdd * (dfz * one_m_z4 - 4.0 * z3 * fz) + (e1 - e0) * (dfz * z4 + 4.0 * z3 * fz);
  if (gt < 1e-36) {
    o.f = rho * ec;
    o.vra = ec + rho * dec_drho + (1.0 - zeta) * dec_dz;
    o.vrb = ec + rho * dec_drho - (1.0 + zeta) * dec_dz;
    return o;
  }
  const double b0 = kBetaPbe / kGammaPbe;
  const double zp = fmax(1.0 + zeta, 1e-24), zm = fmax(1.0 - zeta, 1e-24);
  const double zp13 = cbrt(zp), zm13 = cbrt(zm);
  const double zp23 = zp13 * zp13, zm23 = zm13 * zm13;
  const double phi = 0.5 * (zp23 + zm23), phi2 = phi * phi, phi3 = phi2 * phi;
  const double a_dphi = ((1.0 - zeta) * (1.0 / zp13) - zm23) / 3.0;   // (1 - zeta) dphi/dzeta
  const double b_dphi = ((1.0 + zeta) * (1.0 / zm13) - zp23) / 3.0;   // -(1 + zeta) dphi/dzeta
  const double ct = (16.0 / kPiD) * cbrt(3.0 * kPiD * kPiD);
  const double den_t2 = ct * phi2 * (rho * rho * cbrt(rho));
  const double t2 = gt / den_t2;
  const double gp3 = kGammaPbe * phi3;
  const double w = -ec / gp3;
  double af = 0.0, daw = 0.0;
  if (!(w > 100.0)) {
    const double em1 = expm1(w);
    af = b0 / em1;
    daw = -af * exp(w) / em1;
  }
  const double u = af * t2;
  const double dpol = 1.0 + u + u * u;
  const double za = 1.0 + b0 * t2 * ((1.0 + u) / dpol);
  const double lnz = log(za);
  const double h = gp3 * lnz;
  const double dh_dt2 = gp3 * (b0 * (1.0 + 2.0 * u) / (dpol * dpol)) / za;
  const double dh_dw = gp3 * ((-b0 * t2 * t2 * u * (2.0 + u) / (dpol * dpol)) * daw) / za;
  const double dh_drho = dh_dt2 * (-(7.0 / 3.0) * t2 / rho) + dh_dw * (-dec_drho / gp3);
  const double dh_dphi = 3.0 * kGammaPbe * phi2 * lnz + dh_dw * (-3.0 * w / phi) + dh_dt2 * (-2.0 * t2 / phi);
  const double dh_dec = dh_dw * (-1.0 / gp3);
  const double te = ec + h;
  const double common = te + rho * (dec_drho + dh_drho);
  o.f = rho * te;
  o.vra = common + (1.0 - zeta) * dec_dz * (1.0 + dh_dec) + dh_dphi * a_dphi;
  o.vrb = common - (1.0 + zeta) * dec_dz * (1.0 + dh_dec) + dh_dphi * b_dphi;
  const double vgt = rho * dh_dt2 / den_t2;
  o.vgaa = vgt;
  o.vgab = 2.0 * vgt;
  o.vgbb = vgt;
  return o;
}

// -------------------------------------------------------------------------- CAM-B3LYP (xc.rs:860-960)
// Short-range attenuation of LDA-type exchange, F(a) = 1 - (8/3) a [sqrt(pi) erf(1/(2a)) +
// (2a - 4a^3) exp(-1/(4a^2)) - 3a + 4a^3], with its small-a series and its large-a expansion in
// 1/a^2 (through a^-12, avoiding the cancellation of O(a^4) terms).
__host__ __device__ __forceinline__ void camb3lyp_attenuation(double a, double& f, double& df) {
  const double sqrt_pi = 1.7724538509055160273;
  if (a < 1e-5) {
    f = fmin(fmax(1.0 - (8.0 / 3.0) * a * sqrt_pi + 8.0 * a * a, 0.0), 1.0);
    df = -(8.0 / 3.0) * sqrt_pi + 16.0 * a;
    return;
  }
  if (a >= 2.0) {
    const double z = 1.0 / (a * a);
    const double c[6] = {1.0 / 36.0, -1.0 / 960.0, 1.0 / 26880.0, -1.0 / 829440.0, 1.0 / 28385280.0,
                         -1.0 / 1073479680.0};
    double pw = z;
    f = 0.0;
    df = 0.0;
    for (int k = 0; k < 6; ++k) {
      f += c[k] * pw;
      df -= (2 * (k + 1)) * c[k] * pw / a;
      pw *= z;
    }
    return;
  }
  const double a2 = a * a, a3 = a2 * a;
  const double ev = exp(-0.25 / a2);
  const double bracket = sqrt_pi * erf(0.5 / a) + (2.0 * a - 4.0 * a3) * ev - 3.0 * a + 4.0 * a3;
  f = fmin(fmax(1.0 - (8.0 / 3.0) * a * bracket, 0.0), 1.0);
  const double db = -3.0 + 12.0 * a2 * (1.0 - ev);
  df = -(8.0 / 3.0) * (bracket + a * db);
}

// ITYH-attenuated Slater + B88 exchange of one spin, w(a) = 0.35 + 0.46 F(a) with the gradient-
// dependent Fermi wave vector k = sqrt(9 pi / (2 K)) rho^(1/3), K = -f_x / rho^(4/3), mu = 0.33.
__host__ __device__ __forceinline__ void camb3lyp_x_spin(double r, double g, double& f, double& vr, double& vg) {
  f = vr = vg = 0.0;
  if (r < kRhoFloor) return;
  double fs, vs, fb, vb, gb;
  slater_spin(r, fs, vs);
  b88_spin(r, g, fb, vb, gb);
  const double fx = fs + fb, vrt = vs + vb, vgt = gb;
  const double kb = -fx / pow(r, 4.0 / 3.0);
  const double kf = sqrt(9.0 * kPiD / (2.0 * kb)) * cbrt(r);
  const double a = 0.33 / (2.0 * kf);
  double fa, dfa;
  camb3lyp_attenuation(a, fa, dfa);
  const double w = 0.35 + 0.46 * fa, dw = 0.46 * dfa;
  const double da_dr = a * (0.5 * vrt / fx - 1.0 / r);
  const double da_dg = 0.5 * a * vgt / fx;
  f = w * fx;
  vr = w * vrt + dw * da_dr * fx;
  vg = w * vgt + dw * da_dg * fx;
}

// -------------------------------------------------------------------------- wB97X(-D) (xc.rs:960-1103)
struct Wb97Params {
  double omega, cx[5], css[5], cab[5];
};
// Chai & Head-Gordon, J. Chem. Phys. 128, 084106 (2008) and Phys. Chem. Chem. Phys. 10, 6615 (2008).
__host__ __device__ __forceinline__ Wb97Params wb97_params(bool d) {
  if (!d)
    return Wb97Params{0.30, {0.842294, 0.726479, 1.04760, -5.70635, 13.2794},
                      {1.0, -4.33879, 18.2308, -31.7430, 17.2901}, {1.0, 2.37031, -11.3995, 6.58405, -3.78132}};
  return Wb97Params{0.20, {0.777964, 0.661160, 0.574541, -5.25671, 11.6386},
                    {1.0, -6.90539, 31.3343, -51.0533, 26.4423}, {1.0, 1.79413, -12.0477, 14.0847, -8.50809}};
}

// B97 power series in u = gamma x^2 / (1 + gamma x^2); returns g and dg/dx^2.
__host__ __device__ __forceinline__ void b97_poly(double gp, const double* c, double x2, double& gv, double& dg) {
  const double gx2 = gp * fmax(x2, 0.0);
  const double den = 1.0 + gx2;
  const double u = gx2 / den;
  const double du = gp / (den * den);
  gv = c[0] + u * (c[1] + u * (c[2] + u * (c[3] + u * c[4])));
  dg = (c[1] + u * (2.0 * c[2] + u * (3.0 * c[3] + 4.0 * u * c[4]))) * du;
}

// PW92 LSDA correlation: (rho eps_c, v_rho_a, v_rho_b).
__host__ __device__ __forceinline__ void pw92_lsda(double ra, double rb, double& f, double& va, double& vb) {
  f = va = vb = 0.0;
  const double rho = ra + rb;
  if (rho < kRhoFloor) return;
  const double rs = cbrt(3.0 / (4.0 * kPiD * rho));
  const double drs = -rs / (3.0 * rho);
  const double zeta = fmin(fmax((ra - rb) / rho, -1.0), 1.0);
  double e0, de0, e1, de1, mac, dmac;
  pw92(rs, Pw92Channel{0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294}, e0, de0);
  pw92(rs, Pw92Channel{0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517}, e1, de1);
  pw92(rs, Pw92Channel{0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671}, mac, dmac);
  const double ac = -mac, dac = -dmac;
  double fz, dfz, ifdd;
  spin_f(zeta, fz, dfz, ifdd);
  const double z2 = zeta * zeta, z3 = z2 * zeta, z4 = z2 * z2, om = 1.0 - z4;
  const double ec = e0 + ac * fz * ifdd * om + (e1 - e0) * fz * z4;
  const double dec_drs = de0 + dac * fz * ifdd * om + (de1 - de0) * fz * z4;
  const double dec_dz = ac * ifdd * (dfz * om - 4.0 * z3 * fz) + (e1 - e0) * (dfz * z4 + 4.0 * z3 * fz);
  f = rho * ec;
  va = ec + rho * dec_drs * drs + (1.0 - zeta) * dec_dz;
  vb = ec + rho * dec_drs * drs - (1.0 + zeta) * dec_dz;
}

__host__ __device__ __forceinline__ void wb97_x_spin(double r, double g, const Wb97Params& P, double& f, double& vr,
                                                     double& vg) {
  f = vr = vg = 0.0;
  if (r < kRhoFloor) return;
  double fs, vs;
  slater_spin(r, fs, vs);
  const double r13 = cbrt(r), r43 = r * r13, r83 = r43 * r43;
  const double kf = cbrt(6.0 * kPiD * kPiD * r);
  const double a = P.omega / (2.0 * kf);
  double fa, dfa;
  camb3lyp_attenuation(a, fa, dfa);
  const double da_dr = -a / (3.0 * r);
  const double fsr = fs * fa;
  const double vsr = vs * fa + fs * dfa * da_dr;
  const double x2 = fmax(g, 0.0) / r83;
  double gx, dgx;
  b97_poly(0.004, P.cx, x2, gx, dgx);
  f = fsr * gx;
  vr = vsr * gx + fsr * dgx * (-(8.0 / 3.0) * x2 / r);
  vg = fsr * dgx / r83;
}

__host__ __device__ __forceinline__ XcVal wb97_xc(double ra, double rb, double gaa, double gbb, bool d) {
  const Wb97Params P = wb97_params(d);
  XcVal o = xc_zero();
  double fxa, vxa, gxa, fxb, vxb, gxb;
  wb97_x_spin(ra, gaa, P, fxa, vxa, gxa);
  wb97_x_spin(rb, gbb, P, fxb, vxb, gxb);
  double ft, vta, vtb, fpa, vpa, dum, fpb, vpb;
  pw92_lsda(ra, rb, ft, vta, vtb);
  pw92_lsda(ra, 0.0, fpa, vpa, dum);
  pw92_lsda(0.0, rb, fpb, dum, vpb);
  const double fperp = ft - fpa - fpb, vperp_a = vta - vpa, vperp_b = vtb - vpb;
  double xa2 = 0.0, dxa_r = 0.0, dxa_g = 0.0, xb2 = 0.0, dxb_r = 0.0, dxb_g = 0.0;
  if (ra >= kRhoFloor) {
    const double r83 = pow(ra, 8.0 / 3.0);
    xa2 = fmax(gaa, 0.0) / r83;
    dxa_r = -(8.0 / 3.0) * xa2 / ra;
    dxa_g = 1.0 / r83;
  }
  if (rb >= kRhoFloor) {
    const double r83 = pow(rb, 8.0 / 3.0);
    xb2 = fmax(gbb, 0.0) / r83;
    dxb_r = -(8.0 / 3.0) * xb2 / rb;
    dxb_g = 1.0 / r83;
  }
  double gsa, dgsa, gsb, dgsb, gab, dgab;
  b97_poly(0.2, P.css, xa2, gsa, dgsa);
  b97_poly(0.2, P.css, xb2, gsb, dgsb);
  b97_poly(0.006, P.cab, 0.5 * (xa2 + xb2), gab, dgab);
  o.f = fxa + fxb + fpa * gsa + fpb * gsb + fperp * gab;
  o.vra = vxa + vpa * gsa + fpa * dgsa * dxa_r + vperp_a * gab + fperp * dgab * 0.5 * dxa_r;
  o.vrb = vxb + vpb * gsb + fpb * dgsb * dxb_r + vperp_b * gab + fperp * dgab * 0.5 * dxb_r;
  o.vgaa = gxa + fpa * dgsa * dxa_g + fperp * dgab * 0.5 * dxa_g;
  o.vgbb = gxb + fpb * dgsb * dxb_g + fperp * dgab * 0.5 * dxb_g;
  return o;
}

// -------------------------------------------------------------------------- mixtures (xc.rs:159-223)
__host__ __device__ __forceinline__ XcVal xc_eval(int code, double rho_a, double rho_b, double g_aa, double g_ab,
                                         double g_bb) {
  XcVal o = xc_zero();
  const double ra = fmax(rho_a, 0.0), rb = fmax(rho_b, 0.0);
  if (ra + rb < kRhoFloor) return o;
  const double gaa = fmax(g_aa, 0.0), gbb = fmax(g_bb, 0.0);
  const double gab = g_ab;  // not clamped (xc.rs:167-168)
  double fa, va, fb, vb, ga, gb;
  // exchange-type terms are per spin
  if (code == 0 || code == 1 || code == 3 || code == 4) {  // Slater
    const double sc = (code == 3 || code == 4) ? 0.80 : 1.0;
    slater_spin(ra, fa, va);
    slater_spin(rb, fb, vb);
    o.f += sc * (fa + fb);
    o.vra += sc * va;
    o.vrb += sc * vb;
  }
  if (code == 1 || code == 3 || code == 4) {  // B88 gradient correction
    const double sc = code == 1 ? 1.0 : 0.72;
    b88_spin(ra, gaa, fa, va, ga);
    b88_spin(rb, gbb, fb, vb, gb);
    o.f += sc * (fa + fb);
    o.vra += sc * va;
    o.vrb += sc * vb;
    o.vgaa += sc * ga;
    o.vgbb += sc * gb;
  }
  if (code == 2 || code == 5) {  // PBE exchange
    const double sc = code == 2 ? 1.0 : 0.75;
    pbex_spin(ra, gaa, fa, va, ga);
    pbex_spin(rb, gbb, fb, vb, gb);
    o.f += sc * (fa + fb);
    o.vra += sc * va;
    o.vrb += sc * vb;
    o.vgaa += sc * ga;
    o.vgbb += sc * gb;
  }
  if (code == 0) xc_axpy(o, 1.0, vwn_corr(ra, rb, false));
  if (code == 3) xc_axpy(o, 0.19, vwn_corr(ra, rb, true));
  if (code == 4) xc_axpy(o, 0.19, vwn_corr(ra, rb, false));
  if (code == 1) xc_axpy(o, 1.0, lyp_corr(ra, rb, gaa, gab, gbb));
  if (code == 3 || code == 4) xc_axpy(o, 0.81, lyp_corr(ra, rb, gaa, gab, gbb));
  if (code == 2 || code == 5) xc_axpy(o, 1.0, pbe_corr(ra, rb, gaa, gab, gbb));
  if (code == 6) {  // CAM-B3LYP: attenuated Slater + B88 per spin, 0.19 VWN5, 0.81 LYP
    camb3lyp_x_spin(ra, gaa, fa, va, ga);
    camb3lyp_x_spin(rb, gbb, fb, vb, gb);
    o.f += fa + fb;
    o.vra += va;
    o.vrb += vb;
    o.vgaa += ga;
    o.vgbb += gb;
    xc_axpy(o, 0.19, vwn_corr(ra, rb, false));
    xc_axpy(o, 0.81, lyp_corr(ra, rb, gaa, gab, gbb));
  }
  if (code == 7 || code == 8) o = wb97_xc(ra, rb, gaa, gbb, code == 8);
  return o;
}

// -------------------------------------------------------------------------- closed shell
// The same functionals at rho_a = rho_b = r, gamma_aa = gamma_ab = gamma_bb = g (an RKS point), for
// the tensor-core form.  At zeta = 0 the spin interpolation terms of VWN and PW92 vanish exactly and
// the two LYP brackets coincide, so only the paramagnetic channels and one bracket are evaluated.
// One cube root serves every term (rho^(1/3) = 2^(1/3) r^(1/3), r^(8/3) = r^2 (r^(1/3))^2,
// rho^(-11/3) = rho^(-2/3) / rho^3), asinh(s) = log1p(s + s^2 / (1 + sqrt(1 + s^2))) reuses the
// square root B88 needs anyway, exp(w) = expm1(w) + 1, and the constant factors are literals (their
// values computed in double precision from the definitions beside them).  The results agree with
// xc_eval(code, r, r, g, g, g) to rounding (~1e-15 relative).
struct XcCs {
  double f;   // energy density
  double vr;  // dF/drho_a (= dF/drho_b)
  double vg;  // dF/dgamma_aa + dF/dgamma_ab / 2, the coefficient of the RKS gradient term
};

constexpr double kCsCbrt2 = 1.2599210498948732;       // 2^(1/3)
constexpr double kCsCx = 0.9305257363491;             // 3/4 (6/pi)^(1/3)
constexpr double kCsRsK = 0.6203504908994001;         // (3/(4 pi))^(1/3)
constexpr double kCsK0 = 36.46239897876477;           // 2^(11/3) 0.3 (3 pi^2)^(2/3)
constexpr double kCsCbrt3Pi2 = 3.0936677262801355;    // (3 pi^2)^(1/3)
constexpr double kCsCxu = -0.7385587663820223;        // -3/4 (3/pi)^(1/3)
constexpr double kCsCt = 15.755920349483144;          // (16/pi) (3 pi^2)^(1/3)

// Paramagnetic VWN channel with its derived constants: q = sqrt(4c - b^2), c1 = 2b/q,
// c2 = b x0 / X(x0), c3 = 2(b + 2 x0)/q.
struct VwnPara { double a, x0, b, c, q, c1, c2, c3; };
constexpr VwnPara kVwn5Para{0.0310907, -0.10498, 3.72744, 12.9352,
                            6.15199081975908, 1.2117833427280607, -0.031167608678943783, 1.1435257636284148};
constexpr VwnPara kVwnRpaPara{0.0310907, -0.409286, 13.0720, 42.7198,
                              0.0448998886415768, 582.2731590427809, -0.14253052416798392, 545.8110641572265};

__host__ __device__ __forceinline__ XcCs xc_eval_cs(int code, double r_in, double g_in) {
  if (code >= 6) {  // range-separated functionals: the spin form at rho_a = rho_b
    const XcVal v = xc_eval(code, r_in, r_in, g_in, g_in, g_in);
    return XcCs{v.f, v.vra, v.vgaa + 0.5 * v.vgab};
  }
  XcCs o{0.0, 0.0, 0.0};
  const double r = fmax(r_in, 0.0);
  const double rho = r + r;
  if (rho < kRhoFloor) return o;
  const double g = fmax(g_in, 0.0);
  const double c13 = cbrt(r);
  const double rho13 = kCsCbrt2 * c13;
  const bool spin_on = !(r < kRhoFloor);  // the per-spin floor of the exchange terms
  if (spin_on && (code == 0 || code == 1 || code == 3 || code == 4)) {  // Slater
    const double sc = (code == 3 || code == 4) ? 0.80 : 1.0;
    o.f += sc * (-2.0 * kCsCx * r * c13);
    o.vr += sc * (-(4.0 / 3.0) * kCsCx * c13);
  }
  if (spin_on && (code == 1 || code == 3 || code == 4)) {  // B88
    const double sc = code == 1 ? 1.0 : 0.72;
    const double beta = 0.0042;
    const double r43 = r * c13;
    const double s2 = g / (r43 * r43);
    const double s = sqrt(s2);
    const double q1 = sqrt(1.0 + s2);
    const double ash = log1p(s + s2 / (1.0 + q1));
    const double den = 1.0 + 6.0 * beta * s * ash;
    const double gfun = -beta * s2 / den;
    const double h = -beta * (2.0 + 6.0 * beta * s * ash - 6.0 * beta * s2 / q1) / (den * den);
    o.f += sc * (2.0 * r43 * gfun);
    o.vr += sc * ((4.0 / 3.0) * c13 * (gfun - s2 * h));
    o.vg += sc * (0.5 * h / r43);
  }
  if (spin_on && (code == 2 || code == 5)) {  // PBE exchange (spin scaling: rho_u = rho, gamma_u = 4g)
    const double sc = code == 2 ? 1.0 : 0.75;
    const double r43 = rho * rho13;
    const double exl = kCsCxu * r43;
    const double kf = kCsCbrt3Pi2 * rho13;
    const double den_s2 = 4.0 * kf * kf * rho * rho;
    const double s2 = 4.0 * g / den_s2;
    const double q = 1.0 + (kMu / kKappa) * s2;
    const double fx = 1.0 + kKappa - kKappa / q;
    const double dfx = kMu / (q * q);
    o.f += sc * (exl * fx);
    o.vr += sc * ((4.0 / 3.0) * kCsCxu * rho13 * fx + exl * dfx * (-(8.0 / 3.0) * s2 / rho));
    o.vg += sc * (2.0 * (exl * dfx / den_s2));
  }
  if (code == 0 || code == 3 || code == 4) {  // VWN5 / VWN_RPA, paramagnetic channel
    const double sc = code == 0 ? 1.0 : 0.19;
    const VwnPara ch = code == 3 ? kVwnRpaPara : kVwn5Para;
    const double x = sqrt(kCsRsK / rho13);
    const double X = x * x + ch.b * x + ch.c;
    const double at = atan(ch.q / (2.0 * x + ch.b));
    const double dx0 = x - ch.x0;
    const double ep = ch.a * (log(x * x / X) + ch.c1 * at - ch.c2 * (log(dx0 * dx0 / X) + ch.c3 * at));
    const double dp = ch.a * (ch.c * dx0 - ch.b * x * ch.x0) / (dx0 * X);
    o.f += sc * (rho * ep);
    o.vr += sc * (ep - (1.0 / 3.0) * dp);
  }
  if (code == 1 || code == 3 || code == 4) {  // LYP
    const double sc = code == 1 ? 1.0 : 0.81;
    const double A = 0.04918, B = 0.132, C = 0.2533, D = 0.349;
    const double rm13 = 1.0 / rho13;
    const double den = 1.0 + D * rm13;
    const double g0 = -4.0 * A / (rho * den);
    const double dg0 = -g0 * (1.0 + (2.0 / 3.0) * D * rm13) / (rho * den);
    const double t0 = g0 * r * r;
    const double dt0 = dg0 * r * r + g0 * r;
    if (C * rm13 > 500.0) {
      o.f += sc * t0;
      o.vr += sc * dt0;
    } else {
      const double rho2 = rho * rho;
      const double omega = exp(-C * rm13) / den * (rm13 * rm13 / (rho2 * rho));
      const double delta = C * rm13 + D * rm13 / den;
      const double domega = omega * (delta - 11.0) / (3.0 * rho);
      const double ddelta = -(1.0 / 3.0) * (rm13 / rho) * (C + D / (den * den));
      const double r2 = r * r, r83 = r2 * c13 * c13;
      const double stf = kCsK0 * r2 * (r83 + r83);
      const double dstf = kCsK0 * ((11.0 / 3.0) * r83 * r + r * r83);
      const double cg = r2 * (47.0 - 7.0 * delta) / 18.0 - (2.0 / 3.0) * rho2;
      const double dcg = r * (47.0 - 7.0 * delta) / 18.0 + r2 * (-7.0 * ddelta) / 18.0 - (4.0 / 3.0) * rho;
      const double c25 = 2.5 - delta / 18.0, c11 = (delta - 11.0) / 9.0;
      const double qa = r2 * r / rho;
      const double dqa = (2.0 * r2 * rho - r2 * r) / rho2;
      const double dqb = (r2 * rho - r2 * r) / rho2;
      const double ea = -r2 * c25 - c11 * qa + ((2.0 / 3.0) * rho2 - r2);
      const double dea = -r * c25 + r2 * (ddelta / 18.0) - (ddelta / 9.0) * qa - c11 * dqa + (4.0 / 3.0) * rho;
      const double deb =
          -r * c25 + r2 * (ddelta / 18.0) - (ddelta / 9.0) * qa - c11 * dqb + (4.0 / 3.0) * rho - 2.0 * r;
      const double aaa = cg + ea, aab = 2.0 * cg;
      const double sb = stf + (aaa + aab + aaa) * g;
      const double ds = dstf + (dcg + dea) * g + (2.0 * dcg) * g + (dcg + deb) * g;
      const double ab = A * B;
      o.f += sc * (t0 - ab * omega * sb);
      o.vr += sc * (dt0 - ab * (domega * sb + omega * ds));
      o.vg += sc * (-ab * omega * (aaa + 0.5 * aab));
    }
  }
  if (code == 2 || code == 5) {  // PBE correlation on the paramagnetic PW92 channel
    const double gt = 4.0 * g;
    const double rs = kCsRsK / rho13;
    const double drs = -rs / (3.0 * rho);
    double ec, de0;
    pw92(rs, Pw92Channel{0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294}, ec, de0);
    const double dec_drho = de0 * drs;
    if (gt < 1e-36) {
      o.f += rho * ec;
      o.vr += ec + rho * dec_drho;
    } else {
      const double b0 = kBetaPbe / kGammaPbe;
      const double den_t2 = kCsCt * (rho * rho * rho13);
      const double t2 = gt / den_t2;
      const double gp3 = kGammaPbe;
      const double w = -ec / gp3;
      double af = 0.0, daw = 0.0;
      if (!(w > 100.0)) {
        const double em1 = expm1(w);
        af = b0 / em1;
        daw = -af * (em1 + 1.0) / em1;
      }
      const double u = af * t2;
      const double dpol = 1.0 + u + u * u;
      const double za = 1.0 + b0 * t2 * ((1.0 + u) / dpol);
      const double lnz = log(za);
      const double h = gp3 * lnz;
      const double dh_dt2 = gp3 * (b0 * (1.0 + 2.0 * u) / (dpol * dpol)) / za;
      const double dh_dw = gp3 * ((-b0 * t2 * t2 * u * (2.0 + u) / (dpol * dpol)) * daw) / za;
      const double dh_drho = dh_dt2 * (-(7.0 / 3.0) * t2 / rho) + dh_dw * (-dec_drho / gp3);
      const double te = ec + h;
      o.f += rho * te;
      o.vr += te + rho * (dec_drho + dh_drho);
      o.vg += 2.0 * (rho * dh_dt2 / den_t2);
    }
  }
  return o;
}

}  // namespace cxc
