// host_prep.cpp -- host-side preparation for the XC quadrature library.
//
// Everything here runs once per geometry (CalChem does the same work in Rust before each
// engine is built):
//   * contraction normalisation of Cartesian shells and the per-shell screening data
//     (crates/calchem-basis/src/normalization.rs:20-97, lib.rs:462-573; ao_grid.rs:28-71);
//   * the overlap matrix (crates/calchem-int/src/one_electron.rs:7-31, 115-128), used to seed
//     S-orthonormal densities;
//   * the Lebedev-Laikov tables and the Euler-Maclaurin radial shells of every atom
//     (lebedev.rs:69-247; grid.rs:58-220, 742-760), which the GPU grid builder consumes;
//   * the 128-point batches with their bounding spheres and candidate shells (vxc.rs:443-493).
// Compiled with -ffp-contract=off so that its arithmetic rounds like the reference's Rust.
#include "host_prep.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

namespace cxc {

namespace {
constexpr double kPi = 3.14159265358979323846;

// Integer power with the multiplication order of compiler-rt's __powidf2 (Rust's f64::powi).
double ipow(double a, int b) {
  const bool recip = b < 0;
  double r = 1.0;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

double odd_dfact(int k) {
  double acc = 1.0;
  for (; k > 0; k -= 2) acc *= (double)k;
  return acc;
}

// Cartesian component order of each shell type (calchem-basis/src/lib.rs:135-160).
const int kCart[4][10][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}},
    {{3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {1, 1, 1}, {1, 0, 2}, {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}}};
}  // namespace

double gto_norm(double alpha, int l, int m, int n) {
  const double radial = std::pow(2.0 * alpha / kPi, 0.75);
  const double num = ipow(4.0 * alpha, l + m + n);
  const double den = odd_dfact(2 * l - 1) * odd_dfact(2 * m - 1) * odd_dfact(2 * n - 1);
  return radial * std::sqrt(num / den);
}

int prepare_shells(int n_shells, const int* l, const int* atom, const double* centers, const int* n_prims,
                   const double* exps, const double* coefs, AoShellGpu* so, AoPrimGpu* po, AoCompGpu* co,
                   int* n_ao_out) {
  int ao = 0, pbase = 0, cbase = 0;
  for (int s = 0; s < n_shells; ++s) {
    const int L = l[s], np = n_prims[s];
    if (L < 0 || L > 3 || np <= 0) return -1;
    const double* ex = exps + pbase;
    const double* cf = coefs + pbase;
    for (int p = 0; p < np; ++p)
      if (!(std::isfinite(ex[p]) && ex[p] > 0.0 && std::isfinite(cf[p]))) return -1;
    // <phi|phi> of the raw contraction for the axial component (L,0,0)
    double self = 0.0;
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) {
        const double g = ex[i] + ex[j];
        double ang = 1.0;
        if (L > 0) ang *= odd_dfact(2 * L - 1) / ipow(2.0 * g, L);
        const double sij = gto_norm(ex[i], L, 0, 0) * gto_norm(ex[j], L, 0, 0) * std::pow(kPi / g, 1.5) * ang;
        self += cf[i] * cf[j] * sij;
      }
    if (!(std::isfinite(self) && self > 0.0)) return -1;
    const double scale = 1.0 / std::sqrt(self);
    double amin = INFINITY;
    for (int p = 0; p < np; ++p) {
      const double nrm = gto_norm(ex[p], L, 0, 0);
      po[pbase + p].exponent = ex[p];
      po[pbase + p].weighted_norm = (cf[p] * scale) * nrm;
      amin = std::min(amin, ex[p]);
    }
    amin = std::max(amin, 1e-12);
    const int nf = (L + 1) * (L + 2) / 2;
    const double lead = gto_norm(ex[0], L, 0, 0);
    for (int c = 0; c < nf; ++c) {
      const int* q = kCart[L][c];
      co[cbase + c].scale = lead == 0.0 ? 1.0 : gto_norm(ex[0], q[0], q[1], q[2]) / lead;
      co[cbase + c].lx = q[0];
      co[cbase + c].ly = q[1];
      co[cbase + c].lz = q[2];
      co[cbase + c]._pad = 0;
    }
    AoShellGpu& sh = so[s];
    for (int k = 0; k < 3; ++k) sh.center[k] = centers[3 * s + k];
    sh.r2_cutoff = (40.0 + 4.0 * L) / amin;
    sh.ao_offset = ao;
    sh.n_funcs = nf;
    sh.prim_start = pbase;
    sh.n_prims = np;
    sh.comp_start = cbase;
    sh.atom_index = atom[s];
    ao += nf;
    pbase += np;
    cbase += nf;
  }
  *n_ao_out = ao;
  return 0;
}

namespace {
// Obara-Saika 1-D overlap (primitive.rs:44-63), iterative over a small table.
double os_overlap_1d(int la, int lb, double pa, double pb, double g) {
  double t[8][8];
  const double i2g = 0.5 / g;
  for (int a = 0; a <= la; ++a)
    for (int b = 0; b <= lb; ++b) {
      double v;
      if (a == 0 && b == 0) v = std::sqrt(kPi / g);
      else if (a > 0) {
        v = pa * t[a - 1][b];
        if (a > 1) v += (a - 1) * i2g * t[a - 2][b];
        if (b > 0) v += b * i2g * t[a - 1][b - 1];
      } else {
        v = pb * t[a][b - 1];
        if (b > 1) v += (b - 1) * i2g * t[a][b - 2];
      }
      t[a][b] = v;
    }
  return t[la][lb];
}
}  // namespace

void overlap_matrix(const AoShellGpu* sh, int n_shells, const AoPrimGpu* pr, const AoCompGpu* co, int n_ao,
                    double* S) {
  // weighted_norm carries c_p N(alpha_p; L,0,0); component scale carries N(lmn)/N(L00), which is
  // independent of alpha, so c_p N(alpha_p; lmn) = weighted_norm * scale.
#pragma omp parallel for schedule(dynamic, 4)
  for (int a = 0; a < n_shells; ++a) {
    const AoShellGpu& A = sh[a];
    for (int b = 0; b < n_shells; ++b) {
      const AoShellGpu& B = sh[b];
      double ab2 = 0;
      for (int k = 0; k < 3; ++k) ab2 += (A.center[k] - B.center[k]) * (A.center[k] - B.center[k]);
      for (int ia = 0; ia < A.n_funcs; ++ia) {
        const AoCompGpu& ca = co[A.comp_start + ia];
        for (int ib = 0; ib < B.n_funcs; ++ib) {
          const AoCompGpu& cb = co[B.comp_start + ib];
          double sum = 0;
          for (int p = 0; p < A.n_prims; ++p) {
            const double al = pr[A.prim_start + p].exponent;
            for (int q = 0; q < B.n_prims; ++q) {
              const double be = pr[B.prim_start + q].exponent;
              const double g = al + be;
              double pa[3], pb[3];
              for (int k = 0; k < 3; ++k) {
                const double P = (al * A.center[k] + be * B.center[k]) / g;
                pa[k] = P - A.center[k];
                pb[k] = P - B.center[k];
              }
              const double s = std::exp(-(al * be / g) * ab2) * os_overlap_1d(ca.lx, cb.lx, pa[0], pb[0], g) *
                               os_overlap_1d(ca.ly, cb.ly, pa[1], pb[1], g) *
                               os_overlap_1d(ca.lz, cb.lz, pa[2], pb[2], g);
              sum += pr[A.prim_start + p].weighted_norm * pr[B.prim_start + q].weighted_norm * s;
            }
          }
          S[(size_t)(A.ao_offset + ia) * n_ao + B.ao_offset + ib] = ca.scale * cb.scale * sum;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Lebedev-Laikov rules: orbit generators and the published parameters (Lebedev & Laikov 1999),
// in the generator order CalChem uses (lebedev.rs:79-247) so that point order matches.
// ---------------------------------------------------------------------------------------------
namespace {
struct Orbit { int kind; double a, b, v; };

void emit_signs(std::vector<double>& t, double x, double y, double z, double w) {
  const double sg[2] = {-1.0, 1.0};
  for (double sx : sg)
    for (double sy : sg)
      for (double sz : sg) t.insert(t.end(), {sx * x, sy * y, sz * z, w});
}

void emit_orbit(std::vector<double>& t, const Orbit& o) {
  const double w = 4.0 * kPi * o.v;
  const double sg[2] = {-1.0, 1.0};
  if (o.kind == 1) {
    for (double s : sg) t.insert(t.end(), {s, 0.0, 0.0, w, 0.0, s, 0.0, w, 0.0, 0.0, s, w});
  } else if (o.kind == 2) {
    const double h = std::sqrt(0.5);
    const double hs[2] = {-h, h};
    for (double s1 : hs)
      for (double s2 : hs) t.insert(t.end(), {s1, s2, 0.0, w, s1, 0.0, s2, w, 0.0, s1, s2, w});
  } else if (o.kind == 3) {
    const double c = std::sqrt(1.0 / 3.0);
    emit_signs(t, c, c, c, w);
  } else if (o.kind == 4) {
    const double m = std::sqrt(1.0 - 2.0 * o.a * o.a);
    emit_signs(t, o.a, o.a, m, w);
    emit_signs(t, o.a, m, o.a, w);
    emit_signs(t, m, o.a, o.a, w);
  } else if (o.kind == 5) {
    const double q = std::sqrt(1.0 - o.a * o.a);
    const double pr[2][2] = {{o.a, q}, {q, o.a}};
    for (const auto& uv : pr)
      for (double su : sg)
        for (double st : sg)
          t.insert(t.end(), {su * uv[0], st * uv[1], 0.0, w, su * uv[0], 0.0, st * uv[1], w, 0.0, su * uv[0],
                             st * uv[1], w});
  } else {
    const double c = std::sqrt(1.0 - o.a * o.a - o.b * o.b);
    const double p[6][3] = {{o.a, o.b, c}, {o.b, o.a, c}, {c, o.a, o.b}, {o.a, c, o.b}, {c, o.b, o.a}, {o.b, c, o.a}};
    for (const auto& q : p) emit_signs(t, q[0], q[1], q[2], w);
  }
}

const std::vector<Orbit>& orbits(int n) {
  static const std::vector<Orbit> r26 = {{1, 0, 0, 0.4761904761904762e-1}, {2, 0, 0, 0.3809523809523810e-1},
                                         {3, 0, 0, 0.3214285714285714e-1}};
  static const std::vector<Orbit> r50 = {{1, 0, 0, 0.1269841269841270e-1}, {2, 0, 0, 0.2257495590828924e-1},
                                         {3, 0, 0, 0.2109375000000000e-1},
                                         {4, 0.3015113445777636, 0, 0.2017333553791887e-1}};
  static const std::vector<Orbit> r110 = {
      {1, 0, 0, 0.3828270494937162e-2}, {3, 0, 0, 0.9793737512487512e-2},
      {4, 0.1851156353447362, 0, 0.8211737283191111e-2}, {4, 0.6904210483822922, 0, 0.9942814891178103e-2},
      {4, 0.3956894730559419, 0, 0.9595471336070963e-2}, {5, 0.4783690288121502, 0, 0.9694996361663028e-2}};
  static const std::vector<Orbit> r194 = {
      {1, 0, 0, 0.1782340447244611e-2},
      {2, 0, 0, 0.5716905949977102e-2},
      {3, 0, 0, 0.5573383178848738e-2},
      {4, 0.6712973442695226, 0, 0.5608704082587997e-2},
      {4, 0.2892465627575439, 0, 0.5158237711805383e-2},
      {4, 0.4446933178717437, 0, 0.5518771467273614e-2},
      {4, 0.1299335447650067, 0, 0.4106777028169394e-2},
      {5, 0.3457702197611283, 0, 0.5051846064614808e-2},
      {6, 0.1590417105383530, 0.8360360154824589, 0.5530248916233094e-2}};
  static const std::vector<Orbit> r302 = {
      {1, 0, 0, 0.8545911725128148e-3},
      {3, 0, 0, 0.3599119285025571e-2},
      {4, 0.3515640345570105, 0, 0.3449788424305883e-2},
      {4, 0.6566329410219612, 0, 0.3604822601419882e-2},
      {4, 0.4729054132581005, 0, 0.3576729661743367e-2},
      {4, 0.9618308522614784e-1, 0, 0.2352101413689164e-2},
      {4, 0.2219645236294178, 0, 0.3108953122413675e-2},
      {4, 0.7011766416089545, 0, 0.3650045807677255e-2},
      {5, 0.2644152887060663, 0, 0.2982344963171804e-2},
      {5, 0.5718955891878961, 0, 0.3600820932216460e-2},
      {6, 0.2510034751770465, 0.8000727494073952, 0.3571540554273387e-2},
      {6, 0.1233548532583327, 0.4127724083168531, 0.3392312205006170e-2}};
  static const std::vector<Orbit> r590 = {
      {1, 0, 0, 0.3095121295306187e-3},
      {3, 0, 0, 0.1852379698597489e-2},
      {4, 0.7040954938227469, 0, 0.1871790639277744e-2},
      {4, 0.6807744066455243, 0, 0.1858812585438317e-2},
      {4, 0.6372546939258752, 0, 0.1852028828296213e-2},
      {4, 0.5044419707800358, 0, 0.1846715956151242e-2},
      {4, 0.4215761784010967, 0, 0.1818471778162769e-2},
      {4, 0.3317920736472123, 0, 0.1749564657281154e-2},
      {4, 0.2384736701421887, 0, 0.1617210647254411e-2},
      {4, 0.1459036449157763, 0, 0.1384737234851692e-2},
      {4, 0.06095034115507196, 0, 0.9764331165051050e-3},
      {5, 0.6116843442009876, 0, 0.1857161196774078e-2},
      {5, 0.3964755348199858, 0, 0.1705153996395864e-2},
      {5, 0.1724782009907724, 0, 0.1300321685886048e-2},
      {6, 0.5610263808622060, 0.3518280927733519, 0.1842866472905286e-2},
      {6, 0.4742392842551980, 0.2634716655937950, 0.1802658934377451e-2},
      {6, 0.5984126497885380, 0.1816640840360209, 0.1849830560443660e-2},
      {6, 0.3791035407695563, 0.1720795225656878, 0.1713904507106709e-2},
      {6, 0.2778673190586244, 0.08213021581932511, 0.1555213603396808e-2},
      {6, 0.5033564271075117, 0.08999205842074875, 0.1802239128008525e-2}};
  switch (n) {
    case 26: return r26;
    case 50: return r50;
    case 110: return r110;
    case 194: return r194;
    case 302: return r302;
    default: return r590;
  }
}
}  // namespace

const LebedevTables& lebedev_tables() {
  static LebedevTables T;
  static std::once_flag once;
  std::call_once(once, [] {
    const int sizes[6] = {26, 50, 110, 194, 302, 590};
    for (int i = 0; i < 6; ++i) {
      T.offset[i] = (int)(T.xyzw.size() / 4);
      for (const Orbit& o : orbits(sizes[i])) emit_orbit(T.xyzw, o);
      T.count[i] = (int)(T.xyzw.size() / 4) - T.offset[i];
    }
  });
  return T;
}

int lebedev_index(int npts) {
  switch (npts) {
    case 26: return 0;
    case 50: return 1;
    case 110: return 2;
    case 194: return 3;
    case 302: return 4;
    case 590: return 5;
    default: return -1;
  }
}

double bragg_slater_bohr(int z) {
  // Bragg-Slater radii in Angstrom (Becke 1988 appendix, H = 0.35), grid.rs:58-101.
  static const double tbl[57] = {0,    0.35, 0.35, 1.45, 1.05, 0.85, 0.70, 0.65, 0.60, 0.50, 0.45, 1.80, 1.50, 1.25,
                                 1.10, 1.00, 1.00, 1.00, 1.00, 2.20, 1.80, 1.40, 1.40, 1.40, 1.40, 1.40, 1.40, 1.40,
                                 1.40, 1.40, 1.40, 1.30, 1.25, 1.15, 1.15, 1.15, 1.10, 2.35, 2.00, 1.55, 1.55, 1.55,
                                 1.55, 1.55, 1.55, 1.55, 1.55, 1.55, 1.55, 1.55, 1.45, 1.45, 1.40, 1.40, 1.35, 2.60,
                                 2.15};
  const double ang = (z >= 1 && z <= 56) ? tbl[z] : 1.75;
  return ang * 1.8897261245650618;
}

double becke_shift(int zc, int zd) {
  if (zc == zd) return 0.0;
  const double chi = bragg_slater_bohr(zc) / bragg_slater_bohr(zd);
  const double u = (chi - 1.0) / (chi + 1.0);
  const double a = u / (u * u - 1.0);
  return a < -0.5 ? -0.5 : (a > 0.5 ? 0.5 : a);
}

int radial_count(int z, int level) {
  // grid.rs:142-173, with the Fine-level floor of 99 shells (grid.rs:745-752)
  int n;
  switch (level) {
    case 0: n = z <= 2 ? 25 : (z <= 18 ? 35 : 45); break;
    case 1: n = z <= 2 ? 35 : (z <= 18 ? 50 : 65); break;
    case 2: n = z <= 2 ? 55 : (z <= 18 ? 75 : 90); break;
    default: n = 200;
  }
  return n;
}

int angular_points(double r, double rbs, int level) {
  const double x = r / std::max(rbs, 0.3);
  switch (level) {
    case 0: return x < 0.25 ? 26 : x < 0.75 ? 50 : x < 4.5 ? 110 : 50;
    case 1: return x < 0.20 ? 26 : x < 0.55 ? 50 : x < 1.10 ? 110 : x < 4.50 ? 194 : 110;
    case 2: return x < 0.18 ? 50 : x < 0.50 ? 110 : x < 0.95 ? 194 : x < 5.00 ? 302 : 194;
    default: return 590;
  }
}

void radial_shells(int n_atoms, const int* z, int level, int radial_min, std::vector<RadialShell>& out,
                   long long* n_raw) {
  out.clear();
  const LebedevTables& T = lebedev_tables();
  long long raw = 0;
  for (int a = 0; a < n_atoms; ++a) {
    const double rbs = bragg_slater_bohr(z[a]);
    int nr = std::max(radial_count(z[a], level), radial_min);
    if (level == 2) nr = std::max(nr, 99);
    const double m = (double)(nr + 1);
    for (int i = 1; i <= nr; ++i) {
      const double t = (double)i, mt = m - t;
      RadialShell rs;
      rs.atom = a;
      rs.r = rbs * (t * t) / (mt * mt);
      rs.w_rad = 2.0 * ipow(rbs, 3) * m * ipow(t, 5) / ipow(mt, 7);
      const int li = lebedev_index(angular_points(rs.r, rbs, level));
      rs.leb_offset = T.offset[li];
      rs.n_ang = T.count[li];
      rs.raw_start = raw;
      raw += rs.n_ang;
      out.push_back(rs);
    }
  }
  *n_raw = raw;
}

void radial_shells_atoms(int n_atoms, const int* z, const int* n_rad, const int* region_leb, const double* x_max,
                         std::vector<RadialShell>& out, long long* n_raw) {
  static const int kFineRegion[5] = {50, 110, 194, 302, 194};
  out.clear();
  const LebedevTables& T = lebedev_tables();
  long long raw = 0;
  for (int a = 0; a < n_atoms; ++a) {
    const double rbs = bragg_slater_bohr(z[a]);
    const int nr = n_rad[a] > 0 ? n_rad[a] : std::max(radial_count(z[a], 2), 99);
    const double m = (double)(nr + 1);
    for (int i = 1; i <= nr; ++i) {
      const double t = (double)i, mt = m - t;
      RadialShell rs;
      rs.atom = a;
      rs.r = rbs * (t * t) / (mt * mt);
      rs.w_rad = 2.0 * ipow(rbs, 3) * m * ipow(t, 5) / ipow(mt, 7);
      const double x = rs.r / std::max(rbs, 0.3);
      if (x_max[a] > 0.0 && x > x_max[a]) continue;
      const int k = x < 0.18 ? 0 : x < 0.50 ? 1 : x < 0.95 ? 2 : x < 5.00 ? 3 : 4;
      const int want = region_leb[5 * a + k] > 0 ? region_leb[5 * a + k] : kFineRegion[k];
      const int li = lebedev_index(want);
      rs.leb_offset = T.offset[li];
      rs.n_ang = T.count[li];
      rs.raw_start = raw;
      raw += rs.n_ang;
      out.push_back(rs);
    }
  }
  *n_raw = raw;
}

void becke_tables(int n, const int* z, const double* xyz, std::vector<double>& inv_r, std::vector<double>& a_ij) {
  inv_r.assign((size_t)n * n, 0.0);
  a_ij.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
                   dz = xyz[3 * i + 2] - xyz[3 * j + 2];
      const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
      const double inv = r >= 1e-14 ? 1.0 / r : 0.0;
      const double a = becke_shift(z[i], z[j]);
      inv_r[(size_t)i * n + j] = inv;
      inv_r[(size_t)j * n + i] = inv;
      a_ij[(size_t)i * n + j] = a;
      a_ij[(size_t)j * n + i] = -a;
    }
}

// Candidate shells of one batch (points xyzw[4 idx[k]..], k < n) by the reference's rule
// (vxc.rs:449-489): the shells whose cut-off sphere meets the bounding sphere of the batch's box.
// With `reach`, only those with r^2 <= r2_cutoff (1 + 1e-6) at one point at least are kept: the
// others give exact zeros at every point of the batch (the kernels test r^2 > r2_cutoff per point;
// the margin covers their FP32 form of that test).
// Whether a bound on |phi| and |grad phi| of one of shell s's components reaches `floor` at one of the
// points at least.  With R0 = sum_p w_p exp(-a_p r^2), R1 = -2 sum_p a_p w_p exp(-a_p r^2), l the
// shell's angular momentum and S the largest component scale: |x^i y^j z^k| <= r^l, so
// |phi| <= S r^l sum |w_p| e_p and |d phi / dq| <= S (l r^(l-1) sum |w_p| e_p + 2 r^(l+1) sum a_p |w_p| e_p).
static bool shell_reaches_value(const AoShellGpu& sh, const AoPrimGpu* prims, const AoCompGpu* comps,
                                const double* xyzw, const int* idx, int n, double floor) {
  const int l = sh.n_funcs == 1 ? 0 : sh.n_funcs == 3 ? 1 : sh.n_funcs == 6 ? 2 : 3;
  double smax = 0.0;
  for (int c = 0; c < sh.n_funcs; ++c) smax = std::max(smax, std::fabs(comps[sh.comp_start + c].scale));
  for (int k = 0; k < n; ++k) {
    const double* p = xyzw + 4 * (size_t)idx[k];
    const double px = p[0] - sh.center[0], py = p[1] - sh.center[1], pz = p[2] - sh.center[2];
    const double r2 = px * px + py * py + pz * pz;
    double e0 = 0.0, e1 = 0.0;
    for (int q = 0; q < sh.n_prims; ++q) {
      const AoPrimGpu& pr = prims[sh.prim_start + q];
      const double e = std::fabs(pr.weighted_norm) * std::exp(-pr.exponent * r2);
      e0 += e;
      e1 += pr.exponent * e;
    }
    const double r = std::sqrt(r2);
    const double rl = l == 0 ? 1.0 : (l == 1 ? r : (l == 2 ? r2 : r2 * r));
    const double rl1 = l == 0 ? 0.0 : (l == 1 ? 1.0 : (l == 2 ? r : r2));  // r^(l-1)
    const double b0 = smax * rl * e0;
    const double b1 = smax * (l * rl1 * e0 + 2.0 * rl * r * e1);
    if (b0 >= floor || b1 >= floor) return true;
  }
  return false;
}

// valid: the shell's primitive and component ranges lie in the arrays (the upload rejects them
// otherwise, so the bound is not needed then).
static bool shell_ranges_ok(const AoShellGpu& sh, int n_prims, int n_comps) {
  return sh.n_prims >= 1 && sh.prim_start >= 0 && sh.prim_start + sh.n_prims <= n_prims && sh.n_funcs >= 1 &&
         sh.n_funcs <= 10 && sh.comp_start >= 0 && sh.comp_start + sh.n_funcs <= n_comps;
}

static void batch_candidates(const AoShellGpu* shells, int n_shells, const double* xyzw, const int* idx, int n,
                             bool reach, std::vector<int>& out, const ValueScreen* vs = nullptr) {
  out.clear();
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < n; ++k) {
    const double* p = xyzw + 4 * (size_t)idx[k];
    for (int q = 0; q < 3; ++q) {
      if (p[q] < mn[q]) mn[q] = p[q];
      if (p[q] > mx[q]) mx[q] = p[q];
    }
  }
  const double c[3] = {0.5 * (mn[0] + mx[0]), 0.5 * (mn[1] + mx[1]), 0.5 * (mn[2] + mx[2])};
  const double ex = mx[0] - c[0], ey = mx[1] - c[1], ez = mx[2] - c[2];
  const double rbox = std::sqrt(ex * ex + ey * ey + ez * ez);
  for (int s = 0; s < n_shells; ++s) {
    const double dx = shells[s].center[0] - c[0], dy = shells[s].center[1] - c[1], dz = shells[s].center[2] - c[2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    const double th = rbox + std::sqrt(shells[s].r2_cutoff);
    if (!(d2 <= th * th)) continue;
    if (reach) {
      const double lim = shells[s].r2_cutoff * (1.0 + 1e-6);
      bool hit = false;
      for (int k = 0; k < n && !hit; ++k) {
        const double* p = xyzw + 4 * (size_t)idx[k];
        const double px = p[0] - shells[s].center[0], py = p[1] - shells[s].center[1], pz = p[2] - shells[s].center[2];
        hit = px * px + py * py + pz * pz <= lim;
      }
      if (!hit) continue;
      if (vs && shell_ranges_ok(shells[s], vs->n_prims, vs->n_comps) &&
          !shell_reaches_value(shells[s], vs->prims, vs->comps, xyzw, idx, n, vs->floor))
        continue;
    }
    out.push_back(s);
  }
}

int plan_batches_spatial(const AoShellGpu* shells, int n_shells, const double* xyzw, int n_pts, Plan& plan,
                         int batch_pts, const ValueScreen* vs) {
  plan = Plan();
  std::vector<int> order;
  order.reserve(n_pts);
  for (int g = 0; g < n_pts; ++g)
    if (!(std::fabs(xyzw[4 * (size_t)g + 3]) < 1e-24)) order.push_back(g);
  // recursive bisection along the longest axis of each part's box; the lower part takes a multiple
  // of batch_pts points, so every leaf but the last of a part is a full batch
  std::vector<std::pair<int, int>> stack{{0, (int)order.size()}};
  std::vector<std::pair<int, int>> leaves;
  while (!stack.empty()) {
    const auto [lo, hi] = stack.back();
    stack.pop_back();
    const int len = hi - lo;
    if (len <= batch_pts) {
      if (len > 0) leaves.push_back({lo, hi});
      continue;
    }
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = lo; k < hi; ++k) {
      const double* p = xyzw + 4 * (size_t)order[k];
      for (int q = 0; q < 3; ++q) {
        if (p[q] < mn[q]) mn[q] = p[q];
        if (p[q] > mx[q]) mx[q] = p[q];
      }
    }
    int ax = 0;
    for (int q = 1; q < 3; ++q)
      if (mx[q] - mn[q] > mx[ax] - mn[ax]) ax = q;
    const int nl = len >= 2 * batch_pts ? (len / batch_pts / 2) * batch_pts : len / 2;
    auto key = [&](int a, int b) {
      const double ka = xyzw[4 * (size_t)a + ax], kb = xyzw[4 * (size_t)b + ax];
      return ka < kb || (ka == kb && a < b);  // total order: the same plan on every machine
    };
    std::nth_element(order.begin() + lo, order.begin() + lo + nl, order.begin() + hi, key);
    stack.push_back({lo + nl, hi});
    stack.push_back({lo, lo + nl});
  }
  const int nb = (int)leaves.size();
  std::vector<std::vector<int>> cand(nb);
#pragma omp parallel for schedule(dynamic, 16)
  for (int b = 0; b < nb; ++b)
    batch_candidates(shells, n_shells, xyzw, order.data() + leaves[b].first, leaves[b].second - leaves[b].first,
                     true, cand[b], vs);
  plan.cand_offsets.push_back(0);
  for (int b = 0; b < nb; ++b) {
    if (cand[b].empty()) continue;  // no AO reaches these points: they contribute nothing
    plan.cand_shells.insert(plan.cand_shells.end(), cand[b].begin(), cand[b].end());
    plan.cand_offsets.push_back((int)plan.cand_shells.size());
    for (int k = leaves[b].first; k < leaves[b].second; ++k) {
      const int g = order[k];
      const double* p = xyzw + 4 * (size_t)g;
      GridPtGpu gp;
      gp.x = p[0];
      gp.y = p[1];
      gp.z = p[2];
      gp.batch_id = (int)plan.cand_offsets.size() - 2;
      gp.host_atom = 0;
      plan.pts.push_back(gp);
      plan.weights.push_back(p[3]);
      plan.orig.push_back(g);
    }
  }
  return 0;
}

int plan_batches(const AoShellGpu* shells, int n_shells, const double* xyzw, int n_pts, Plan& plan, int batch_pts) {
  plan = Plan();
  std::vector<int> keep;
  keep.reserve(batch_pts);
  for (int s0 = 0; s0 < n_pts; s0 += batch_pts) {
    const int len = std::min(batch_pts, n_pts - s0);
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    keep.clear();
    for (int g = 0; g < len; ++g) {
      const double* p = xyzw + 4 * (size_t)(s0 + g);
      if (std::fabs(p[3]) < 1e-24) continue;
      keep.push_back(s0 + g);
      for (int q = 0; q < 3; ++q) {
        if (p[q] < mn[q]) mn[q] = p[q];
        if (p[q] > mx[q]) mx[q] = p[q];
      }
    }
    if (keep.empty()) continue;
    const double c[3] = {0.5 * (mn[0] + mx[0]), 0.5 * (mn[1] + mx[1]), 0.5 * (mn[2] + mx[2])};
    const double ex = mx[0] - c[0], ey = mx[1] - c[1], ez = mx[2] - c[2];
    const double rbox = std::sqrt(ex * ex + ey * ey + ez * ez);
    const size_t cand0 = plan.cand_shells.size();
    for (int s = 0; s < n_shells; ++s) {
      const double dx = shells[s].center[0] - c[0], dy = shells[s].center[1] - c[1], dz = shells[s].center[2] - c[2];
      const double d2 = dx * dx + dy * dy + dz * dz;
      const double th = rbox + std::sqrt(shells[s].r2_cutoff);
      if (d2 <= th * th) plan.cand_shells.push_back(s);
    }
    if (plan.cand_shells.size() == cand0) continue;
    const int bid = (int)plan.cand_offsets.size();
    if (bid == 0) plan.cand_offsets.push_back(0);
    plan.cand_offsets.push_back((int)plan.cand_shells.size());
    for (int g : keep) {
      const double* p = xyzw + 4 * (size_t)g;
      GridPtGpu gp;
      gp.x = p[0];
      gp.y = p[1];
      gp.z = p[2];
      gp.batch_id = (int)plan.cand_offsets.size() - 2;
      gp.host_atom = 0;
      plan.pts.push_back(gp);
      plan.weights.push_back(p[3]);
      plan.orig.push_back(g);
    }
  }
  if (plan.cand_offsets.empty()) plan.cand_offsets.push_back(0);
  return 0;
}

}  // namespace cxc
