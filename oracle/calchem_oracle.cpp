// calchem_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// FP64 CPU restatement of CalChem's DFT exchange-correlation quadrature, used
// as the checker for the GPU implementation in calchem_gb300 and as the timed
// CPU baseline ("restated reference CPU algorithm").  Nothing in the product
// path links or calls this file.
//
// Each function cites the CalChem source it restates (paths are relative to the
// CalChem repository root).  CalChem's Rust workspace cannot be built offline
// (its crates are not vendored), so parity with the reference is pinned only by
// the reference's own known-answer tests (Lebedev exactness, analytic Gaussian
// integrals, finite-difference derivative checks), which tests/ re-run against
// this oracle.  No absolute Exc/Vxc value is published by the reference.
//
// Compiled with -ffp-contract=off so that a*b+c is not fused: Rust does not
// contract floating-point expressions either.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {
// cpu_gemm.cpp: the register-blocked FMA product of the timed CPU baseline.
void gemm_acc(int M, int N, int K, const double* A, long ars, long acs, const double* B, long ldb, double* C,
              long ldc);
}  // namespace orc

namespace {

constexpr double kPi = 3.14159265358979323846;          // std::f64::consts::PI
constexpr double kAngToBohr = 1.8897261245650618;       // calchem-model/src/lib.rs:4
constexpr double kRhoCutoff = 1e-18;                    // xc.rs:13
constexpr double kDensityScreen = 1e-18;                // vxc.rs:23
constexpr int kBatch = 128;                             // vxc.rs:96
constexpr int kGridChunk = 256;                         // vxc.rs:22

// compiler-rt __powidf2 order of multiplications, which is what Rust's f64::powi lowers to.
inline double powi(double a, int b) {
  const bool recip = b < 0;
  double r = 1.0;
  while (true) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

inline double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

// ============================================================================
// Lebedev-Laikov rules (crates/calchem-dft/src/lebedev.rs:69-247)
// ============================================================================
struct Quad { double x, y, z, w; };

void push_octant(std::vector<Quad>& out, double x, double y, double z, double w) {
  // lebedev.rs:69-77
  for (double sx : {-1.0, 1.0})
    for (double sy : {-1.0, 1.0})
      for (double sz : {-1.0, 1.0}) out.push_back({sx * x, sy * y, sz * z, w});
}

void push_orbit(std::vector<Quad>& out, int kind, double a, double b, double v) {
  // lebedev.rs:79-142
  const double w = 4.0 * kPi * v;
  switch (kind) {
    case 1:
      for (double s : {-1.0, 1.0}) {
        out.push_back({s, 0.0, 0.0, w});
        out.push_back({0.0, s, 0.0, w});
        out.push_back({0.0, 0.0, s, w});
      }
      break;
    case 2: {
      const double s = std::sqrt(0.5);
      for (double s1 : {-s, s})
        for (double s2 : {-s, s}) {
          out.push_back({s1, s2, 0.0, w});
          out.push_back({s1, 0.0, s2, w});
          out.push_back({0.0, s1, s2, w});
        }
      break;
    }
    case 3: {
      const double s = std::sqrt(1.0 / 3.0);
      push_octant(out, s, s, s, w);
      break;
    }
    case 4: {
      const double m = std::sqrt(1.0 - 2.0 * a * a);
      push_octant(out, a, a, m, w);
      push_octant(out, a, m, a, w);
      push_octant(out, m, a, a, w);
      break;
    }
    case 5: {
      const double q = std::sqrt(1.0 - a * a);
      const double ut[2][2] = {{a, q}, {q, a}};
      for (auto& p : ut)
        for (double su : {-1.0, 1.0})
          for (double st : {-1.0, 1.0}) {
            out.push_back({su * p[0], st * p[1], 0.0, w});
            out.push_back({su * p[0], 0.0, st * p[1], w});
            out.push_back({0.0, su * p[0], st * p[1], w});
          }
      break;
    }
    case 6: {
      const double c = std::sqrt(1.0 - a * a - b * b);
      const double perms[6][3] = {{a, b, c}, {b, a, c}, {c, a, b}, {a, c, b}, {c, b, a}, {b, c, a}};
      for (auto& p : perms) push_octant(out, p[0], p[1], p[2], w);
      break;
    }
  }
}

std::vector<Quad> build_lebedev(int n) {
  // lebedev.rs:144-247; published Lebedev-Laikov (1999) orbit parameters.
  std::vector<Quad> o;
  switch (n) {
    case 26:
      push_orbit(o, 1, 0, 0, 0.4761904761904762e-1);
      push_orbit(o, 2, 0, 0, 0.3809523809523810e-1);
      push_orbit(o, 3, 0, 0, 0.3214285714285714e-1);
      break;
    case 50:
      push_orbit(o, 1, 0, 0, 0.1269841269841270e-1);
      push_orbit(o, 2, 0, 0, 0.2257495590828924e-1);
      push_orbit(o, 3, 0, 0, 0.2109375000000000e-1);
      push_orbit(o, 4, 0.3015113445777636, 0, 0.2017333553791887e-1);
      break;
    case 110:
      push_orbit(o, 1, 0, 0, 0.3828270494937162e-2);
      push_orbit(o, 3, 0, 0, 0.9793737512487512e-2);
      push_orbit(o, 4, 0.1851156353447362, 0, 0.8211737283191111e-2);
      push_orbit(o, 4, 0.6904210483822922, 0, 0.9942814891178103e-2);
      push_orbit(o, 4, 0.3956894730559419, 0, 0.9595471336070963e-2);
      push_orbit(o, 5, 0.4783690288121502, 0, 0.9694996361663028e-2);
      break;
    case 194:
      push_orbit(o, 1, 0, 0, 0.1782340447244611e-2);
      push_orbit(o, 2, 0, 0, 0.5716905949977102e-2);
      push_orbit(o, 3, 0, 0, 0.5573383178848738e-2);
      push_orbit(o, 4, 0.6712973442695226, 0, 0.5608704082587997e-2);
      push_orbit(o, 4, 0.2892465627575439, 0, 0.5158237711805383e-2);
      push_orbit(o, 4, 0.4446933178717437, 0, 0.5518771467273614e-2);
      push_orbit(o, 4, 0.1299335447650067, 0, 0.4106777028169394e-2);
      push_orbit(o, 5, 0.3457702197611283, 0, 0.5051846064614808e-2);
      push_orbit(o, 6, 0.1590417105383530, 0.8360360154824589, 0.5530248916233094e-2);
      break;
    case 302:
      push_orbit(o, 1, 0, 0, 0.8545911725128148e-3);
      push_orbit(o, 3, 0, 0, 0.3599119285025571e-2);
      push_orbit(o, 4, 0.3515640345570105, 0, 0.3449788424305883e-2);
      push_orbit(o, 4, 0.6566329410219612, 0, 0.3604822601419882e-2);
      push_orbit(o, 4, 0.4729054132581005, 0, 0.3576729661743367e-2);
      push_orbit(o, 4, 0.9618308522614784e-1, 0, 0.2352101413689164e-2);
      push_orbit(o, 4, 0.2219645236294178, 0, 0.3108953122413675e-2);
      push_orbit(o, 4, 0.7011766416089545, 0, 0.3650045807677255e-2);
      push_orbit(o, 5, 0.2644152887060663, 0, 0.2982344963171804e-2);
      push_orbit(o, 5, 0.5718955891878961, 0, 0.3600820932216460e-2);
      push_orbit(o, 6, 0.2510034751770465, 0.8000727494073952, 0.3571540554273387e-2);
      push_orbit(o, 6, 0.1233548532583327, 0.4127724083168531, 0.3392312205006170e-2);
      break;
    case 590: {
      push_orbit(o, 1, 0, 0, 0.3095121295306187e-3);
      push_orbit(o, 3, 0, 0, 0.1852379698597489e-2);
      const double b4[9][2] = {{0.7040954938227469, 0.1871790639277744e-2},
                               {0.6807744066455243, 0.1858812585438317e-2},
                               {0.6372546939258752, 0.1852028828296213e-2},
                               {0.5044419707800358, 0.1846715956151242e-2},
                               {0.4215761784010967, 0.1818471778162769e-2},
                               {0.3317920736472123, 0.1749564657281154e-2},
                               {0.2384736701421887, 0.1617210647254411e-2},
                               {0.1459036449157763, 0.1384737234851692e-2},
                               {0.06095034115507196, 0.9764331165051050e-3}};
      for (auto& p : b4) push_orbit(o, 4, p[0], 0, p[1]);
      const double c5[3][2] = {{0.6116843442009876, 0.1857161196774078e-2},
                               {0.3964755348199858, 0.1705153996395864e-2},
                               {0.1724782009907724, 0.1300321685886048e-2}};
      for (auto& p : c5) push_orbit(o, 5, p[0], 0, p[1]);
      const double d6[6][3] = {{0.5610263808622060, 0.3518280927733519, 0.1842866472905286e-2},
                               {0.4742392842551980, 0.2634716655937950, 0.1802658934377451e-2},
                               {0.5984126497885380, 0.1816640840360209, 0.1849830560443660e-2},
                               {0.3791035407695563, 0.1720795225656878, 0.1713904507106709e-2},
                               {0.2778673190586244, 0.08213021581932511, 0.1555213603396808e-2},
                               {0.5033564271075117, 0.08999205842074875, 0.1802239128008525e-2}};
      for (auto& p : d6) push_orbit(o, 6, p[0], p[1], p[2]);
      break;
    }
    default:
      break;
  }
  return o;
}

const std::vector<Quad>& lebedev(int n) {
  static std::once_flag flags[6];
  static std::vector<Quad> rules[6];
  int idx = n == 26 ? 0 : n == 50 ? 1 : n == 110 ? 2 : n == 194 ? 3 : n == 302 ? 4 : 5;
  std::call_once(flags[idx], [&] { rules[idx] = build_lebedev(n); });
  return rules[idx];
}

// ============================================================================
// Molecular grid (crates/calchem-dft/src/grid.rs)
// ============================================================================
enum Level { kCoarse = 0, kMedium = 1, kFine = 2, kUltraFine = 3 };

double bragg_slater_radius_bohr(int z) {
  // grid.rs:58-101
  double a;
  if (z == 1 || z == 2) a = 0.35;
  else if (z == 3) a = 1.45;
  else if (z == 4) a = 1.05;
  else if (z == 5) a = 0.85;
  else if (z == 6) a = 0.70;
  else if (z == 7) a = 0.65;
  else if (z == 8) a = 0.60;
  else if (z == 9) a = 0.50;
  else if (z == 10) a = 0.45;
  else if (z == 11) a = 1.80;
  else if (z == 12) a = 1.50;
  else if (z == 13) a = 1.25;
  else if (z == 14) a = 1.10;
  else if (z == 15) a = 1.00;
  else if (z >= 16 && z <= 18) a = 1.00;
  else if (z == 19) a = 2.20;
  else if (z == 20) a = 1.80;
  else if (z >= 21 && z <= 30) a = 1.40;
  else if (z == 31) a = 1.30;
  else if (z == 32) a = 1.25;
  else if (z >= 33 && z <= 35) a = 1.15;
  else if (z == 36) a = 1.10;
  else if (z == 37) a = 2.35;
  else if (z == 38) a = 2.00;
  else if (z >= 39 && z <= 49) a = 1.55;
  else if (z == 50 || z == 51) a = 1.45;
  else if (z == 52 || z == 53) a = 1.40;
  else if (z == 54) a = 1.35;
  else if (z == 55) a = 2.60;
  else if (z == 56) a = 2.15;
  else a = 1.75;
  return a * kAngToBohr;
}

double becke_asymmetry(int zc, int zd) {
  // grid.rs:105-115
  if (zc == zd) return 0.0;
  const double rc = bragg_slater_radius_bohr(zc), rd = bragg_slater_radius_bohr(zd);
  const double chi = rc / rd;
  const double u = (chi - 1.0) / (chi + 1.0);
  const double a = u / (u * u - 1.0);
  return clampd(a, -0.5, 0.5);
}

int radial_shell_count(int z, int level) {
  // grid.rs:142-173
  switch (level) {
    case kCoarse: return z <= 2 ? 25 : (z <= 18 ? 35 : 45);
    case kMedium: return z <= 2 ? 35 : (z <= 18 ? 50 : 65);
    case kFine: return z <= 2 ? 55 : (z <= 18 ? 75 : 90);
    default: return 200;
  }
}

int pruned_angular_points(double r, double r_bs, int level) {
  // grid.rs:176-220
  const double ratio = r / std::max(r_bs, 0.3);
  switch (level) {
    case kCoarse:
      return ratio < 0.25 ? 26 : ratio < 0.75 ? 50 : ratio < 4.5 ? 110 : 50;
    case kMedium:
      return ratio < 0.20 ? 26 : ratio < 0.55 ? 50 : ratio < 1.10 ? 110 : ratio < 4.50 ? 194 : 110;
    case kFine:
      return ratio < 0.18 ? 50 : ratio < 0.50 ? 110 : ratio < 0.95 ? 194 : ratio < 5.00 ? 302 : 194;
    default:
      return 590;
  }
}

struct BeckeTable {
  // grid.rs:268-318
  int n = 0;
  std::vector<double> coords, inv_rij, a_ij;
  BeckeTable(int n_atoms, const int* z, const double* xyz) : n(n_atoms) {
    coords.assign(xyz, xyz + 3 * n);
    inv_rij.assign((size_t)n * n, 0.0);
    a_ij.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) {
        const double dx = coords[3 * i] - coords[3 * j];
        const double dy = coords[3 * i + 1] - coords[3 * j + 1];
        const double dz = coords[3 * i + 2] - coords[3 * j + 2];
        const double rij = std::sqrt(dx * dx + dy * dy + dz * dz);
        const double inv = rij >= 1e-14 ? 1.0 / rij : 0.0;
        const double a = becke_asymmetry(z[i], z[j]);
        inv_rij[(size_t)i * n + j] = inv;
        inv_rij[(size_t)j * n + i] = inv;
        a_ij[(size_t)i * n + j] = a;
        a_ij[(size_t)j * n + i] = -a;
      }
  }
};

inline double becke_step_fast(double nu) {
  // grid.rs:320-332
  if (nu <= -1.0) return 1.0;
  if (nu >= 1.0) return 0.0;
  const double f1 = 0.5 * nu * (3.0 - nu * nu);
  const double f2 = 0.5 * f1 * (3.0 - f1 * f1);
  const double f3 = 0.5 * f2 * (3.0 - f2 * f2);
  return 0.5 * (1.0 - f3);
}

double becke_weight_fast(const BeckeTable& t, std::vector<double>& dist, std::vector<double>& s_hb,
                         std::vector<int>& active, int host, const double r[3]) {
  // grid.rs:338-419 (two-pass screened Becke partition)
  const int n = t.n;
  if (n <= 1) return 1.0;
  for (int a = 0; a < n; ++a) {
    const double dx = r[0] - t.coords[3 * a], dy = r[1] - t.coords[3 * a + 1], dz = r[2] - t.coords[3 * a + 2];
    dist[a] = std::sqrt(dx * dx + dy * dy + dz * dz);
  }
  const double r_host = dist[host];
  const size_t row_host = (size_t)host * n;
  double p_host = 1.0;
  active.clear();
  for (int b = 0; b < n; ++b) {
    if (b == host) continue;
    const double inv_r = t.inv_rij[row_host + b];
    if (inv_r == 0.0) continue;
    const double mu = clampd((r_host - dist[b]) * inv_r, -1.0, 1.0);
    const double a_hb = t.a_ij[row_host + b];
    const double nu = mu + a_hb * (1.0 - mu * mu);
    const double s = becke_step_fast(nu);
    p_host *= s;
    if (p_host < 1e-20) return 0.0;
    s_hb[b] = s;
    if (1.0 - s > 1e-17) active.push_back(b);
  }
  if (active.empty()) return 1.0;
  double sum_p = p_host;
  for (int a : active) {
    const double r_a = dist[a];
    const size_t row_a = (size_t)a * n;
    double p_a = 1.0 - s_hb[a];
    if (p_a < 1e-20) continue;
    for (int b = 0; b < n; ++b) {
      if (b == host || b == a) continue;
      const double inv_r = t.inv_rij[row_a + b];
      if (inv_r == 0.0) continue;
      const double mu = clampd((r_a - dist[b]) * inv_r, -1.0, 1.0);
      const double nu = mu + t.a_ij[row_a + b] * (1.0 - mu * mu);
      p_a *= becke_step_fast(nu);
      if (p_a < 1e-20) break;
    }
    sum_p += p_a;
  }
  return sum_p <= 0.0 ? 0.0 : p_host / sum_p;
}

struct GridPoint { double x, y, z, w, raw_w; int host; };

void generate_atom_points(int n_atoms, const int* z, const double* xyz, const BeckeTable& table,
                          int level, int radial_min, int atom, std::vector<GridPoint>& out) {
  // grid.rs:732-782
  const double r_bs = bragg_slater_radius_bohr(z[atom]);
  const int base_min = level == kFine ? 99 : 0;
  const int n_rad = std::max(std::max(radial_shell_count(z[atom], level), radial_min), base_min);
  const double m = (double)(n_rad + 1);
  std::vector<double> dist(n_atoms), s_hb(n_atoms);
  std::vector<int> active;
  active.reserve(n_atoms);
  for (int i = 1; i <= n_rad; ++i) {
    const double t = (double)i;
    const double mt = m - t;
    const double r = r_bs * (t * t) / (mt * mt);
    const double w_rad = 2.0 * powi(r_bs, 3) * m * powi(t, 5) / powi(mt, 7);
    const auto& ang = lebedev(pruned_angular_points(r, r_bs, level));
    for (const Quad& q : ang) {
      const double raw_w = w_rad * q.w;
      double c[3] = {xyz[3 * atom] + r * q.x, xyz[3 * atom + 1] + r * q.y, xyz[3 * atom + 2] + r * q.z};
      const double bw = becke_weight_fast(table, dist, s_hb, active, atom, c);
      const double w_tot = raw_w * bw;
      if (w_tot > 1e-18) out.push_back({c[0], c[1], c[2], w_tot, raw_w, atom});
    }
  }
}

std::vector<GridPoint> build_grid(int n_atoms, const int* z, const double* xyz, int level, int radial_min) {
  // grid.rs:784-828 (atom-major concatenation of the per-atom point lists)
  BeckeTable table(n_atoms, z, xyz);
  std::vector<std::vector<GridPoint>> per_atom(n_atoms);
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < n_atoms; ++a) generate_atom_points(n_atoms, z, xyz, table, level, radial_min, a, per_atom[a]);
  std::vector<GridPoint> pts;
  for (auto& v : per_atom) pts.insert(pts.end(), v.begin(), v.end());
  return pts;
}

// ============================================================================
// Basis normalisation (crates/calchem-basis/src/normalization.rs, lib.rs:462-573)
// ============================================================================
double dfact_odd(int k) {
  // normalization.rs:5-16
  if (k <= 0) return 1.0;
  double acc = 1.0;
  while (k > 0) { acc *= (double)k; k -= 2; }
  return acc;
}

double primitive_norm(double alpha, int l, int m, int n) {
  // normalization.rs:20-29
  const int lt = l + m + n;
  const double radial = std::pow(2.0 * alpha / kPi, 0.75);
  const double num = powi(4.0 * alpha, lt);
  const double den = dfact_odd(2 * l - 1) * dfact_odd(2 * m - 1) * dfact_odd(2 * n - 1);
  return radial * std::sqrt(num / den);
}

double self_overlap_norm(double ai, double aj, int l, int m, int n) {
  // normalization.rs:33-50
  const double g = ai + aj;
  const double ni = primitive_norm(ai, l, m, n), nj = primitive_norm(aj, l, m, n);
  const double radial = std::pow(kPi / g, 1.5);
  double ang = 1.0;
  if (l > 0) ang *= dfact_odd(2 * l - 1) / powi(2.0 * g, l);
  if (m > 0) ang *= dfact_odd(2 * m - 1) / powi(2.0 * g, m);
  if (n > 0) ang *= dfact_odd(2 * n - 1) / powi(2.0 * g, n);
  return ni * nj * radial * ang;
}

// Cartesian component order (calchem-basis/src/lib.rs:135-160)
const int kComps[4][10][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}},
    {{3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {1, 1, 1}, {1, 0, 2}, {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}}};
const int kNComp[4] = {1, 3, 6, 10};

struct Shell {
  int l = 0, atom = 0, ao_offset = 0;
  double center[3];
  std::vector<double> exps, coeffs, norms;  // contraction-normalised coeff, axial primitive norm
  // ao_grid.rs:28-71 (PrecomputedAoShell)
  double r2_cut = 0, r_cut = 0;
  std::vector<double> wnorm;        // coeff * norm
  double comp_scale[10];
  int ncomp() const { return kNComp[l]; }
};

struct Basis {
  int n_ao = 0;
  std::vector<Shell> shells;
};

Basis make_basis(int n_shells, const int* ls, const int* atoms, const double* centers, const int* nprims,
                 const double* exps, const double* coefs) {
  Basis b;
  size_t p = 0;
  for (int s = 0; s < n_shells; ++s) {
    Shell sh;
    sh.l = ls[s];
    sh.atom = atoms[s];
    for (int q = 0; q < 3; ++q) sh.center[q] = centers[3 * s + q];
    const int np = nprims[s];
    sh.exps.assign(exps + p, exps + p + np);
    std::vector<double> raw(coefs + p, coefs + p + np);
    p += np;
    // normalized_contraction (normalization.rs:59-97) with rep_lmn = (L,0,0)
    double so = 0.0;
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) so += raw[i] * raw[j] * self_overlap_norm(sh.exps[i], sh.exps[j], sh.l, 0, 0);
    const double scale = 1.0 / std::sqrt(so);
    sh.coeffs.resize(np);
    sh.norms.resize(np);
    sh.wnorm.resize(np);
    double amin = INFINITY;
    for (int i = 0; i < np; ++i) {
      sh.coeffs[i] = raw[i] * scale;
      sh.norms[i] = primitive_norm(sh.exps[i], sh.l, 0, 0);
      sh.wnorm[i] = sh.coeffs[i] * sh.norms[i];
      amin = std::min(amin, sh.exps[i]);
    }
    amin = std::max(amin, 1e-12);
    sh.r2_cut = (40.0 + 4.0 * sh.l) / amin;
    sh.r_cut = std::sqrt(sh.r2_cut);
    const double lead = sh.norms[0];
    for (int c = 0; c < sh.ncomp(); ++c) {
      const int* lmn = kComps[sh.l][c];
      sh.comp_scale[c] = lead == 0.0 ? 1.0 : primitive_norm(sh.exps[0], lmn[0], lmn[1], lmn[2]) / lead;
    }
    sh.ao_offset = b.n_ao;
    b.n_ao += sh.ncomp();
    b.shells.push_back(std::move(sh));
  }
  return b;
}

// ============================================================================
// AO values and gradients (crates/calchem-dft/src/ao_grid.rs:80-299)
// ============================================================================
inline void pow012(double x, int l, double& p, double& d1, double& d2) {
  // ao_grid.rs:80-95
  switch (l) {
    case 0: p = 1.0; d1 = 0.0; d2 = 0.0; break;
    case 1: p = x; d1 = 1.0; d2 = 0.0; break;
    case 2: p = x * x; d1 = 2.0 * x; d2 = 2.0; break;
    case 3: p = x * x * x; d1 = 3.0 * x * x; d2 = 6.0 * x; break;
    default: {
      const double lf = l;
      p = powi(x, l); d1 = lf * powi(x, l - 1); d2 = lf * (lf - 1.0) * powi(x, l - 2);
    }
  }
}

struct AoVal { int mu; double v, gx, gy, gz; };

// eval_aos_grad_filtered (ao_grid.rs:182-230)
void eval_aos_grad(const Basis& bs, const std::vector<int>& shells, const double r[3], std::vector<AoVal>& out) {
  out.clear();
  for (int si : shells) {
    const Shell& sh = bs.shells[si];
    const double dx = r[0] - sh.center[0], dy = r[1] - sh.center[1], dz = r[2] - sh.center[2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > sh.r2_cut) continue;
    double r0 = 0.0, r1 = 0.0;
    for (size_t p = 0; p < sh.exps.size(); ++p) {
      const double e = sh.wnorm[p] * std::exp(-sh.exps[p] * r2);
      r0 += e;
      r1 -= 2.0 * sh.exps[p] * e;
    }
    if (std::fabs(r0) < 1e-18 && std::fabs(r1) < 1e-18) continue;
    for (int c = 0; c < sh.ncomp(); ++c) {
      const int* lmn = kComps[sh.l][c];
      const double scale = sh.comp_scale[c];
      double px, dpx, t, py, dpy, pz, dpz;
      pow012(dx, lmn[0], px, dpx, t);
      pow012(dy, lmn[1], py, dpy, t);
      pow012(dz, lmn[2], pz, dpz, t);
      const double m = px * py * pz;
      const double val = scale * m * r0;
      const double gx = scale * (dpx * py * pz * r0 + m * dx * r1);
      const double gy = scale * (px * dpy * pz * r0 + m * dy * r1);
      const double gz = scale * (px * py * dpz * r0 + m * dz * r1);
      if (std::fabs(val) > 1e-16 || std::fabs(gx) > 1e-16 || std::fabs(gy) > 1e-16 || std::fabs(gz) > 1e-16)
        out.push_back({sh.ao_offset + c, val, gx, gy, gz});
    }
  }
}

// eval_aos_hess (ao_grid.rs:234-299); out10 = [val, gx, gy, gz, hxx, hxy, hxz, hyy, hyz, hzz] per AO
void eval_aos_hess_all(const Basis& bs, const double r[3], double* out10) {
  std::memset(out10, 0, sizeof(double) * 10 * bs.n_ao);
  for (const Shell& sh : bs.shells) {
    const double dx = r[0] - sh.center[0], dy = r[1] - sh.center[1], dz = r[2] - sh.center[2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > sh.r2_cut) continue;
    double r0 = 0, r1 = 0, r2r = 0;
    for (size_t p = 0; p < sh.exps.size(); ++p) {
      const double e = sh.wnorm[p] * std::exp(-sh.exps[p] * r2);
      r0 += e;
      r1 -= 2.0 * sh.exps[p] * e;
      r2r += 4.0 * sh.exps[p] * sh.exps[p] * e;
    }
    if (std::fabs(r0) < 1e-18 && std::fabs(r1) < 1e-18 && std::fabs(r2r) < 1e-18) continue;
    for (int c = 0; c < sh.ncomp(); ++c) {
      const int* lmn = kComps[sh.l][c];
      const double s = sh.comp_scale[c];
      double px, dpx, d2px, py, dpy, d2py, pz, dpz, d2pz;
      pow012(dx, lmn[0], px, dpx, d2px);
      pow012(dy, lmn[1], py, dpy, d2py);
      pow012(dz, lmn[2], pz, dpz, d2pz);
      const double m = px * py * pz;
      const double dm[3] = {dpx * py * pz, px * dpy * pz, px * py * dpz};
      double* o = out10 + 10 * (sh.ao_offset + c);
      o[0] = s * m * r0;
      o[1] = s * (dm[0] * r0 + m * dx * r1);
      o[2] = s * (dm[1] * r0 + m * dy * r1);
      o[3] = s * (dm[2] * r0 + m * dz * r1);
      o[4] = s * (d2px * py * pz * r0 + (2.0 * dm[0] * dx + m) * r1 + m * dx * dx * r2r);
      o[5] = s * (dpx * dpy * pz * r0 + (dm[0] * dy + dm[1] * dx) * r1 + m * dx * dy * r2r);
      o[6] = s * (dpx * py * dpz * r0 + (dm[0] * dz + dm[2] * dx) * r1 + m * dx * dz * r2r);
      o[7] = s * (px * d2py * pz * r0 + (2.0 * dm[1] * dy + m) * r1 + m * dy * dy * r2r);
      o[8] = s * (px * dpy * dpz * r0 + (dm[1] * dz + dm[2] * dy) * r1 + m * dy * dz * r2r);
      o[9] = s * (px * py * d2pz * r0 + (2.0 * dm[2] * dz + m) * r1 + m * dz * dz * r2r);
    }
  }
}

// ============================================================================
// XC functionals (crates/calchem-dft/src/xc.rs:136-828)
// ============================================================================
struct XcOut {
  double f = 0, vra = 0, vrb = 0, vgaa = 0, vgab = 0, vgbb = 0;
  void add(double s, const XcOut& o) {
    f += s * o.f; vra += s * o.vra; vrb += s * o.vrb;
    vgaa += s * o.vgaa; vgab += s * o.vgab; vgbb += s * o.vgbb;
  }
};

void slater_one(double rs, double& f, double& v) {
  // xc.rs:233-243
  if (rs < kRhoCutoff) { f = 0; v = 0; return; }
  const double cx = 0.75 * std::pow(6.0 / kPi, 1.0 / 3.0);
  const double r13 = std::cbrt(rs);
  f = -cx * rs * r13;
  v = -(4.0 / 3.0) * cx * r13;
}

XcOut slater_x(double ra, double rb) {
  // xc.rs:245-251
  XcOut o;
  double fa, va, fb, vb;
  slater_one(ra, fa, va);
  slater_one(rb, fb, vb);
  o.f = fa + fb; o.vra = va; o.vrb = vb;
  return o;
}

struct VwnCh { double a, x0, b, c; };
struct VwnParams { VwnCh para, ferro, stiff; };
// xc.rs:270-334
const VwnParams kVwn5 = {{0.0310907, -0.10498, 3.72744, 12.9352},
                         {0.01554535, -0.32500, 7.06042, 18.0578},
                         {-0.016886863940389905, -0.00475840, 1.13107, 13.0045}};
const VwnParams kVwnRpa = {{0.0310907, -0.409286, 13.0720, 42.7198},
                           {0.01554535, -0.743294, 20.1231, 101.578},
                           {-0.016886863940389905, -0.228344, 1.06835, 11.4813}};

void vwn_channel(double x, const VwnCh& ch, double& eps, double& rs_deps) {
  // xc.rs:337-352
  const double xx = x * x + ch.b * x + ch.c;
  const double xx0 = ch.x0 * ch.x0 + ch.b * ch.x0 + ch.c;
  const double q = std::sqrt(4.0 * ch.c - ch.b * ch.b);
  const double at = std::atan(q / (2.0 * x + ch.b));
  const double xm = x - ch.x0;
  eps = ch.a * (std::log(x * x / xx) + (2.0 * ch.b / q) * at -
                (ch.b * ch.x0 / xx0) * (std::log(xm * xm / xx) + (2.0 * (ch.b + 2.0 * ch.x0) / q) * at));
  rs_deps = ch.a * (ch.c * xm - ch.b * x * ch.x0) / (xm * xx);
}

void spin_interp(double zeta, double& fz, double& dfz, double& fdd0) {
  // xc.rs:355-366
  const double c2 = std::cbrt(2.0) - 1.0;
  const double denom = 2.0 * c2;
  fdd0 = 4.0 / (9.0 * c2);
  const double zp = std::max(1.0 + zeta, 0.0), zm = std::max(1.0 - zeta, 0.0);
  const double zp13 = std::cbrt(zp), zm13 = std::cbrt(zm);
  fz = (zp * zp13 + zm * zm13 - 2.0) / denom;
  dfz = (4.0 / (3.0 * denom)) * (zp13 - zm13);
}

XcOut vwn_c(double ra, double rb, const VwnParams& P) {
  // xc.rs:369-404
  XcOut o;
  const double rho = ra + rb;
  if (rho < kRhoCutoff) return o;
  const double rs = std::cbrt(3.0 / (4.0 * kPi * rho));
  const double x = std::sqrt(rs);
  const double zeta = clampd((ra - rb) / rho, -1.0, 1.0);
  double ep, rdep, ef, rdef, ac, rdac;
  vwn_channel(x, P.para, ep, rdep);
  vwn_channel(x, P.ferro, ef, rdef);
  vwn_channel(x, P.stiff, ac, rdac);
  double fz, dfz, fdd0;
  spin_interp(zeta, fz, dfz, fdd0);
  const double z2 = zeta * zeta, z3 = z2 * zeta, z4 = z2 * z2, omz4 = 1.0 - z4;
  const double ifd = 1.0 / fdd0;
  const double dec = ef - ep, rddec = rdef - rdep;
  const double ec = ep + ac * fz * ifd * omz4 + dec * fz * z4;
  const double rs_dec = rdep + rdac * fz * ifd * omz4 + rddec * fz * z4;
  const double dec_dz = ac * ifd * (dfz * omz4 - 4.0 * z3 * fz) + dec * (dfz * z4 + 4.0 * z3 * fz);
  const double base = ec - (1.0 / 3.0) * rs_dec;
  o.f = rho * ec;
  o.vra = base + (1.0 - zeta) * dec_dz;
  o.vrb = base - (1.0 + zeta) * dec_dz;
  return o;
}

void b88_one(double rs, double g, double& f, double& vr, double& vg) {
  // xc.rs:410-436
  if (rs < kRhoCutoff) { f = vr = vg = 0; return; }
  const double beta = 0.0042;
  const double r13 = std::cbrt(rs), r43 = rs * r13;
  const double s2 = std::max(g, 0.0) / (r43 * r43);
  const double s = std::sqrt(s2);
  const double as = std::asinh(s);
  const double den = 1.0 + 6.0 * beta * s * as;
  const double gg = -beta * s2 / den;
  const double sq = std::sqrt(1.0 + s2);
  const double h = -beta * (2.0 + 6.0 * beta * s * as - 6.0 * beta * s2 / sq) / (den * den);
  f = r43 * gg;
  vr = (4.0 / 3.0) * r13 * (gg - s2 * h);
  vg = 0.5 * h / r43;
}

XcOut b88_x(double ra, double rb, double gaa, double gbb) {
  XcOut o;
  double fa, va, ga, fb, vb, gb;
  b88_one(ra, gaa, fa, va, ga);
  b88_one(rb, gbb, fb, vb, gb);
  o.f = fa + fb; o.vra = va; o.vrb = vb; o.vgaa = ga; o.vgbb = gb;
  return o;
}

void lyp_bracket(double ra, double rb, double delta, double ddelta, double gaa, double gab, double gbb,
                 double& s, double& ds, double& a_aa, double& a_ab, double& a_bb) {
  // xc.rs:433-501
  const double rho = ra + rb, rho2 = rho * rho;
  const double cf = 0.3 * std::pow(3.0 * kPi * kPi, 2.0 / 3.0);
  const double k0 = std::pow(2.0, 11.0 / 3.0) * cf;
  const double ra83 = ra > 0.0 ? std::pow(ra, 8.0 / 3.0) : 0.0;
  const double rb83 = rb > 0.0 ? std::pow(rb, 8.0 / 3.0) : 0.0;
  const double s_tf = k0 * ra * rb * (ra83 + rb83);
  const double ds_tf = k0 * ((11.0 / 3.0) * ra83 * rb + rb * rb83);
  const double cg = ra * rb * (47.0 - 7.0 * delta) / 18.0 - (2.0 / 3.0) * rho2;
  const double dcg = rb * (47.0 - 7.0 * delta) / 18.0 + ra * rb * (-7.0 * ddelta) / 18.0 - (4.0 / 3.0) * rho;
  const double qaa = ra * ra * rb / rho;
  const double dqaa = (2.0 * ra * rb * rho - ra * ra * rb) / rho2;
  const double eaa = -ra * rb * (2.5 - delta / 18.0) - ((delta - 11.0) / 9.0) * qaa + ((2.0 / 3.0) * rho2 - rb * rb);
  const double deaa = -rb * (2.5 - delta / 18.0) + ra * rb * (ddelta / 18.0) - (ddelta / 9.0) * qaa -
                      ((delta - 11.0) / 9.0) * dqaa + (4.0 / 3.0) * rho;
  const double qbb = ra * rb * rb / rho;
  const double dqbb = (rb * rb * rho - ra * rb * rb) / rho2;
  const double ebb = -ra * rb * (2.5 - delta / 18.0) - ((delta - 11.0) / 9.0) * qbb + ((2.0 / 3.0) * rho2 - ra * ra);
  const double debb = -rb * (2.5 - delta / 18.0) + ra * rb * (ddelta / 18.0) - (ddelta / 9.0) * qbb -
                      ((delta - 11.0) / 9.0) * dqbb + (4.0 / 3.0) * rho - 2.0 * ra;
  a_aa = cg + eaa;
  a_ab = 2.0 * cg;
  a_bb = cg + ebb;
  s = s_tf + a_aa * gaa + a_ab * gab + a_bb * gbb;
  ds = ds_tf + (dcg + deaa) * gaa + (2.0 * dcg) * gab + (dcg + debb) * gbb;
}

XcOut lyp_c(double ra, double rb, double gaa, double gab, double gbb) {
  // xc.rs:503-547
  XcOut o;
  const double rho = ra + rb;
  if (rho < kRhoCutoff) return o;
  const double A = 0.04918, B = 0.132, C = 0.2533, D = 0.349;
  const double r13 = std::pow(rho, -1.0 / 3.0);
  if (C * r13 > 500.0) {
    const double den = 1.0 + D * r13;
    const double g0 = -4.0 * A / (rho * den);
    const double dg0 = -g0 * (1.0 + (2.0 / 3.0) * D * r13) / (rho * den);
    o.f = g0 * ra * rb;
    o.vra = dg0 * ra * rb + g0 * rb;
    o.vrb = dg0 * ra * rb + g0 * ra;
    return o;
  }
  const double den = 1.0 + D * r13;
  const double g0 = -4.0 * A / (rho * den);
  const double dg0 = -g0 * (1.0 + (2.0 / 3.0) * D * r13) / (rho * den);
  const double t0 = g0 * ra * rb;
  const double dt0a = dg0 * ra * rb + g0 * rb;
  const double dt0b = dg0 * ra * rb + g0 * ra;
  const double omega = std::exp(-C * r13) / den * std::pow(rho, -11.0 / 3.0);
  const double delta = C * r13 + D * r13 / den;
  const double domega = omega * (delta - 11.0) / (3.0 * rho);
  const double r43i = r13 / rho;
  const double ddelta = -(1.0 / 3.0) * r43i * (C + D / (den * den));
  double s, dsa, aaa, aab, abb, s2, dsb, t1, t2, t3;
  lyp_bracket(ra, rb, delta, ddelta, gaa, gab, gbb, s, dsa, aaa, aab, abb);
  lyp_bracket(rb, ra, delta, ddelta, gbb, gab, gaa, s2, dsb, t1, t2, t3);
  const double ab = A * B;
  o.f = t0 - ab * omega * s;
  o.vra = dt0a - ab * (domega * s + omega * dsa);
  o.vrb = dt0b - ab * (domega * s + omega * dsb);
  o.vgaa = -ab * omega * aaa;
  o.vgab = -ab * omega * aab;
  o.vgbb = -ab * omega * abb;
  return o;
}

// PbeAbParams::CALCHEM_ANALYTIC (xc.rs:566-573)
const double kPbeKappa = 0.804, kPbeMu = 0.2195149727645171, kPbeBeta = 0.06672455060314922,
             kPbeGamma = 0.0310906908696549, kPw92A0 = 0.0310907, kPw92A1 = 0.01554535;

void pbe_x_one(double rs, double g, double& f, double& vr, double& vg) {
  // xc.rs:576-603
  if (rs < kRhoCutoff) { f = vr = vg = 0; return; }
  const double ru = 2.0 * rs, gu = 4.0 * std::max(g, 0.0);
  const double cxu = -0.75 * std::pow(3.0 / kPi, 1.0 / 3.0);
  const double r13 = std::cbrt(ru), r43 = ru * r13;
  const double exl = cxu * r43;
  const double kf = std::cbrt(3.0 * kPi * kPi * ru);
  const double ds2 = 4.0 * kf * kf * ru * ru;
  const double s2 = gu / ds2;
  const double opm = 1.0 + (kPbeMu / kPbeKappa) * s2;
  const double fx = 1.0 + kPbeKappa - kPbeKappa / opm;
  const double dfx = kPbeMu / (opm * opm);
  const double fu = exl * fx;
  const double dfr = (4.0 / 3.0) * cxu * r13 * fx + exl * dfx * (-(8.0 / 3.0) * s2 / ru);
  const double dfg = exl * dfx / ds2;
  f = 0.5 * fu; vr = dfr; vg = 2.0 * dfg;
}

XcOut pbe_x(double ra, double rb, double gaa, double gbb) {
  XcOut o;
  double fa, va, ga, fb, vb, gb;
  pbe_x_one(ra, gaa, fa, va, ga);
  pbe_x_one(rb, gbb, fb, vb, gb);
  o.f = fa + fb; o.vra = va; o.vrb = vb; o.vgaa = ga; o.vgbb = gb;
  return o;
}

struct Pw92 { double a, a1, b1, b2, b3, b4; };
// xc.rs:639-664
const Pw92 kPwG0 = {0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294};
const Pw92 kPwG1 = {0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517};
const Pw92 kPwGA = {0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671};

void pw92_g(double rs, const Pw92& ch, double& g, double& dg) {
  // xc.rs:667-681
  const double x = std::sqrt(rs), x2 = rs, x3 = x2 * x, x4 = x2 * x2;
  const double q0 = -2.0 * ch.a * (1.0 + ch.a1 * rs);
  const double q1 = 2.0 * ch.a * (ch.b1 * x + ch.b2 * x2 + ch.b3 * x3 + ch.b4 * x4);
  const double dq1 = ch.a * (ch.b1 / x + 2.0 * ch.b2 + 3.0 * ch.b3 * x + 4.0 * ch.b4 * x2);
  const double ln = std::log(1.0 + 1.0 / q1);
  g = q0 * ln;
  dg = -2.0 * ch.a * ch.a1 * ln - q0 * dq1 / (q1 * (q1 + 1.0));
}

XcOut pbe_c(double ra, double rb, double gaa, double gab, double gbb) {
  // xc.rs:699-828
  XcOut o;
  const double rho = ra + rb;
  if (rho < kRhoCutoff) return o;
  const double gt = std::max(gaa + 2.0 * gab + gbb, 0.0);
  const double rs = std::cbrt(3.0 / (4.0 * kPi * rho));
  const double drs = -rs / (3.0 * rho);
  const double zeta = clampd((ra - rb) / rho, -1.0, 1.0);
  Pw92 g0 = kPwG0; g0.a = kPw92A0;
  Pw92 g1 = kPwG1; g1.a = kPw92A1;
  double e0, de0, e1, de1, mac, dmac;
  pw92_g(rs, g0, e0, de0);
  pw92_g(rs, g1, e1, de1);
  pw92_g(rs, kPwGA, mac, dmac);
  const double ac = -mac, dac = -dmac;
  double fz, dfz, fdd0;
  spin_interp(zeta, fz, dfz, fdd0);
  const double ifd = 1.0 / fdd0;
  const double z2 = zeta * zeta, z3 = z2 * zeta, z4 = z2 * z2, omz4 = 1.0 - z4;
  const double ec = e0 + ac * fz * ifd * omz4 + (e1 - e0) * fz * z4;
  const double dec_drs = de0 + dac * fz * ifd * omz4 + (de1 - de0) * fz * z4;
  const double dec_drho = dec_drs * drs;
  const double dec_dz = ac * ifd * (dfz * omz4 - 4.0 * z3 * fz) + (e1 - e0) * (dfz * z4 + 4.0 * z3 * fz);
  if (gt < 1e-36) {
    o.f = rho * ec;
    o.vra = ec + rho * dec_drho + (1.0 - zeta) * dec_dz;
    o.vrb = ec + rho * dec_drho - (1.0 + zeta) * dec_dz;
    return o;
  }
  const double b0 = kPbeBeta / kPbeGamma;
  const double zp = std::max(1.0 + zeta, 1e-24), zm = std::max(1.0 - zeta, 1e-24);
  const double zp23 = powi(std::cbrt(zp), 2), zm23 = powi(std::cbrt(zm), 2);
  const double phi = 0.5 * (zp23 + zm23), phi2 = phi * phi, phi3 = phi2 * phi;
  const double omz_dphi = ((1.0 - zeta) * (1.0 / std::cbrt(zp)) - zm23) / 3.0;
  const double mopz_dphi = ((1.0 + zeta) * (1.0 / std::cbrt(zm)) - zp23) / 3.0;
  const double ct = (16.0 / kPi) * std::cbrt(3.0 * kPi * kPi);
  const double rho73 = rho * rho * std::cbrt(rho);
  const double dt2 = ct * phi2 * rho73;
  const double t2 = gt / dt2;
  const double w = -ec / (kPbeGamma * phi3);
  double af, daw;
  if (w > 100.0) { af = 0; daw = 0; }
  else {
    const double em1 = std::expm1(w), ew = std::exp(w);
    af = b0 / em1;
    daw = -af * ew / em1;
  }
  const double u = af * t2;
  const double dp = 1.0 + u + u * u;
  const double qr = (1.0 + u) / dp;
  const double za = 1.0 + b0 * t2 * qr;
  const double lnz = std::log(za);
  const double h = kPbeGamma * phi3 * lnz;
  const double dz_dt2 = b0 * (1.0 + 2.0 * u) / (dp * dp);
  const double dz_da = -b0 * t2 * t2 * u * (2.0 + u) / (dp * dp);
  const double dh_dt2 = kPbeGamma * phi3 * dz_dt2 / za;
  const double dh_dw = kPbeGamma * phi3 * (dz_da * daw) / za;
  const double dh_drho = dh_dt2 * (-(7.0 / 3.0) * t2 / rho) + dh_dw * (-dec_drho / (kPbeGamma * phi3));
  const double dh_dphi = 3.0 * kPbeGamma * phi2 * lnz + dh_dw * (-3.0 * w / phi) + dh_dt2 * (-2.0 * t2 / phi);
  const double dh_dec = dh_dw * (-1.0 / (kPbeGamma * phi3));
  const double te = ec + h;
  const double common = te + rho * (dec_drho + dh_drho);
  o.f = rho * te;
  o.vra = common + (1.0 - zeta) * dec_dz * (1.0 + dh_dec) + dh_dphi * omz_dphi;
  o.vrb = common - (1.0 + zeta) * dec_dz * (1.0 + dh_dec) + dh_dphi * mopz_dphi;
  const double vgt = rho * dh_dt2 / dt2;
  o.vgaa = vgt; o.vgab = 2.0 * vgt; o.vgbb = vgt;
  return o;
}

// Short-range attenuation F(a) of LDA-type exchange (xc.rs:863-907).  The reference evaluates erf
// with calchem_int::erf_approx (boys.rs:5, Cody's rational approximations); std::erf is used here,
// both accurate to ~1e-16.
void atten(double a, double& f, double& df) {
  const double sp = std::sqrt(kPi);
  if (a < 1e-5) {
    f = clampd(1.0 - (8.0 / 3.0) * a * sp + 8.0 * a * a, 0.0, 1.0);
    df = -(8.0 / 3.0) * sp + 16.0 * a;
    return;
  }
  if (a >= 2.0) {
    const double z = 1.0 / (a * a);
    const double c[6] = {1.0 / 36.0, -1.0 / 960.0, 1.0 / 26880.0, -1.0 / 829440.0, 1.0 / 28385280.0,
                         -1.0 / 1073479680.0};
    f = 0.0; df = 0.0;
    double pw = z;
    for (int k = 0; k < 6; ++k) {
      f += c[k] * pw;
      df -= (2 * (k + 1)) * c[k] * pw / a;
      pw *= z;
    }
    return;
  }
  const double a2 = a * a, a3 = a2 * a;
  const double ev = std::exp(-0.25 / a2);
  const double br = sp * std::erf(0.5 / a) + (2.0 * a - 4.0 * a3) * ev - 3.0 * a + 4.0 * a3;
  f = clampd(1.0 - (8.0 / 3.0) * a * br, 0.0, 1.0);
  df = -(8.0 / 3.0) * (br + a * (-3.0 + 12.0 * a2 * (1.0 - ev)));
}

void cam_x_one(double r, double g, double& f, double& vr, double& vg) {
  // xc.rs:910-944: ITYH attenuation with the B88-based Fermi wave vector, w = 0.35 + 0.46 F
  f = vr = vg = 0.0;
  if (r < kRhoCutoff) return;
  double fs, vs, fb, vb, gb;
  slater_one(r, fs, vs);
  b88_one(r, g, fb, vb, gb);
  const double fx = fs + fb, vrt = vs + vb;
  const double kb = -fx / std::pow(r, 4.0 / 3.0);
  const double kf = std::sqrt(9.0 * kPi / (2.0 * kb)) * std::cbrt(r);
  const double a = 0.33 / (2.0 * kf);
  double fa, dfa;
  atten(a, fa, dfa);
  const double w = 0.35 + 0.46 * fa, dw = 0.46 * dfa;
  f = w * fx;
  vr = w * vrt + dw * (a * (0.5 * vrt / fx - 1.0 / r)) * fx;
  vg = w * gb + dw * (0.5 * a * gb / fx) * fx;
}

struct Wb97 { double omega, cx[5], css[5], cab[5]; };
// xc.rs:1008-1017 (Chai & Head-Gordon 2008)
const Wb97 kWb97xParams = {0.30, {0.842294, 0.726479, 1.04760, -5.70635, 13.2794},
                     {1.0, -4.33879, 18.2308, -31.7430, 17.2901}, {1.0, 2.37031, -11.3995, 6.58405, -3.78132}};
const Wb97 kWb97xdParams = {0.20, {0.777964, 0.661160, 0.574541, -5.25671, 11.6386},
                      {1.0, -6.90539, 31.3343, -51.0533, 26.4423}, {1.0, 1.79413, -12.0477, 14.0847, -8.50809}};

void b97_series(double gp, const double* c, double x2, double& gv, double& dg) {
  // xc.rs:964-973
  const double gx2 = gp * std::max(x2, 0.0), den = 1.0 + gx2, u = gx2 / den;
  gv = c[0] + u * (c[1] + u * (c[2] + u * (c[3] + u * c[4])));
  dg = (c[1] + u * (2.0 * c[2] + u * (3.0 * c[3] + 4.0 * u * c[4]))) * (gp / (den * den));
}

void pw92_lsda(double ra, double rb, double& f, double& va, double& vb) {
  // xc.rs:975-1006
  f = va = vb = 0.0;
  const double rho = ra + rb;
  if (rho < kRhoCutoff) return;
  const double rs = std::cbrt(3.0 / (4.0 * kPi * rho)), drs = -rs / (3.0 * rho);
  const double zeta = clampd((ra - rb) / rho, -1.0, 1.0);
  double e0, de0, e1, de1, mac, dmac;
  pw92_g(rs, kPwG0, e0, de0);
  pw92_g(rs, kPwG1, e1, de1);
  pw92_g(rs, kPwGA, mac, dmac);
  const double ac = -mac, dac = -dmac;
  double fz, dfz, fdd0;
  spin_interp(zeta, fz, dfz, fdd0);
  const double ifd = 1.0 / fdd0;
  const double z2 = zeta * zeta, z3 = z2 * zeta, z4 = z2 * z2, om = 1.0 - z4;
  const double ec = e0 + ac * fz * ifd * om + (e1 - e0) * fz * z4;
  const double decr = de0 + dac * fz * ifd * om + (de1 - de0) * fz * z4;
  const double decz = ac * ifd * (dfz * om - 4.0 * z3 * fz) + (e1 - e0) * (dfz * z4 + 4.0 * z3 * fz);
  f = rho * ec;
  va = ec + rho * decr * drs + (1.0 - zeta) * decz;
  vb = ec + rho * decr * drs - (1.0 + zeta) * decz;
}

void wb97_x_one(double r, double g, const Wb97& P, double& f, double& vr, double& vg) {
  // xc.rs:1020-1050
  f = vr = vg = 0.0;
  if (r < kRhoCutoff) return;
  double fs, vs;
  slater_one(r, fs, vs);
  const double r43 = r * std::cbrt(r), r83 = r43 * r43;
  const double a = P.omega / (2.0 * std::cbrt(6.0 * kPi * kPi * r));
  double fa, dfa;
  atten(a, fa, dfa);
  const double fsr = fs * fa, vsr = vs * fa + fs * dfa * (-a / (3.0 * r));
  const double x2 = std::max(g, 0.0) / r83;
  double gx, dgx;
  b97_series(0.004, P.cx, x2, gx, dgx);
  f = fsr * gx;
  vr = vsr * gx + fsr * dgx * (-(8.0 / 3.0) * x2 / r);
  vg = fsr * dgx / r83;
}

XcOut wb97(double ra, double rb, double gaa, double gbb, const Wb97& P) {
  // xc.rs:1052-1103
  XcOut o;
  double fxa, vxa, gxa, fxb, vxb, gxb;
  wb97_x_one(ra, gaa, P, fxa, vxa, gxa);
  wb97_x_one(rb, gbb, P, fxb, vxb, gxb);
  double ft, vta, vtb, fpa, vpa, dm, fpb, vpb;
  pw92_lsda(ra, rb, ft, vta, vtb);
  pw92_lsda(ra, 0.0, fpa, vpa, dm);
  pw92_lsda(0.0, rb, fpb, dm, vpb);
  const double fpe = ft - fpa - fpb;
  double xa2 = 0, dxar = 0, dxag = 0, xb2 = 0, dxbr = 0, dxbg = 0;
  if (ra >= kRhoCutoff) {
    const double r83 = std::pow(ra, 8.0 / 3.0);
    xa2 = std::max(gaa, 0.0) / r83; dxar = -(8.0 / 3.0) * xa2 / ra; dxag = 1.0 / r83;
  }
  if (rb >= kRhoCutoff) {
    const double r83 = std::pow(rb, 8.0 / 3.0);
    xb2 = std::max(gbb, 0.0) / r83; dxbr = -(8.0 / 3.0) * xb2 / rb; dxbg = 1.0 / r83;
  }
  double gsa, dgsa, gsb, dgsb, gab, dgab;
  b97_series(0.2, P.css, xa2, gsa, dgsa);
  b97_series(0.2, P.css, xb2, gsb, dgsb);
  b97_series(0.006, P.cab, 0.5 * (xa2 + xb2), gab, dgab);
  o.f = fxa + fxb + fpa * gsa + fpb * gsb + fpe * gab;
  o.vra = vxa + vpa * gsa + fpa * dgsa * dxar + (vta - vpa) * gab + fpe * dgab * 0.5 * dxar;
  o.vrb = vxb + vpb * gsb + fpb * dgsb * dxbr + (vtb - vpb) * gab + fpe * dgab * 0.5 * dxbr;
  o.vgaa = gxa + fpa * dgsa * dxag + fpe * dgab * 0.5 * dxag;
  o.vgbb = gxb + fpb * dgsb * dxbg + fpe * dgab * 0.5 * dxbg;
  return o;
}

// eval_xc_spin (xc.rs:159-223).  Codes follow the XcFunctional enum order (xc.rs:16-35).
enum Xc { kSvwn5 = 0, kBlyp = 1, kPbe = 2, kB3lyp = 3, kB3lyp5 = 4, kPbe0 = 5, kCamB3lyp = 6, kWb97x = 7, kWb97xd = 8 };

XcOut eval_xc(int func, double rho_a, double rho_b, double gamma_aa, double gamma_ab, double gamma_bb) {
  XcOut o;
  const double ra = std::max(rho_a, 0.0), rb = std::max(rho_b, 0.0);
  if (ra + rb < kRhoCutoff) return o;
  const double gaa = std::max(gamma_aa, 0.0), gbb = std::max(gamma_bb, 0.0);
  switch (func) {
    case kSvwn5: o = slater_x(ra, rb); o.add(1.0, vwn_c(ra, rb, kVwn5)); break;
    case kBlyp:
      o = slater_x(ra, rb);
      o.add(1.0, b88_x(ra, rb, gaa, gbb));
      o.add(1.0, lyp_c(ra, rb, gaa, gamma_ab, gbb));
      break;
    case kPbe: o = pbe_x(ra, rb, gaa, gbb); o.add(1.0, pbe_c(ra, rb, gaa, gamma_ab, gbb)); break;
    case kB3lyp:
    case kB3lyp5:
      o.add(0.80, slater_x(ra, rb));
      o.add(0.72, b88_x(ra, rb, gaa, gbb));
      o.add(0.19, vwn_c(ra, rb, func == kB3lyp ? kVwnRpa : kVwn5));
      o.add(0.81, lyp_c(ra, rb, gaa, gamma_ab, gbb));
      break;
    case kPbe0:
      o.add(0.75, pbe_x(ra, rb, gaa, gbb));
      o.add(1.00, pbe_c(ra, rb, gaa, gamma_ab, gbb));
      break;
    case kCamB3lyp: {  // xc.rs:214-219
      double fa, va, ga, fb, vb, gb;
      cam_x_one(ra, gaa, fa, va, ga);
      cam_x_one(rb, gbb, fb, vb, gb);
      o.f = fa + fb; o.vra = va; o.vrb = vb; o.vgaa = ga; o.vgbb = gb;
      o.add(0.19, vwn_c(ra, rb, kVwn5));
      o.add(0.81, lyp_c(ra, rb, gaa, gamma_ab, gbb));
      break;
    }
    case kWb97x: o = wb97(ra, rb, gaa, gbb, kWb97xParams); break;
    case kWb97xd: o = wb97(ra, rb, gaa, gbb, kWb97xdParams); break;
  }
  return o;
}

// ============================================================================
// Vxc assembly (crates/calchem-dft/src/vxc.rs)
// ============================================================================
struct Kahan {
  double s = 0.0, c = 0.0;
  void add(double x) {  // vxc.rs:226-229 (compensated sum as written there)
    const double term = x - c;
    const double next = s + term;
    c = (next - s) - term;
    s = next;
  }
};

// Block screening used by every path: bounding sphere + shell cutoff (vxc.rs:112-159, 446-493).
bool block_candidates(const Basis& bs, const GridPoint* pts, int npts, std::vector<int>& pt_idx,
                      std::vector<int>& cand) {
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  pt_idx.clear();
  cand.clear();
  for (int g = 0; g < npts; ++g) {
    if (std::fabs(pts[g].w) < 1e-24) continue;
    pt_idx.push_back(g);
    const double c[3] = {pts[g].x, pts[g].y, pts[g].z};
    for (int q = 0; q < 3; ++q) { if (c[q] < mn[q]) mn[q] = c[q]; if (c[q] > mx[q]) mx[q] = c[q]; }
  }
  if (pt_idx.empty()) return false;
  const double ce[3] = {0.5 * (mn[0] + mx[0]), 0.5 * (mn[1] + mx[1]), 0.5 * (mn[2] + mx[2])};
  const double dx = mx[0] - ce[0], dy = mx[1] - ce[1], dz = mx[2] - ce[2];
  const double rbox = std::sqrt(dx * dx + dy * dy + dz * dz);
  for (size_t s = 0; s < bs.shells.size(); ++s) {
    const Shell& sh = bs.shells[s];
    const double ex = sh.center[0] - ce[0], ey = sh.center[1] - ce[1], ez = sh.center[2] - ce[2];
    const double d2 = ex * ex + ey * ey + ez * ez;
    const double th = rbox + sh.r_cut;
    if (d2 <= th * th) cand.push_back((int)s);
  }
  return true;
}

struct Ws {
  std::vector<int> pt_idx, cand, ao_idx, loc, ao2loc;
  std::vector<AoVal> act;
  std::vector<double> p_sub, pb_sub, v_sub, vb_sub, phi_p, z, zb;
};

// accumulate_rks_points_with (vxc.rs:99-276) + Nelec
void rks_points_chunk(const Basis& bs, const GridPoint* chunk, int n_chunk, const double* P, int func, Kahan& e,
                      Kahan& ne, double* v_loc, Ws& ws) {
  const int n = bs.n_ao;
  ws.ao2loc.assign(n, -1);
  for (int s0 = 0; s0 < n_chunk; s0 += kBatch) {
    const int nb = std::min(kBatch, n_chunk - s0);
    const GridPoint* sub = chunk + s0;
    if (!block_candidates(bs, sub, nb, ws.pt_idx, ws.cand)) continue;
    ws.ao_idx.clear();
    for (int s : ws.cand)
      for (int c = 0; c < bs.shells[s].ncomp(); ++c) ws.ao_idx.push_back(bs.shells[s].ao_offset + c);
    const int m = (int)ws.ao_idx.size();
    if (m == 0) continue;
    for (int i = 0; i < m; ++i) ws.ao2loc[ws.ao_idx[i]] = i;
    ws.p_sub.assign((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) ws.p_sub[(size_t)i * m + j] = P[(size_t)ws.ao_idx[i] * n + ws.ao_idx[j]];
    ws.v_sub.assign((size_t)m * m, 0.0);
    for (int g = 0; g < nb; ++g) {
      const GridPoint& gp = sub[g];
      const double w = gp.w;
      if (std::fabs(w) < 1e-24) continue;
      const double r[3] = {gp.x, gp.y, gp.z};
      eval_aos_grad(bs, ws.cand, r, ws.act);
      if (ws.act.empty()) continue;
      const int pm = (int)ws.act.size();
      ws.loc.resize(pm);
      for (int k = 0; k < pm; ++k) ws.loc[k] = ws.ao2loc[ws.act[k].mu];
      ws.phi_p.resize(pm);
      double rho = 0, gr[3] = {0, 0, 0};
      for (int k = 0; k < pm; ++k) {
        const double* prow = &ws.p_sub[(size_t)ws.loc[k] * m];
        double s = 0;
        for (int j = 0; j < pm; ++j) s += prow[ws.loc[j]] * ws.act[j].v;
        ws.phi_p[k] = s;
        rho += ws.act[k].v * s;
        gr[0] += 2.0 * ws.act[k].gx * s;
        gr[1] += 2.0 * ws.act[k].gy * s;
        gr[2] += 2.0 * ws.act[k].gz * s;
      }
      if (rho < kDensityScreen) continue;
      const double rs = 0.5 * rho;
      const double gss = 0.25 * (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
      const XcOut o = eval_xc(func, rs, rs, gss, gss, gss);
      e.add(w * o.f);
      ne.add(w * rho);
      const double us = o.vgaa + 0.5 * o.vgab;
      const double u[3] = {us * gr[0], us * gr[1], us * gr[2]};
      ws.z.resize(pm);
      const double hw = 0.5 * w * o.vra;
      for (int k = 0; k < pm; ++k)
        ws.z[k] = hw * ws.act[k].v + w * (u[0] * ws.act[k].gx + u[1] * ws.act[k].gy + u[2] * ws.act[k].gz);
      for (int i = 0; i < pm; ++i) {
        double* vrow = &ws.v_sub[(size_t)ws.loc[i] * m];
        for (int j = 0; j <= i; ++j) vrow[ws.loc[j]] += ws.z[i] * ws.act[j].v + ws.act[i].v * ws.z[j];
      }
    }
    for (int i = 0; i < m; ++i) {
      double* orow = v_loc + (size_t)ws.ao_idx[i] * n;
      for (int j = 0; j <= i; ++j) orow[ws.ao_idx[j]] += ws.v_sub[(size_t)i * m + j];
    }
    for (int mu : ws.ao_idx) ws.ao2loc[mu] = -1;
  }
}

// accumulate_uks_points (vxc.rs:1141-1348) + per-spin Nelec
void uks_points_chunk(const Basis& bs, const GridPoint* chunk, int n_chunk, const double* Pa, const double* Pb,
                      int func, Kahan& e, Kahan& nea, Kahan& neb, double* va, double* vb, Ws& ws) {
  const int n = bs.n_ao;
  ws.ao2loc.assign(n, -1);
  for (int s0 = 0; s0 < n_chunk; s0 += kBatch) {
    const int nb = std::min(kBatch, n_chunk - s0);
    const GridPoint* sub = chunk + s0;
    if (!block_candidates(bs, sub, nb, ws.pt_idx, ws.cand)) continue;
    ws.ao_idx.clear();
    for (int s : ws.cand)
      for (int c = 0; c < bs.shells[s].ncomp(); ++c) ws.ao_idx.push_back(bs.shells[s].ao_offset + c);
    const int m = (int)ws.ao_idx.size();
    if (m == 0) continue;
    for (int i = 0; i < m; ++i) ws.ao2loc[ws.ao_idx[i]] = i;
    ws.p_sub.assign((size_t)m * m, 0.0);
    ws.pb_sub.assign((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        ws.p_sub[(size_t)i * m + j] = Pa[(size_t)ws.ao_idx[i] * n + ws.ao_idx[j]];
        ws.pb_sub[(size_t)i * m + j] = Pb[(size_t)ws.ao_idx[i] * n + ws.ao_idx[j]];
      }
    ws.v_sub.assign((size_t)m * m, 0.0);
    ws.vb_sub.assign((size_t)m * m, 0.0);
    for (int g = 0; g < nb; ++g) {
      const GridPoint& gp = sub[g];
      const double w = gp.w;
      if (std::fabs(w) < 1e-24) continue;
      const double r[3] = {gp.x, gp.y, gp.z};
      eval_aos_grad(bs, ws.cand, r, ws.act);
      if (ws.act.empty()) continue;
      const int pm = (int)ws.act.size();
      ws.loc.resize(pm);
      for (int k = 0; k < pm; ++k) ws.loc[k] = ws.ao2loc[ws.act[k].mu];
      double rho_a = 0, rho_b = 0, ga[3] = {0, 0, 0}, gb[3] = {0, 0, 0};
      for (int k = 0; k < pm; ++k) {
        const double* pa = &ws.p_sub[(size_t)ws.loc[k] * m];
        const double* pb = &ws.pb_sub[(size_t)ws.loc[k] * m];
        double sa = 0, sb = 0;
        for (int j = 0; j < pm; ++j) {
          sa += pa[ws.loc[j]] * ws.act[j].v;
          sb += pb[ws.loc[j]] * ws.act[j].v;
        }
        rho_a += ws.act[k].v * sa;
        rho_b += ws.act[k].v * sb;
        const double gk[3] = {ws.act[k].gx, ws.act[k].gy, ws.act[k].gz};
        for (int q = 0; q < 3; ++q) {
          ga[q] += 2.0 * gk[q] * sa;
          gb[q] += 2.0 * gk[q] * sb;
        }
      }
      const double ra = std::max(rho_a, 0.0), rb = std::max(rho_b, 0.0);
      if (ra + rb < kDensityScreen) continue;
      const double gaa = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
      const double gab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
      const double gbb = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
      const XcOut o = eval_xc(func, ra, rb, gaa, gab, gbb);
      e.add(w * o.f);
      nea.add(w * ra);
      neb.add(w * rb);
      double ua[3], ub[3];
      for (int q = 0; q < 3; ++q) {
        ua[q] = 2.0 * o.vgaa * ga[q] + o.vgab * gb[q];
        ub[q] = 2.0 * o.vgbb * gb[q] + o.vgab * ga[q];
      }
      ws.z.resize(pm);
      ws.zb.resize(pm);
      const double hwa = 0.5 * w * o.vra, hwb = 0.5 * w * o.vrb;
      for (int k = 0; k < pm; ++k) {
        const AoVal& a = ws.act[k];
        ws.z[k] = hwa * a.v + w * (ua[0] * a.gx + ua[1] * a.gy + ua[2] * a.gz);
        ws.zb[k] = hwb * a.v + w * (ub[0] * a.gx + ub[1] * a.gy + ub[2] * a.gz);
      }
      for (int i = 0; i < pm; ++i) {
        double* ra_row = &ws.v_sub[(size_t)ws.loc[i] * m];
        double* rb_row = &ws.vb_sub[(size_t)ws.loc[i] * m];
        for (int j = 0; j <= i; ++j) {
          ra_row[ws.loc[j]] += ws.z[i] * ws.act[j].v + ws.act[i].v * ws.z[j];
          rb_row[ws.loc[j]] += ws.zb[i] * ws.act[j].v + ws.act[i].v * ws.zb[j];
        }
      }
    }
    for (int i = 0; i < m; ++i) {
      const int mu = ws.ao_idx[i];
      for (int j = 0; j <= i; ++j) {
        const int nu = ws.ao_idx[j];
        const double a = ws.v_sub[(size_t)i * m + j], b = ws.vb_sub[(size_t)i * m + j];
        va[(size_t)mu * n + nu] += a;
        vb[(size_t)mu * n + nu] += b;
        if (i != j) {
          va[(size_t)nu * n + mu] += a;
          vb[(size_t)nu * n + mu] += b;
        }
      }
    }
    for (int mu : ws.ao_idx) ws.ao2loc[mu] = -1;
  }
}

int n_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// bounded_worker_count / bounded_grid_chunk_size (vxc.rs:25-49) without the env-var memory caps.
int worker_count(int n, int channels, int threads) {
  const double bytes = std::max(1.0, (double)n * n * 8.0 * channels);
  const double budget = 4.0 * 1024 * 1024 * 1024;
  return std::max(1, std::min(threads, (int)std::max(1.0, std::floor(budget / bytes))));
}

// evaluate_vxc_rks (vxc.rs:280-384), materialised-grid branch.
void vxc_rks_points(const Basis& bs, const std::vector<GridPoint>& pts, const double* P, int func, int threads,
                    double* exc, double* nelec, double* V) {
  const int n = bs.n_ao;
  std::memset(V, 0, sizeof(double) * (size_t)n * n);
  *exc = 0;
  *nelec = 0;
  if (n == 0 || pts.empty()) return;
  const int workers = worker_count(n, 1, threads);
  const int N = (int)pts.size();
  const int chunk = std::max(kGridChunk, (N + workers - 1) / workers);
  const int nchunks = (N + chunk - 1) / chunk;
  std::vector<std::vector<double>> vloc(nchunks);
  std::vector<Kahan> es(nchunks), ns(nchunks);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int c = 0; c < nchunks; ++c) {
    Ws ws;
    vloc[c].assign((size_t)n * n, 0.0);
    const int s = c * chunk, len = std::min(chunk, N - s);
    rks_points_chunk(bs, pts.data() + s, len, P, func, es[c], ns[c], vloc[c].data(), ws);
  }
  double e = 0, ne = 0;
  for (int c = 0; c < nchunks; ++c) {
    e += es[c].s;
    ne += ns[c].s;
    for (size_t i = 0; i < (size_t)n * n; ++i) V[i] += vloc[c][i];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) V[(size_t)j * n + i] = V[(size_t)i * n + j];
  *exc = e;
  *nelec = ne;
}

// evaluate_vxc_uks (vxc.rs:1352-1470), materialised-grid branch.
void vxc_uks_points(const Basis& bs, const std::vector<GridPoint>& pts, const double* Pa, const double* Pb, int func,
                    int threads, double* exc, double* nea, double* neb, double* Va, double* Vb) {
  const int n = bs.n_ao;
  std::memset(Va, 0, sizeof(double) * (size_t)n * n);
  std::memset(Vb, 0, sizeof(double) * (size_t)n * n);
  *exc = *nea = *neb = 0;
  if (n == 0 || pts.empty()) return;
  const int workers = worker_count(n, 2, threads);
  const int N = (int)pts.size();
  const int chunk = std::max(kGridChunk, (N + workers - 1) / workers);
  const int nchunks = (N + chunk - 1) / chunk;
  std::vector<std::vector<double>> va(nchunks), vb(nchunks);
  std::vector<Kahan> es(nchunks), na(nchunks), nb(nchunks);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int c = 0; c < nchunks; ++c) {
    Ws ws;
    va[c].assign((size_t)n * n, 0.0);
    vb[c].assign((size_t)n * n, 0.0);
    const int s = c * chunk, len = std::min(chunk, N - s);
    uks_points_chunk(bs, pts.data() + s, len, Pa, Pb, func, es[c], na[c], nb[c], va[c].data(), vb[c].data(), ws);
  }
  for (int c = 0; c < nchunks; ++c) {
    *exc += es[c].s;
    *nea += na[c].s;
    *neb += nb[c].s;
    for (size_t i = 0; i < (size_t)n * n; ++i) {
      Va[i] += va[c][i];
      Vb[i] += vb[c][i];
    }
  }
}

// ---------------------------------------------------------------------------
// RksVxcEngine CPU path (vxc.rs:429-716 construction, 801-985 evaluate).
// ---------------------------------------------------------------------------
struct CachedBatch {
  std::vector<int> ao;     // global AO indices (ascending)
  std::vector<double> w;   // surviving point weights
  std::vector<double> phi, dx, dy, dz;  // row-major m x b
};

struct RksEngine {
  const Basis* bs = nullptr;
  std::vector<GridPoint> pts;
  bool cached = false;
  double cache_bytes = 0;
  double work = 0;  // sum over batches of m_b^2 n_b (the two contractions' size)
  std::vector<CachedBatch> batches;
};

RksEngine* rks_engine_create(const Basis& bs, const std::vector<GridPoint>& pts, double cap_bytes, int threads) {
  auto* eng = new RksEngine;
  eng->bs = &bs;
  eng->pts = pts;
  const int N = (int)pts.size();
  const int nbatch = (N + kBatch - 1) / kBatch;
  std::vector<std::vector<int>> cand(nbatch), pidx(nbatch);
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
  for (int b = 0; b < nbatch; ++b) {
    const int s = b * kBatch, len = std::min(kBatch, N - s);
    std::vector<int> pi, ca;
    if (block_candidates(bs, pts.data() + s, len, pi, ca)) { pidx[b] = pi; cand[b] = ca; }
  }
  double total = 0;
  for (int b = 0; b < nbatch; ++b) {
    int m = 0;
    for (int s : cand[b]) m += bs.shells[s].ncomp();
    total += (double)m * (double)pidx[b].size() * 4.0 * 8.0;
    eng->work += (double)m * (double)m * (double)pidx[b].size();
  }
  eng->cache_bytes = total;
  if (total > cap_bytes) return eng;  // the engine then runs evaluate_vxc_rks (vxc.rs:802-804)
  eng->cached = true;
  eng->batches.resize(nbatch);
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
  for (int b = 0; b < nbatch; ++b) {
    if (pidx[b].empty() || cand[b].empty()) continue;
    CachedBatch& cb = eng->batches[b];
    for (int s : cand[b])
      for (int c = 0; c < bs.shells[s].ncomp(); ++c) cb.ao.push_back(bs.shells[s].ao_offset + c);
    const int m = (int)cb.ao.size(), nb = (int)pidx[b].size();
    std::vector<int> ao2loc(bs.n_ao, -1);
    for (int i = 0; i < m; ++i) ao2loc[cb.ao[i]] = i;
    cb.phi.assign((size_t)m * nb, 0.0);
    cb.dx.assign((size_t)m * nb, 0.0);
    cb.dy.assign((size_t)m * nb, 0.0);
    cb.dz.assign((size_t)m * nb, 0.0);
    std::vector<AoVal> act;
    for (int g = 0; g < nb; ++g) {
      const GridPoint& gp = pts[b * kBatch + pidx[b][g]];
      cb.w.push_back(gp.w);
      const double r[3] = {gp.x, gp.y, gp.z};
      eval_aos_grad(bs, cand[b], r, act);
      for (const AoVal& a : act) {
        const size_t idx = (size_t)ao2loc[a.mu] * nb + g;
        cb.phi[idx] = a.v;
        cb.dx[idx] = a.gx;
        cb.dy[idx] = a.gy;
        cb.dz[idx] = a.gz;
      }
    }
  }
  return eng;
}

// blocked: the two contractions by the register-blocked FMA product of cpu_gemm.cpp (the timed CPU
// baseline, as CalChem runs faer's GEMM) instead of the checker's plain loops; same sums, other order.
void rks_engine_evaluate(const RksEngine& eng, const double* P, int func, int threads, double* exc, double* nelec,
                         double* V, int batch_begin, int batch_end, bool blocked) {
  const Basis& bs = *eng.bs;
  const int n = bs.n_ao;
  if (!eng.cached) {
    vxc_rks_points(bs, eng.pts, P, func, threads, exc, nelec, V);
    return;
  }
  std::memset(V, 0, sizeof(double) * (size_t)n * n);
  *exc = 0;
  *nelec = 0;
  const int nb_all = (int)eng.batches.size();
  if (batch_end < 0 || batch_end > nb_all) batch_end = nb_all;
  if (batch_begin < 0) batch_begin = 0;
  const int nbat = batch_end - batch_begin;
  if (n == 0 || nbat <= 0) return;
  const int workers = worker_count(n, 1, threads);
  const int clen = std::max(1, (nbat + workers - 1) / workers);
  const int nchunks = (nbat + clen - 1) / clen;
  std::vector<std::vector<double>> vloc(nchunks);
  std::vector<Kahan> es(nchunks), ns(nchunks);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int c = 0; c < nchunks; ++c) {
    std::vector<double>& vl = vloc[c];
    vl.assign((size_t)n * n, 0.0);
    std::vector<double> psub, t, z, vsub, phit;
    double rho[kBatch], gx[kBatch], gy[kBatch], gz[kBatch], wv[kBatch], ux[kBatch], uy[kBatch], uz[kBatch];
    const int b0 = batch_begin + c * clen, b1 = std::min(batch_end, b0 + clen);
    for (int bi = b0; bi < b1; ++bi) {
      const CachedBatch& cb = eng.batches[bi];
      const int m = (int)cb.ao.size(), b = (int)cb.w.size();
      if (m == 0 || b == 0) continue;
      psub.assign((size_t)m * m, 0.0);
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) psub[(size_t)i * m + j] = P[(size_t)cb.ao[i] * n + cb.ao[j]];
      // T = P_sub * Phi (gemm_nn_into, calchem-tensor/src/lib.rs:114-124)
      t.assign((size_t)m * b, 0.0);
      if (blocked) {
        orc::gemm_acc(m, b, m, psub.data(), m, 1, cb.phi.data(), b, t.data(), b);
      } else {
        for (int i = 0; i < m; ++i)
          for (int k = 0; k < m; ++k) {
            const double pik = psub[(size_t)i * m + k];
            const double* prow = &cb.phi[(size_t)k * b];
            double* trow = &t[(size_t)i * b];
            for (int g = 0; g < b; ++g) trow[g] += pik * prow[g];
          }
      }
      for (int g = 0; g < b; ++g) rho[g] = gx[g] = gy[g] = gz[g] = 0.0;
      for (int i = 0; i < m; ++i)
        for (int g = 0; g < b; ++g) {
          const size_t o = (size_t)i * b + g;
          const double tg = t[o];
          rho[g] += cb.phi[o] * tg;
          gx[g] += cb.dx[o] * tg;
          gy[g] += cb.dy[o] * tg;
          gz[g] += cb.dz[o] * tg;
        }
      bool any = false;
      for (int g = 0; g < b; ++g) {
        const double rt = rho[g];
        if (rt < kDensityScreen) { wv[g] = ux[g] = uy[g] = uz[g] = 0.0; continue; }
        any = true;
        const double w = cb.w[g];
        const double grx = 2.0 * gx[g], gry = 2.0 * gy[g], grz = 2.0 * gz[g];
        const double rs = 0.5 * rt;
        const double gss = 0.25 * (grx * grx + gry * gry + grz * grz);
        const XcOut o = eval_xc(func, rs, rs, gss, gss, gss);
        es[c].add(w * o.f);
        ns[c].add(w * rt);
        wv[g] = 0.5 * w * o.vra;
        const double us = w * (o.vgaa + 0.5 * o.vgab);
        ux[g] = us * grx; uy[g] = us * gry; uz[g] = us * grz;
      }
      if (!any) continue;
      z.assign((size_t)m * b, 0.0);
      for (int i = 0; i < m; ++i)
        for (int g = 0; g < b; ++g) {
          const size_t o = (size_t)i * b + g;
          z[o] = wv[g] * cb.phi[o] + ux[g] * cb.dx[o] + uy[g] * cb.dy[o] + uz[g] * cb.dz[o];
        }
      // V_sub = Z * Phi^T (gemm_nt_into, calchem-tensor/src/lib.rs:126-135)
      vsub.assign((size_t)m * m, 0.0);
      if (blocked) {
        phit.resize((size_t)b * m);  // Phi^T, b x m, so that the product streams rows of both operands
        for (int i = 0; i < m; ++i)
          for (int g = 0; g < b; ++g) phit[(size_t)g * m + i] = cb.phi[(size_t)i * b + g];
        orc::gemm_acc(m, m, b, z.data(), b, 1, phit.data(), m, vsub.data(), m);
      } else {
        for (int i = 0; i < m; ++i)
          for (int j = 0; j < m; ++j) {
            const double* zr = &z[(size_t)i * b];
            const double* pr = &cb.phi[(size_t)j * b];
            double s = 0;
            for (int g = 0; g < b; ++g) s += zr[g] * pr[g];
            vsub[(size_t)i * m + j] = s;
          }
      }
      for (int i = 0; i < m; ++i) {
        double* orow = &vl[(size_t)cb.ao[i] * n];
        for (int j = 0; j <= i; ++j) orow[cb.ao[j]] += vsub[(size_t)i * m + j] + vsub[(size_t)j * m + i];
      }
    }
  }
  for (int c = 0; c < nchunks; ++c) {
    *exc += es[c].s;
    *nelec += ns[c].s;
    for (size_t i = 0; i < (size_t)n * n; ++i) V[i] += vloc[c][i];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) V[(size_t)j * n + i] = V[(size_t)i * n + j];
}

// ============================================================================
// Overlap matrix (crates/calchem-int/src/one_electron.rs:7-31, 115-128; primitive.rs:1-78)
// ============================================================================
double overlap_1d(int la, int lb, double pa, double pb, double g) {
  if (la < 0 || lb < 0) return 0.0;
  if (la == 0 && lb == 0) return std::sqrt(kPi / g);
  const double i2g = 0.5 / g;
  if (la > 0)
    return pa * overlap_1d(la - 1, lb, pa, pb, g) + (la - 1) * i2g * overlap_1d(la - 2, lb, pa, pb, g) +
           lb * i2g * overlap_1d(la - 1, lb - 1, pa, pb, g);
  return pb * overlap_1d(la, lb - 1, pa, pb, g) + la * i2g * overlap_1d(la - 1, lb - 1, pa, pb, g) +
         (lb - 1) * i2g * overlap_1d(la, lb - 2, pa, pb, g);
}

void overlap_matrix(const Basis& bs, double* S) {
  const int n = bs.n_ao;
  const int ns = (int)bs.shells.size();
#pragma omp parallel for schedule(dynamic, 4)
  for (int a = 0; a < ns; ++a) {
    const Shell& A = bs.shells[a];
    for (int b = 0; b < ns; ++b) {
      const Shell& B = bs.shells[b];
      for (int ia = 0; ia < A.ncomp(); ++ia) {
        const int* ca = kComps[A.l][ia];
        for (int ib = 0; ib < B.ncomp(); ++ib) {
          const int* cb = kComps[B.l][ib];
          double sum = 0;
          for (size_t p = 0; p < A.exps.size(); ++p) {
            const double na = primitive_norm(A.exps[p], ca[0], ca[1], ca[2]);
            for (size_t q = 0; q < B.exps.size(); ++q) {
              const double nb = primitive_norm(B.exps[q], cb[0], cb[1], cb[2]);
              const double al = A.exps[p], be = B.exps[q], g = al + be, mu = al * be / g;
              double ab[3], P[3], PA[3], PB[3], r2 = 0;
              for (int k = 0; k < 3; ++k) {
                ab[k] = A.center[k] - B.center[k];
                r2 += ab[k] * ab[k];
                P[k] = (al * A.center[k] + be * B.center[k]) / g;
                PA[k] = P[k] - A.center[k];
                PB[k] = P[k] - B.center[k];
              }
              const double kab = std::exp(-mu * r2);
              const double s = kab * overlap_1d(ca[0], cb[0], PA[0], PB[0], g) *
                               overlap_1d(ca[1], cb[1], PA[1], PB[1], g) * overlap_1d(ca[2], cb[2], PA[2], PB[2], g);
              sum += A.coeffs[p] * B.coeffs[q] * na * nb * s;
            }
          }
          S[(size_t)(A.ao_offset + ia) * n + B.ao_offset + ib] = sum;
        }
      }
    }
  }
}

}  // namespace

// ============================================================================
// C interface used by oracle/oracle.py (tests, smoke check and CPU baseline only).
// ============================================================================
extern "C" {

int orc_lebedev(int n, double* xyzw) {
  if (n != 26 && n != 50 && n != 110 && n != 194 && n != 302 && n != 590) return -1;
  const auto& r = lebedev(n);
  for (size_t i = 0; i < r.size(); ++i) {
    xyzw[4 * i] = r[i].x; xyzw[4 * i + 1] = r[i].y; xyzw[4 * i + 2] = r[i].z; xyzw[4 * i + 3] = r[i].w;
  }
  return (int)r.size();
}

double orc_bragg_slater_bohr(int z) { return bragg_slater_radius_bohr(z); }
int orc_radial_shell_count(int z, int level) { return radial_shell_count(z, level); }

// ============================================================================
// XC nuclear gradient (vxc.rs:1769-1912) and the Becke weight derivative (grid.rs:423-584)
// ============================================================================
double becke_poly(double x) { return 1.5 * x - 0.5 * x * x * x; }
double becke_poly_d(double x) { return 1.5 - 1.5 * x * x; }

void becke_step_d(double nu, double& s, double& ds) {
  // grid.rs:129-140
  const double x = clampd(nu, -1.0, 1.0);
  const double f1 = becke_poly(x), d1 = becke_poly_d(x);
  const double f2 = becke_poly(f1), d2 = becke_poly_d(f1);
  const double f3 = becke_poly(f2), d3 = becke_poly_d(f2);
  s = 0.5 * (1.0 - f3);
  ds = -0.5 * d3 * d2 * d1;
}

void becke_weight_gradient(int n, const int* z, const double* xyz, int host, const double r[3], double raw_w,
                           double f_xc, double* grad) {
  // grid.rs:423-584: derivative of the Becke partition weight P_host / sum_C P_C with respect to every
  // nucleus except the host (whose term follows from translational invariance), times raw_w f_xc
  if (n <= 1 || std::fabs(f_xc) < 1e-18 || raw_w == 0.0) return;
  std::vector<double> dr(n), vr(3 * n), smat((size_t)n * n, 1.0), dsmu((size_t)n * n, 0.0), cell(n, 1.0);
  for (int c = 0; c < n; ++c) {
    for (int q = 0; q < 3; ++q) vr[3 * c + q] = r[q] - xyz[3 * c + q];
    dr[c] = std::sqrt(vr[3 * c] * vr[3 * c] + vr[3 * c + 1] * vr[3 * c + 1] + vr[3 * c + 2] * vr[3 * c + 2]);
  }
  for (int c = 0; c < n; ++c)
    for (int d = c + 1; d < n; ++d) {
      const double dx = xyz[3 * c] - xyz[3 * d], dy = xyz[3 * c + 1] - xyz[3 * d + 1], dz = xyz[3 * c + 2] - xyz[3 * d + 2];
      const double rcd = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (rcd < 1e-14) continue;
      const double mu = clampd((dr[c] - dr[d]) / rcd, -1.0, 1.0);
      const double a = becke_asymmetry(z[c], z[d]);
      double scd, dsdnu;
      becke_step_d(mu + a * (1.0 - mu * mu), scd, dsdnu);
      const double dmu = dsdnu * (1.0 - 2.0 * a * mu);
      smat[(size_t)c * n + d] = scd;
      smat[(size_t)d * n + c] = 1.0 - scd;
      dsmu[(size_t)c * n + d] = dmu;
      dsmu[(size_t)d * n + c] = dmu;
      cell[c] *= scd;
      cell[d] *= 1.0 - scd;
    }
  double zs = 0.0;
  for (double v : cell) zs += v;
  if (zs <= 1e-30) return;
  const double wn = cell[host] / zs, pref = raw_w * f_xc / zs;
  auto prod_except = [&](int c, int skip) {
    const double sv = smat[(size_t)c * n + skip];
    if (sv > 1e-12) return cell[c] / sv;
    double pr = 1.0;
    for (int d = 0; d < n; ++d)
      if (d != c && d != skip) pr *= smat[(size_t)c * n + d];
    return pr;
  };
  double hacc[3] = {0, 0, 0};
  for (int a = 0; a < n; ++a) {
    if (a == host) continue;
    const double ra = dr[a];
    if (ra < 1e-14) continue;
    const double dra[3] = {-vr[3 * a] / ra, -vr[3 * a + 1] / ra, -vr[3 * a + 2] / ra};
    double dph[3] = {0, 0, 0}, dzs[3] = {0, 0, 0};
    for (int b = 0; b < n; ++b) {
      if (b == a) continue;
      const double v[3] = {xyz[3 * a] - xyz[3 * b], xyz[3 * a + 1] - xyz[3 * b + 1], xyz[3 * a + 2] - xyz[3 * b + 2]};
      const double rab = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (rab < 1e-14) continue;
      const double mu = clampd((ra - dr[b]) / rab, -1.0, 1.0);
      const double slope = dsmu[(size_t)a * n + b];
      if (std::fabs(slope) < 1e-30) continue;
      const double pa = prod_except(a, b), pb = prod_except(b, a);
      for (int q = 0; q < 3; ++q) {
        const double ds = slope * (dra[q] - mu * v[q] / rab) / rab;
        dzs[q] += pa * ds - pb * ds;
        if (b == host) dph[q] += -pb * ds;
      }
    }
    for (int q = 0; q < 3; ++q) {
      const double dw = pref * (dph[q] - wn * dzs[q]);
      grad[3 * a + q] += dw;
      hacc[q] -= dw;
    }
  }
  for (int q = 0; q < 3; ++q) grad[3 * host + q] += hacc[q];
}

void xc_gradient(const Basis& bs, const std::vector<GridPoint>& pts, int n_atoms, const int* z, const double* xyz,
                 const double* Pa, const double* Pb, int func, int parts, double* grad) {
  // vxc.rs:1769-1900 (xc_nuclear_gradient_cpu), one pass over the points; parts: 1 = AO terms
  // (with the host-atom term), 2 = Becke weight term, 3 = both
  const int n = bs.n_ao;
  std::fill(grad, grad + 3 * n_atoms, 0.0);
  if (n_atoms <= 1) return;
  std::vector<int> atom_of(n);
  for (const Shell& sh : bs.shells)
    for (int c = 0; c < sh.ncomp(); ++c) atom_of[sh.ao_offset + c] = sh.atom;
  std::vector<double> h(10 * (size_t)n), sa(n), sb(n), ga(3 * (size_t)n), gb(3 * (size_t)n);
  for (const GridPoint& gp : pts) {
    if (std::fabs(gp.raw_w) < 1e-24) continue;
    const double r[3] = {gp.x, gp.y, gp.z};
    eval_aos_hess_all(bs, r, h.data());
    double ra = 0, rb = 0, gra[3] = {0, 0, 0}, grb[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
      double s1 = 0, s2 = 0, a3[3] = {0, 0, 0}, b3[3] = {0, 0, 0};
      for (int j = 0; j < n; ++j) {
        const double pa = Pa[(size_t)i * n + j], pb = Pb[(size_t)i * n + j];
        s1 += pa * h[10 * j];
        s2 += pb * h[10 * j];
        for (int q = 0; q < 3; ++q) {
          a3[q] += pa * h[10 * j + 1 + q];
          b3[q] += pb * h[10 * j + 1 + q];
        }
      }
      sa[i] = s1;
      sb[i] = s2;
      for (int q = 0; q < 3; ++q) {
        ga[3 * i + q] = a3[q];
        gb[3 * i + q] = b3[q];
      }
      ra += h[10 * i] * s1;
      rb += h[10 * i] * s2;
      for (int q = 0; q < 3; ++q) {
        gra[q] += 2.0 * h[10 * i + 1 + q] * s1;
        grb[q] += 2.0 * h[10 * i + 1 + q] * s2;
      }
    }
    ra = std::max(ra, 0.0);
    rb = std::max(rb, 0.0);
    if (ra + rb < 1e-18) continue;
    const double gaa = gra[0] * gra[0] + gra[1] * gra[1] + gra[2] * gra[2];
    const double gab = gra[0] * grb[0] + gra[1] * grb[1] + gra[2] * grb[2];
    const double gbb = grb[0] * grb[0] + grb[1] * grb[1] + grb[2] * grb[2];
    const XcOut o = eval_xc(func, ra, rb, gaa, gab, gbb);
    const double w = gp.w;
    if ((parts & 1) && std::fabs(w) > 1e-24) {
      double ua[3], ub[3];
      for (int q = 0; q < 3; ++q) {
        ua[q] = 2.0 * o.vgaa * gra[q] + o.vgab * grb[q];
        ub[q] = 2.0 * o.vgbb * grb[q] + o.vgab * gra[q];
      }
      double sum[3] = {0, 0, 0};
      static const int hidx[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};
      for (int i = 0; i < n; ++i) {
        const double* hi = h.data() + 10 * i;
        if (hi[0] == 0 && hi[1] == 0 && hi[2] == 0 && hi[3] == 0 && hi[4] == 0 && hi[5] == 0 && hi[6] == 0 &&
            hi[7] == 0 && hi[8] == 0 && hi[9] == 0)
          continue;
        const double uga = ua[0] * ga[3 * i] + ua[1] * ga[3 * i + 1] + ua[2] * ga[3 * i + 2];
        const double ugb = ub[0] * gb[3 * i] + ub[1] * gb[3 * i + 1] + ub[2] * gb[3 * i + 2];
        for (int q = 0; q < 3; ++q) {
          const double dq = hi[1 + q];
          const double uha = ua[0] * hi[hidx[q][0]] + ua[1] * hi[hidx[q][1]] + ua[2] * hi[hidx[q][2]];
          const double uhb = ub[0] * hi[hidx[q][0]] + ub[1] * hi[hidx[q][1]] + ub[2] * hi[hidx[q][2]];
          const double ta = o.vra * dq * sa[i] + uha * sa[i] + dq * uga;
          const double tb = o.vrb * dq * sb[i] + uhb * sb[i] + dq * ugb;
          const double f = -2.0 * w * (ta + tb);
          grad[3 * atom_of[i] + q] += f;
          sum[q] += f;
        }
      }
      for (int q = 0; q < 3; ++q) grad[3 * gp.host + q] -= sum[q];
    }
    if (parts & 2) becke_weight_gradient(n_atoms, z, xyz, gp.host, r, gp.raw_w, o.f, grad);
  }
}

struct OrcGrid { std::vector<GridPoint> pts; };

void* orc_grid_build(int n_atoms, const int* z, const double* xyz_bohr, int level, int radial_min) {
  auto* g = new OrcGrid;
  g->pts = build_grid(n_atoms, z, xyz_bohr, level, radial_min);
  return g;
}

void* orc_grid_from_points(int n, const double* xyzw, const int* host) {
  auto* g = new OrcGrid;
  g->pts.resize(n);
  for (int i = 0; i < n; ++i) g->pts[i] = {xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2], xyzw[4 * i + 3], 0.0, host[i]};
  return g;
}

// As orc_grid_from_points with the weights before the Becke partition (for the gradient).
void* orc_grid_from_points_raw(int n, const double* xyzw, const double* raw_w, const int* host) {
  auto* g = new OrcGrid;
  g->pts.resize(n);
  for (int i = 0; i < n; ++i)
    g->pts[i] = {xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2], xyzw[4 * i + 3], raw_w[i], host[i]};
  return g;
}

int orc_grid_size(void* g) { return (int)static_cast<OrcGrid*>(g)->pts.size(); }

void orc_grid_points(void* gp, double* xyzw, double* raw_w, int* host) {
  auto* g = static_cast<OrcGrid*>(gp);
  for (size_t i = 0; i < g->pts.size(); ++i) {
    const GridPoint& p = g->pts[i];
    xyzw[4 * i] = p.x; xyzw[4 * i + 1] = p.y; xyzw[4 * i + 2] = p.z; xyzw[4 * i + 3] = p.w;
    if (raw_w) raw_w[i] = p.raw_w;
    if (host) host[i] = p.host;
  }
}

void orc_grid_free(void* g) { delete static_cast<OrcGrid*>(g); }

double orc_becke_weight(int n_atoms, const int* z, const double* xyz, int host, const double* r) {
  BeckeTable t(n_atoms, z, xyz);
  std::vector<double> d(n_atoms), s(n_atoms);
  std::vector<int> act;
  return becke_weight_fast(t, d, s, act, host, r);
}

void* orc_basis_create(int n_shells, const int* ls, const int* atoms, const double* centers, const int* nprims,
                       const double* exps, const double* coefs) {
  return new Basis(make_basis(n_shells, ls, atoms, centers, nprims, exps, coefs));
}
int orc_basis_nao(void* b) { return static_cast<Basis*>(b)->n_ao; }
void orc_basis_free(void* b) { delete static_cast<Basis*>(b); }

// Per shell: r2_cut; per primitive: weighted norm; per AO: comp scale.
void orc_basis_shell_data(void* bp, double* r2cut, double* wnorm, double* comp_scale) {
  const Basis& b = *static_cast<Basis*>(bp);
  size_t p = 0;
  for (size_t s = 0; s < b.shells.size(); ++s) {
    r2cut[s] = b.shells[s].r2_cut;
    for (double w : b.shells[s].wnorm) wnorm[p++] = w;
    for (int c = 0; c < b.shells[s].ncomp(); ++c) comp_scale[b.shells[s].ao_offset + c] = b.shells[s].comp_scale[c];
  }
}

// AO values/gradients at points (all shells, filtered as eval_aos_grad): out[g][mu][4]
void orc_ao_grad(void* bp, int npts, const double* xyz, double* out) {
  const Basis& b = *static_cast<Basis*>(bp);
  std::vector<int> all(b.shells.size());
  for (size_t s = 0; s < all.size(); ++s) all[s] = (int)s;
  std::memset(out, 0, sizeof(double) * 4 * (size_t)npts * b.n_ao);
  std::vector<AoVal> act;
  for (int g = 0; g < npts; ++g) {
    eval_aos_grad(b, all, xyz + 3 * g, act);
    for (const AoVal& a : act) {
      double* o = out + ((size_t)g * b.n_ao + a.mu) * 4;
      o[0] = a.v; o[1] = a.gx; o[2] = a.gy; o[3] = a.gz;
    }
  }
}

void orc_ao_hess(void* bp, int npts, const double* xyz, double* out) {
  const Basis& b = *static_cast<Basis*>(bp);
  for (int g = 0; g < npts; ++g) eval_aos_hess_all(b, xyz + 3 * g, out + (size_t)g * 10 * b.n_ao);
}

// XC nuclear gradient dExc/dR (Eh/Bohr, [n_atoms][3]) at fixed Pa, Pb, for a grid built by
// orc_grid_build (raw weights and host atoms) of the molecule (z, xyz).
void orc_xc_gradient(void* bp, void* gp, int n_atoms, const int* z, const double* xyz, const double* Pa,
                     const double* Pb, int func, int parts, double* grad) {
  xc_gradient(*static_cast<Basis*>(bp), static_cast<OrcGrid*>(gp)->pts, n_atoms, z, xyz, Pa, Pb, func, parts, grad);
}

// CAM-B3LYP attenuated exchange of one spin (xc.rs:910-944): out = (f, v_rho, v_gamma).
void orc_cam_x_one(double rho, double gamma, double* out) { cam_x_one(rho, gamma, out[0], out[1], out[2]); }

// eval_xc_spin for arrays of points: in[g][5] -> out[g][6]
void orc_eval_xc(int func, int npts, const double* in, double* out) {
  for (int g = 0; g < npts; ++g) {
    const double* i = in + 5 * g;
    const XcOut o = eval_xc(func, i[0], i[1], i[2], i[3], i[4]);
    double* p = out + 6 * g;
    p[0] = o.f; p[1] = o.vra; p[2] = o.vrb; p[3] = o.vgaa; p[4] = o.vgab; p[5] = o.vgbb;
  }
}

void orc_lyp(const double* in, double* out) {
  const XcOut o = lyp_c(in[0], in[1], in[2], in[3], in[4]);
  out[0] = o.f; out[1] = o.vra; out[2] = o.vrb; out[3] = o.vgaa; out[4] = o.vgab; out[5] = o.vgbb;
}

void orc_vxc_rks_points(void* bp, void* gp, const double* P, int func, int threads, double* exc, double* nelec,
                        double* V) {
  vxc_rks_points(*static_cast<Basis*>(bp), static_cast<OrcGrid*>(gp)->pts, P, func,
                 threads > 0 ? threads : n_threads(), exc, nelec, V);
}

void orc_vxc_uks_points(void* bp, void* gp, const double* Pa, const double* Pb, int func, int threads, double* exc,
                        double* nea, double* neb, double* Va, double* Vb) {
  vxc_uks_points(*static_cast<Basis*>(bp), static_cast<OrcGrid*>(gp)->pts, Pa, Pb, func,
                 threads > 0 ? threads : n_threads(), exc, nea, neb, Va, Vb);
}

// cap_bytes < 0 selects the reference default (2560 MiB, vxc.rs:612).
void* orc_rks_engine_create(void* bp, void* gp, double cap_bytes, int threads) {
  if (cap_bytes < 0) cap_bytes = 2560.0 * 1024 * 1024;
  return rks_engine_create(*static_cast<Basis*>(bp), static_cast<OrcGrid*>(gp)->pts, cap_bytes,
                           threads > 0 ? threads : n_threads());
}
int orc_rks_engine_is_cached(void* e) { return static_cast<RksEngine*>(e)->cached ? 1 : 0; }
double orc_rks_engine_cache_bytes(void* e) { return static_cast<RksEngine*>(e)->cache_bytes; }
int orc_rks_engine_n_batches(void* e) { return (int)static_cast<RksEngine*>(e)->batches.size(); }
double orc_rks_engine_work(void* e) { return static_cast<RksEngine*>(e)->work; }
void orc_rks_engine_evaluate(void* e, const double* P, int func, int threads, double* exc, double* nelec, double* V,
                             int batch_begin, int batch_end, int blocked) {
  rks_engine_evaluate(*static_cast<RksEngine*>(e), P, func, threads > 0 ? threads : n_threads(), exc, nelec, V,
                      batch_begin, batch_end, blocked != 0);
}
void orc_rks_engine_free(void* e) { delete static_cast<RksEngine*>(e); }

void orc_overlap(void* bp, double* S) { overlap_matrix(*static_cast<Basis*>(bp), S); }

int orc_max_threads() { return n_threads(); }

}  // extern "C"
