// integrals.cpp -- one- and two-electron integrals over the prepared Cartesian shells, for the SCF
// harness around the XC quadrature (kinetic, nuclear attraction, electron repulsion).
//
// McMurchie-Davidson scheme (McMurchie & Davidson, J. Comput. Phys. 26, 218 (1978)):
//   * a product of two Cartesian Gaussians is expanded in Hermite Gaussians with coefficients
//     E_t^{ij} from the recursions
//       E_0^{00} = exp(-mu X_AB^2),  mu = a b / p,  p = a + b,
//       E_t^{i+1,j} = E_{t-1}^{ij} / (2p) + X_PA E_t^{ij} + (t + 1) E_{t+1}^{ij}   (and likewise j);
//   * Coulomb integrals over Hermite Gaussians are R_{tuv}^0(alpha, R_PC), from
//       R_000^n = (-2 alpha)^n F_n(alpha R^2),
//       R_{t+1,u,v}^n = t R_{t-1,u,v}^{n+1} + X_PC R_{t,u,v}^{n+1}   (and likewise u, v);
//   * the Boys function F_n(T) = int_0^1 s^(2n) exp(-T s^2) ds is summed from its series
//     F_n(T) = exp(-T) sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) and recursed downwards for T < 35,
//     and for larger T taken from F_0 = sqrt(pi / T) erf(sqrt T) / 2 and recursed upwards.
// An AO is scale * sum_p weighted_norm_p x^l y^m z^n exp(-alpha_p r^2) exactly as the quadrature
// evaluates it (AoShellGpu / AoPrimGpu / AoCompGpu), so these integrals and the XC matrix use the
// same functions.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/calchem_xc.h"

namespace {

constexpr int kMaxL = 4;            // per shell (f has l = 3)
constexpr int kMaxN = 4 * kMaxL + 1;  // Boys orders for (ab|cd)

void boys(int nmax, double T, double* F) {
  if (T < 35.0) {
    // series for the highest order, then downward recursion
    const double a = nmax + 0.5;
    double term = 1.0 / (2.0 * a), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= T / (a + k);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    const double e = std::exp(-T);
    F[nmax] = e * sum;
    for (int n = nmax; n > 0; --n) F[n - 1] = (2.0 * T * F[n] + e) / (2.0 * n - 1.0);
  } else {
    const double e = std::exp(-T);
    F[0] = 0.5 * std::sqrt(M_PI / T) * std::erf(std::sqrt(T));
    for (int n = 0; n < nmax; ++n) F[n + 1] = ((2.0 * n + 1.0) * F[n] - e) / (2.0 * T);
  }
}

// Hermite coefficients E[i][j][t] for one Cartesian direction.
struct Herm {
  double e[kMaxL + 3][kMaxL + 3][2 * kMaxL + 6];
};

void hermite(int imax, int jmax, double a, double b, double xa, double xb, Herm& H) {
  const double p = a + b, mu = a * b / p, xab = xa - xb;
  const double xp = (a * xa + b * xb) / p, xpa = xp - xa, xpb = xp - xb, inv2p = 0.5 / p;
  std::memset(&H, 0, sizeof(H));
  H.e[0][0][0] = std::exp(-mu * xab * xab);
  for (int i = 0; i <= imax; ++i)
    for (int j = 0; j <= jmax; ++j) {
      if (i == 0 && j == 0) continue;
      for (int t = 0; t <= i + j; ++t) {
        double v;
        if (i > 0) {
          const auto& s = H.e[i - 1][j];
          v = (t > 0 ? inv2p * s[t - 1] : 0.0) + xpa * s[t] + (t + 1) * s[t + 1];
        } else {
          const auto& s = H.e[i][j - 1];
          v = (t > 0 ? inv2p * s[t - 1] : 0.0) + xpb * s[t] + (t + 1) * s[t + 1];
        }
        H.e[i][j][t] = v;
      }
    }
}

// R_{tuv}^0 for t + u + v <= L into R[t][u][v] (dimension L + 1 each).
struct RTab {
  int L;
  std::vector<double> r;  // [n][t][u][v]
  double& at(int n, int t, int u, int v) { return r[(((size_t)n * (L + 1) + t) * (L + 1) + u) * (L + 1) + v]; }
};

void hermite_coulomb(int L, double alpha, double x, double y, double z, RTab& R) {
  R.L = L;
  R.r.assign((size_t)(L + 1) * (L + 1) * (L + 1) * (L + 1), 0.0);
  double F[kMaxN + 2];
  boys(L, alpha * (x * x + y * y + z * z), F);
  double f = 1.0;
  for (int n = 0; n <= L; ++n) {
    R.at(n, 0, 0, 0) = f * F[n];
    f *= -2.0 * alpha;
  }
  for (int n = L - 1; n >= 0; --n)
    for (int t = 0; t <= L - n; ++t)
      for (int u = 0; u <= L - n - t; ++u)
        for (int v = 0; v <= L - n - t - u; ++v) {
          if (t + u + v == 0) continue;
          double val;
          if (t > 0)
            val = (t > 1 ? (t - 1) * R.at(n + 1, t - 2, u, v) : 0.0) + x * R.at(n + 1, t - 1, u, v);
          else if (u > 0)
            val = (u > 1 ? (u - 1) * R.at(n + 1, t, u - 2, v) : 0.0) + y * R.at(n + 1, t, u - 1, v);
          else
            val = (v > 1 ? (v - 1) * R.at(n + 1, t, u, v - 2) : 0.0) + z * R.at(n + 1, t, u, v - 1);
          R.at(n, t, u, v) = val;
        }
}

struct Prim {
  double a, w;  // exponent, weighted norm
};

struct ShellView {
  int l, n_funcs, ao;
  double c[3];
  std::vector<Prim> prims;
  std::vector<int> lx, ly, lz;
  std::vector<double> scale;
};

std::vector<ShellView> views(const AoShellGpu* sh, int ns, const AoPrimGpu* pr, const AoCompGpu* co) {
  std::vector<ShellView> v(ns);
  for (int s = 0; s < ns; ++s) {
    ShellView& x = v[s];
    const AoCompGpu& c0 = co[sh[s].comp_start];
    x.l = c0.lx + c0.ly + c0.lz;
    x.n_funcs = sh[s].n_funcs;
    x.ao = sh[s].ao_offset;
    for (int k = 0; k < 3; ++k) x.c[k] = sh[s].center[k];
    for (int p = 0; p < sh[s].n_prims; ++p)
      x.prims.push_back({pr[sh[s].prim_start + p].exponent, pr[sh[s].prim_start + p].weighted_norm});
    for (int c = 0; c < sh[s].n_funcs; ++c) {
      const AoCompGpu& q = co[sh[s].comp_start + c];
      x.lx.push_back(q.lx);
      x.ly.push_back(q.ly);
      x.lz.push_back(q.lz);
      x.scale.push_back(q.scale);
    }
  }
  return v;
}

bool valid(const AoShellGpu* sh, int ns, const AoCompGpu* co, int n_ao) {
  for (int s = 0; s < ns; ++s) {
    const int nf = sh[s].n_funcs;
    if (!(nf == 1 || nf == 3 || nf == 6 || nf == 10) || sh[s].ao_offset < 0 || sh[s].ao_offset + nf > n_ao ||
        sh[s].comp_start < 0)
      return false;
    const AoCompGpu& c0 = co[sh[s].comp_start];
    if (c0.lx + c0.ly + c0.lz > 3) return false;
  }
  return true;
}

}  // namespace

extern "C" {

int calchem_scf_boys(int n_max, double t, double* f_out) {
  if (n_max < 0 || n_max > kMaxN || !(t >= 0.0) || !f_out) return -1;
  boys(n_max, t, f_out);
  return 0;
}

int calchem_scf_one_electron(const AoShellGpu* shells, int n_shells, const AoPrimGpu* prims, const AoCompGpu* comps,
                             int n_ao, int n_atoms, const double* charges, const double* xyz_bohr, double* s_out,
                             double* t_out, double* v_out) {
  if (!shells || !prims || !comps || n_shells <= 0 || n_ao <= 0 || n_atoms < 0 || (n_atoms > 0 && (!charges || !xyz_bohr)))
    return -1;
  if (!valid(shells, n_shells, comps, n_ao)) return -2;
  const std::vector<ShellView> V = views(shells, n_shells, prims, comps);
  const size_t nn = (size_t)n_ao * n_ao;
  if (s_out) std::memset(s_out, 0, nn * sizeof(double));
  if (t_out) std::memset(t_out, 0, nn * sizeof(double));
  if (v_out) std::memset(v_out, 0, nn * sizeof(double));
#pragma omp parallel for schedule(dynamic)
  for (int sa = 0; sa < n_shells; ++sa) {
    Herm Hx, Hy, Hz;
    RTab R;
    for (int sb = 0; sb <= sa; ++sb) {
      const ShellView &A = V[sa], &B = V[sb];
      std::vector<double> S(A.n_funcs * B.n_funcs, 0.0), T(S.size(), 0.0), P(S.size(), 0.0);
      for (const Prim& pa : A.prims)
        for (const Prim& pb : B.prims) {
          const double a = pa.a, b = pb.a, p = a + b;
          // j + 2 for the kinetic integrals
          hermite(A.l, B.l + 2, a, b, A.c[0], B.c[0], Hx);
          hermite(A.l, B.l + 2, a, b, A.c[1], B.c[1], Hy);
          hermite(A.l, B.l + 2, a, b, A.c[2], B.c[2], Hz);
          const double pre = pa.w * pb.w;
          const double sp = std::pow(M_PI / p, 1.5);
          const double P3[3] = {(a * A.c[0] + b * B.c[0]) / p, (a * A.c[1] + b * B.c[1]) / p,
                                (a * A.c[2] + b * B.c[2]) / p};
          for (int i = 0; i < A.n_funcs; ++i)
            for (int j = 0; j < B.n_funcs; ++j) {
              const int ix = A.lx[i], iy = A.ly[i], iz = A.lz[i], jx = B.lx[j], jy = B.ly[j], jz = B.lz[j];
              auto s1 = [&](const Herm& H, int u, int w) { return w < 0 ? 0.0 : H.e[u][w][0]; };
              const double sx = s1(Hx, ix, jx), sy = s1(Hy, iy, jy), sz = s1(Hz, iz, jz);
              auto k1 = [&](const Herm& H, int u, int w) {
                return -2.0 * b * b * s1(H, u, w + 2) + b * (2 * w + 1) * s1(H, u, w) -
                       0.5 * w * (w - 1) * s1(H, u, w - 2);
              };
              const size_t o = (size_t)i * B.n_funcs + j;
              S[o] += pre * sx * sy * sz * sp;
              T[o] += pre * sp * (k1(Hx, ix, jx) * sy * sz + sx * k1(Hy, iy, jy) * sz + sx * sy * k1(Hz, iz, jz));
            }
          if (v_out) {
            const int L = A.l + B.l;
            for (int c = 0; c < n_atoms; ++c) {
              hermite_coulomb(L, p, P3[0] - xyz_bohr[3 * c], P3[1] - xyz_bohr[3 * c + 1], P3[2] - xyz_bohr[3 * c + 2],
                              R);
              const double f = -charges[c] * 2.0 * M_PI / p * pre;
              for (int i = 0; i < A.n_funcs; ++i)
                for (int j = 0; j < B.n_funcs; ++j) {
                  const int ix = A.lx[i], iy = A.ly[i], iz = A.lz[i], jx = B.lx[j], jy = B.ly[j], jz = B.lz[j];
                  double acc = 0.0;
                  for (int t = 0; t <= ix + jx; ++t)
                    for (int u = 0; u <= iy + jy; ++u)
                      for (int v = 0; v <= iz + jz; ++v)
                        acc += Hx.e[ix][jx][t] * Hy.e[iy][jy][u] * Hz.e[iz][jz][v] * R.at(0, t, u, v);
                  P[(size_t)i * B.n_funcs + j] += f * acc;
                }
            }
          }
        }
      for (int i = 0; i < A.n_funcs; ++i)
        for (int j = 0; j < B.n_funcs; ++j) {
          const size_t o = (size_t)i * B.n_funcs + j;
          const double sc = A.scale[i] * B.scale[j];
          const size_t r = (size_t)(A.ao + i), c = (size_t)(B.ao + j);
          if (s_out) s_out[r * n_ao + c] = s_out[c * n_ao + r] = sc * S[o];
          if (t_out) t_out[r * n_ao + c] = t_out[c * n_ao + r] = sc * T[o];
          if (v_out) v_out[r * n_ao + c] = v_out[c * n_ao + r] = sc * P[o];
        }
    }
  }
  return 0;
}

int calchem_scf_eri(const AoShellGpu* shells, int n_shells, const AoPrimGpu* prims, const AoCompGpu* comps, int n_ao,
                    double* eri_out) {
  if (!shells || !prims || !comps || n_shells <= 0 || n_ao <= 0 || !eri_out) return -1;
  if (n_ao > 400) return -3;  // the dense n^4 tensor is for small molecules only
  if (!valid(shells, n_shells, comps, n_ao)) return -2;
  const std::vector<ShellView> V = views(shells, n_shells, prims, comps);
  const size_t n = (size_t)n_ao;
  // shell pairs with their Hermite expansions per primitive pair, then quartets over pairs
  struct PrimPair {
    double p, w, P[3];
    Herm hx, hy, hz;
  };
  struct Pair {
    int a, b;
    std::vector<PrimPair> pp;
  };
  std::vector<Pair> pairs;
  for (int sa = 0; sa < n_shells; ++sa)
    for (int sb = 0; sb <= sa; ++sb) {
      Pair pr;
      pr.a = sa;
      pr.b = sb;
      const ShellView &A = V[sa], &B = V[sb];
      for (const Prim& x : A.prims)
        for (const Prim& y : B.prims) {
          PrimPair q;
          q.p = x.a + y.a;
          q.w = x.w * y.w;
          for (int k = 0; k < 3; ++k) q.P[k] = (x.a * A.c[k] + y.a * B.c[k]) / q.p;
          hermite(A.l, B.l, x.a, y.a, A.c[0], B.c[0], q.hx);
          hermite(A.l, B.l, x.a, y.a, A.c[1], B.c[1], q.hy);
          hermite(A.l, B.l, x.a, y.a, A.c[2], B.c[2], q.hz);
          pr.pp.push_back(q);
        }
      pairs.push_back(std::move(pr));
    }
  const int np = (int)pairs.size();
#pragma omp parallel for schedule(dynamic)
  for (int i1 = 0; i1 < np; ++i1) {
    RTab R;
    for (int i2 = 0; i2 <= i1; ++i2) {
      const Pair &ab = pairs[i1], &cd = pairs[i2];
      const ShellView &A = V[ab.a], &B = V[ab.b], &C = V[cd.a], &D = V[cd.b];
      const int L = A.l + B.l + C.l + D.l;
      const int na = A.n_funcs, nb = B.n_funcs, nc = C.n_funcs, nd = D.n_funcs;
      std::vector<double> out((size_t)na * nb * nc * nd, 0.0);
      for (const PrimPair& x : ab.pp)
        for (const PrimPair& y : cd.pp) {
          const double alpha = x.p * y.p / (x.p + y.p);
          hermite_coulomb(L, alpha, x.P[0] - y.P[0], x.P[1] - y.P[1], x.P[2] - y.P[2], R);
          const double pre = 2.0 * std::pow(M_PI, 2.5) / (x.p * y.p * std::sqrt(x.p + y.p)) * x.w * y.w;
          for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j) {
              const int ix = A.lx[i] , iy = A.ly[i], iz = A.lz[i], jx = B.lx[j], jy = B.ly[j], jz = B.lz[j];
              for (int k = 0; k < nc; ++k)
                for (int l = 0; l < nd; ++l) {
                  const int kx = C.lx[k], ky = C.ly[k], kz = C.lz[k], lx = D.lx[l], ly = D.ly[l], lz = D.lz[l];
                  double acc = 0.0;
                  for (int t = 0; t <= ix + jx; ++t)
                    for (int u = 0; u <= iy + jy; ++u)
                      for (int v = 0; v <= iz + jz; ++v) {
                        const double e1 = x.hx.e[ix][jx][t] * x.hy.e[iy][jy][u] * x.hz.e[iz][jz][v];
                        if (e1 == 0.0) continue;
                        double inner = 0.0;
                        for (int tt = 0; tt <= kx + lx; ++tt)
                          for (int uu = 0; uu <= ky + ly; ++uu)
                            for (int vv = 0; vv <= kz + lz; ++vv) {
                              const double e2 = y.hx.e[kx][lx][tt] * y.hy.e[ky][ly][uu] * y.hz.e[kz][lz][vv];
                              const double sg = ((tt + uu + vv) & 1) ? -1.0 : 1.0;
                              inner += sg * e2 * R.at(0, t + tt, u + uu, v + vv);
                            }
                        acc += e1 * inner;
                      }
                  out[(((size_t)i * nb + j) * nc + k) * nd + l] += pre * acc;
                }
            }
        }
      for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j)
          for (int k = 0; k < nc; ++k)
            for (int l = 0; l < nd; ++l) {
              const double v = out[(((size_t)i * nb + j) * nc + k) * nd + l] * A.scale[i] * B.scale[j] * C.scale[k] *
                               D.scale[l];
              const size_t p = A.ao + i, q = B.ao + j, r = C.ao + k, s = D.ao + l;
              const size_t idx[8][4] = {{p, q, r, s}, {q, p, r, s}, {p, q, s, r}, {q, p, s, r},
                                        {r, s, p, q}, {s, r, p, q}, {r, s, q, p}, {s, r, q, p}};
              for (auto& x4 : idx) eri_out[((x4[0] * n + x4[1]) * n + x4[2]) * n + x4[3]] = v;
            }
    }
  }
  return 0;
}

}  // extern "C"
