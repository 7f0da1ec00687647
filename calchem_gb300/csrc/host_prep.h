// host_prep.h -- host-side preparation routines (see host_prep.cpp).
#pragma once

#include <vector>

#include "../../include/calchem_xc.h"

namespace cxc {

constexpr int kPlanBatch = 128;

double gto_norm(double alpha, int l, int m, int n);
int prepare_shells(int n_shells, const int* l, const int* atom, const double* centers, const int* n_prims,
                   const double* exps, const double* coefs, AoShellGpu* so, AoPrimGpu* po, AoCompGpu* co,
                   int* n_ao_out);
void overlap_matrix(const AoShellGpu* sh, int n_shells, const AoPrimGpu* pr, const AoCompGpu* co, int n_ao,
                    double* S);

struct LebedevTables {
  std::vector<double> xyzw;  // concatenated rules, 4 doubles per point
  int offset[6];
  int count[6];
};
const LebedevTables& lebedev_tables();
int lebedev_index(int npts);

double bragg_slater_bohr(int z);
double becke_shift(int zc, int zd);
int radial_count(int z, int level);
int angular_points(double r, double rbs, int level);

struct RadialShell {
  int atom;
  int leb_offset;
  int n_ang;
  int pad;
  double r;
  double w_rad;
  long long raw_start;
};
void radial_shells(int n_atoms, const int* z, int level, int radial_min, std::vector<RadialShell>& out,
                   long long* n_raw);
// Per-atom grids: atom a gets n_rad[a] Euler-Maclaurin shells (<= 0: the Fine count); a shell at
// x = r / max(R_BS, 0.3) takes region_leb[5 a + k] Lebedev points in the Fine level's pruning region
// k (x < 0.18, 0.5, 0.95, 5, beyond; <= 0: the Fine choice 50 / 110 / 194 / 302 / 194), and shells
// with x > x_max[a] are left out (x_max[a] <= 0: none).
void radial_shells_atoms(int n_atoms, const int* z, const int* n_rad, const int* region_leb, const double* x_max,
                         std::vector<RadialShell>& out, long long* n_raw);
void becke_tables(int n, const int* z, const double* xyz, std::vector<double>& inv_r, std::vector<double>& a_ij);

// Reference-layout batch plan (what RksVxcEngine::new_with_gpu uploads, vxc.rs:497-545).
struct Plan {
  std::vector<GridPtGpu> pts;
  std::vector<double> weights;
  std::vector<int> cand_offsets;
  std::vector<int> cand_shells;
  std::vector<int> orig;  // index of every kept point in the caller's point array
};
// Chunks of batch_pts consecutive points (kPlanBatch = 128 in the reference, vxc.rs:96).
int plan_batches(const AoShellGpu* shells, int n_shells, const double* xyzw, int n_pts, Plan& plan,
                 int batch_pts = kPlanBatch);
// Value screen of the compact plan: a candidate shell is dropped from a batch when a bound on every
// component's |phi| and |grad phi| stays below `floor` at all of the batch's points.  With floor
// kZeroFloor (1e-17) the dropped shells are exactly zero at those points in every form of the
// quadrature (the reference zeroes components whose value and gradient are all <= 1e-16,
// ao_grid.rs:182-230), so results change only by the order of additions of zeros; a larger floor is
// an approximation that the caller chooses.
constexpr double kZeroFloor = 1e-17;
struct ValueScreen {
  const AoPrimGpu* prims;
  const AoCompGpu* comps;
  int n_prims, n_comps;
  double floor;
};
// Spatially compact batches: the kept points ordered by recursive bisection (leaves of batch_pts
// points), then chunked; candidates by the reference's rule, narrowed to the shells that reach at
// least one point of the batch (and, with vs, whose values reach vs->floor there).  Every point sees
// the same nonzero AOs as under plan_batches.
int plan_batches_spatial(const AoShellGpu* shells, int n_shells, const double* xyzw, int n_pts, Plan& plan,
                         int batch_pts = kPlanBatch, const ValueScreen* vs = nullptr);

}  // namespace cxc
