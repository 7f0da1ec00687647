// grid_build.h -- device-side molecular grid construction (see grid_build.cu).
#pragma once

#include <cuda_runtime.h>

namespace cxc {

struct RadialShellDev {
  int atom;
  int leb_offset;
  int n_ang;
  int pad;
  double r;
  double w_rad;
  long long raw_start;
};

struct GridBuildArgs {
  int n_atoms;
  const double* xyz;      // atoms, Bohr
  const double* inv_r;    // n x n inverse distances (0 for coincident atoms)
  const double* a_ij;     // n x n Becke size adjustments
  const double* lebedev;  // concatenated rules, (x, y, z, w) per point
  const RadialShellDev* shells;
  double* raw;            // 4 per raw point
  double* raw_w;          // 1 per raw point
  unsigned char* flags;   // keep flag per raw point
  int* counts;            // kept per shell
  double* out_xyzw;
  double* out_raw_w;
  int* out_host;
};

cudaError_t launch_grid_expand(const GridBuildArgs& a, int n_shells, cudaStream_t st);
cudaError_t launch_grid_scan(const int* counts, int n, long long* offsets, cudaStream_t st);
cudaError_t launch_grid_compact(const GridBuildArgs& a, const long long* offsets, int n_shells, cudaStream_t st);

}  // namespace cxc
