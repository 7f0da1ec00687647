// launch.h -- host-side launchers of the device kernels, shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace cxc {
// FP64 form (vxc_fp64.cu)
cudaError_t launch_fp64(const DevGrid& G, const EvalArgs& A, int n_ctas, cudaStream_t st);
size_t fp64_smem_bytes();
// Per-molecule deterministic (Exc, N_a, N_b) sums: batches [batch_off[i], batch_off[i + 1]) go to
// out[i * n_out ...]; batch_off = nullptr for one molecule.
cudaError_t launch_reduce(const double* part, int n_batches, const int* batch_off, int n_mols, double* out, int n_out,
                          cudaStream_t st);
cudaError_t launch_reduce(const double* part, int n_batches, double* out, int n_out, cudaStream_t st);
// Symmetric completion of each molecule's Vxc block (mol_n / mol_off = nullptr for one molecule).
cudaError_t launch_mirror(double* V, int max_n, const int* mol_n, const long long* mol_off, int n_mols, int from_upper,
                          cudaStream_t st);
cudaError_t launch_mirror(double* V, int n, int from_upper, cudaStream_t st);
// Per-atom (Exc, tr(D Vxc)) shares: out[2 a ..] = sums of point_out over atom a's points.
cudaError_t launch_atom_shares(const double* point_out, const int* atom_pts, const int* atom_off, int n_atoms,
                               double* out, cudaStream_t st);
// Tensor-core form (vxc_mixed.cu)
int mixed_supported(int mode);
size_t mixed_slab_doubles(int max_m);
int mixed_ctas_per_sm(int tile_n);
int mixed_max_m();
cudaError_t launch_closed_shell_points(int xc, int precision, int n, const double* rho, const double* gam,
                                       double* out, cudaStream_t st);
cudaError_t launch_mixed(const DevGrid& G, const EvalArgs& A, int n_ctas, cudaStream_t st);
cudaError_t launch_mixed_prepare(const double* P, int n_total, const int* mol_n, const long long* mol_off,
                                 const int* mol_ao_off, int n_mols, void* out, int* fexp, cudaStream_t st);
// TD-DFT kernel coefficients per point (fxc.cu): rho_grad [n][4] of the total density -> out [n][11].
cudaError_t launch_fxc_coef(const double* rho_grad, const double* w, int n_pts, int code, double* out,
                            cudaStream_t st);
// XC nuclear gradient (xc_grad.cu): per-CTA scratch, shared memory, the persistent kernel and the
// batch-ordered sum of its [batch][atom][3] partials into grad.
size_t grad_slab_doubles(int max_m, int n_atoms);
size_t grad_smem_bytes(int n_atoms);
int grad_max_atoms();
cudaError_t launch_xc_grad(const DevGrid& G, const GradArgs& A, int n_ctas, cudaStream_t st);
cudaError_t launch_grad_reduce(const double* part, int n_batches, int n_atoms, double* grad, cudaStream_t st);
// Tensor-core form of the gradient (xc_grad_mixed.cu): GradArgs.Pa points at the split densities of
// launch_mixed_prepare (alpha, then beta); part must be zeroed; *status is set on a wait expiry.
size_t grad_mixed_slab_doubles(int max_m, int n_atoms);
int grad_mixed_max_m();
cudaError_t launch_xc_grad_mixed(const DevGrid& G, const GradArgs& A, int n_ctas, int* status, cudaStream_t st);
// The weight derivative of the tensor-core form as its own kernel (GradArgs.fx_out given to the
// quadrature kernel): per-CTA rows of per-atom sums in part [becke_kernel_ctas(n_pts)][3 n_atoms].
bool becke_kernel_fits(int n_atoms);
int becke_kernel_ctas(int n_pts);
cudaError_t launch_becke_mixed(const DevGrid& G, const GradArgs& A, const double* fx, double* part, cudaStream_t st);
// grad[k] += sum over rows r (in order) of part[r][k]
cudaError_t launch_grad_accumulate(const double* part, int n_rows, int n_atoms, double* grad, cudaStream_t st);
// Dynamic shared-memory limits of the persistent kernels, set once per process (the launchers call
// these; a graph capture calls them first so that no attribute is set while capturing).
cudaError_t fp64_set_attributes();
cudaError_t mixed_set_attributes();
}  // namespace cxc
