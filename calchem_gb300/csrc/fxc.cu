// fxc.cu -- per-point coefficients of the TD-DFT exchange-correlation kernel (FxcKernel::new,
// crates/calchem-dft/src/fxc.rs:176-366).
//
// For the ground-state total density at every grid point (rho, grad rho from the FP64 kernel's
// density mode), the kernel's second derivatives are taken, as in the reference, by finite
// differences of the spin-resolved first derivatives (the same FP64 functionals):
//   singlet (alpha and beta perturbed alike), steps h_r = 1e-5 rho_s and h_g = 1e-5 gamma_s,
//     k_rr = d v_rho_a / d rho_s,   k_rg = d u / d rho_s,   k_gg = 2 d u / d gamma_s,
//     u = 2 v_gamma_aa + v_gamma_ab,  u_iso = u at the point   (4-point central differences);
//   triplet (alpha and beta perturbed oppositely),
//     k_rr = d [(v_rho_a - v_rho_b) / 2] / d tau,   k_rg = d (v_gamma_aa - v_gamma_bb) / d tau,
//     k_gg = 2 d (v_gamma_aa - v_gamma_bb) / d zeta,   u_iso = 2 v_gamma_aa - v_gamma_ab
//     (odd in the perturbation, so the two-point formula (8 f(h) - f(2h)) / (6 h) is used);
// gradient terms only for GGA functionals, k_gg only where gamma_s > 1e-28.  Points with |w| < 1e-22
// or rho < 1e-12 get all-zero coefficients (the reference drops them; they contribute nothing).
#include <cuda_runtime.h>

#include "common.cuh"
#include "xc_device.cuh"

namespace cxc {

namespace {

__device__ __noinline__ XcVal xc_eval_call(int code, double ra, double rb, double gaa, double gab, double gbb) {
  return xc_eval(code, ra, rb, gaa, gab, gbb);
}

__global__ void __launch_bounds__(128) fxc_coef_kernel(const double* __restrict__ rho_grad,
                                                       const double* __restrict__ w, int n_pts, int code,
                                                       double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pts) return;
  double c[11];
#pragma unroll
  for (int k = 0; k < 11; ++k) c[k] = 0.0;
  const double rho_t = rho_grad[4 * (size_t)i];
  if (!(fabs(w[i]) < 1e-22) && !(rho_t < 1e-12)) {
    const bool gga = code != 0;
    const double rs = 0.5 * rho_t;
    const double gs[3] = {0.5 * rho_grad[4 * (size_t)i + 1], 0.5 * rho_grad[4 * (size_t)i + 2],
                          0.5 * rho_grad[4 * (size_t)i + 3]};
    const double gam = gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2];
    const XcVal o0 = xc_eval_call(code, rs, rs, gam, gam, gam);
    const double hr = 1e-5 * rs;
    double vr[4], ug[4];
    const double off[4] = {-2.0, -1.0, 1.0, 2.0};
    for (int k = 0; k < 4; ++k) {
      const double r = rs + off[k] * hr;
      const XcVal o = xc_eval_call(code, r, r, gam, gam, gam);
      vr[k] = o.vra;
      ug[k] = 2.0 * o.vgaa + o.vgab;
    }
    const double inv12 = 1.0 / (12.0 * hr);
    c[0] = gs[0];
    c[1] = gs[1];
    c[2] = gs[2];
    c[3] = (vr[0] - 8.0 * vr[1] + 8.0 * vr[2] - vr[3]) * inv12;
    if (gga) {
      c[4] = (ug[0] - 8.0 * ug[1] + 8.0 * ug[2] - ug[3]) * inv12;
      c[6] = 2.0 * o0.vgaa + o0.vgab;
      if (gam > 1e-28) {
        const double hg = 1e-5 * gam;
        double u[4];
        for (int k = 0; k < 4; ++k) {
          const double g = gam + off[k] * hg;
          const XcVal o = xc_eval_call(code, rs, rs, g, g, g);
          u[k] = 2.0 * o.vgaa + o.vgab;
        }
        c[5] = 2.0 * (u[0] - 8.0 * u[1] + 8.0 * u[2] - u[3]) / (12.0 * hg);
      }
    }
    // triplet
    const XcVal t1 = xc_eval_call(code, rs + hr, rs - hr, gam, gam, gam);
    const XcVal t2 = xc_eval_call(code, rs + 2.0 * hr, rs - 2.0 * hr, gam, gam, gam);
    const double inv6 = 1.0 / (6.0 * hr);
    c[7] = (8.0 * (0.5 * (t1.vra - t1.vrb)) - 0.5 * (t2.vra - t2.vrb)) * inv6;
    if (gga) {
      c[8] = (8.0 * (t1.vgaa - t1.vgbb) - (t2.vgaa - t2.vgbb)) * inv6;
      c[10] = 2.0 * o0.vgaa - o0.vgab;
      if (gam > 1e-28) {
        const double hg = 1e-5 * gam;
        const XcVal z1 = xc_eval_call(code, rs, rs, gam + hg, gam, gam - hg);
        const XcVal z2 = xc_eval_call(code, rs, rs, gam + 2.0 * hg, gam, gam - 2.0 * hg);
        c[9] = 2.0 * (8.0 * (z1.vgaa - z1.vgbb) - (z2.vgaa - z2.vgbb)) / (6.0 * hg);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 11; ++k) out[11 * (size_t)i + k] = c[k];
}

}  // namespace

cudaError_t launch_fxc_coef(const double* rho_grad, const double* w, int n_pts, int code, double* out,
                            cudaStream_t st) {
  fxc_coef_kernel<<<(n_pts + 127) / 128, 128, 0, st>>>(rho_grad, w, n_pts, code, out);
  return cudaGetLastError();
}

}  // namespace cxc
