// common.cuh -- device data model shared by the grid, FP64 and tensor-core Vxc kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/calchem_xc.h"

namespace cxc {

constexpr int kBlockPts = 128;  // points per batch (vxc.rs:96)

// One batch of <= 128 consecutive grid points and the shells that can touch it.
// Built on the host from the reference's batching rules (vxc.rs:443-493).
struct BatchDesc {
  int pt_start;    // first point (index into the point arrays)
  int n_pts;       // points in the batch (<= 128)
  int cand_start;  // first entry in cand_shells / cand_loc
  int n_cand;      // candidate shells
  int ao_start;    // first entry in batch_ao (local AO -> global AO)
  int m;           // AOs of the candidate shells
  int mol;         // molecule of the batch in a multi-molecule grid (0 otherwise)
  int pad1;
};

// Evaluation modes of the block kernels.
enum Mode : int {
  kModeRho = 0,   // drop-in eval_rho: write rho and grad rho per point
  kModeAccum = 1, // drop-in accum: read (w v_rho / 2, w u) per point, add into V (lower triangle)
  kModeRks = 2,   // fused closed shell
  kModeUks = 3,   // fused open shell
  kModeFxc = 4    // TD-DFT kernel contraction: per trial matrix M_b, dV_b = f_xc[M_b] (fxc.rs:374-645)
};

struct DevGrid {
  int n_pts, n_ao, n_shells, n_batches;
  const AoShellGpu* shells;
  const AoPrimGpu* prims;
  const AoCompGpu* comps;
  const double* px;  // point coordinates and weights (SoA)
  const double* py;
  const double* pz;
  const double* pw;
  const BatchDesc* batches;
  const int* cand_shells;  // shell index per candidate
  const int* cand_loc;     // local AO row of the candidate's first component
  const int* batch_ao;     // global AO per local row
  const int* order;        // batch processing order (cost descending)
  // Basis constants as float pairs (hi + lo) for the FP32 AO evaluation of the tensor-core path:
  // (exponent hi, exponent lo, weighted norm hi, weighted norm lo) per primitive and
  // (scale hi, scale lo) per Cartesian component.
  const float4* prim_f;
  const float2* comp_f;
  const float2* shell_cf;  // shell centres as float pairs, 3 per shell (x, y, z)
  // Multi-molecule grids: molecule i has mol_n[i] AOs, its density and Vxc are the mol_n[i]^2
  // block starting at element mol_off[i] of the packed matrices, and its rows start at
  // mol_ao_off[i] of packed per-AO vectors.  nullptr for a single molecule (n_ao AOs, offset 0).
  const int* mol_n;
  const long long* mol_off;
  const int* mol_ao_off;
  long long nn_total;  // elements of the packed matrices (n_ao^2 for a single molecule)
  int n_total;         // rows of the packed matrices (n_ao for a single molecule)
};

__device__ __forceinline__ int mol_nao(const DevGrid& G, int mol) { return G.mol_n ? G.mol_n[mol] : G.n_ao; }
__device__ __forceinline__ long long mol_mat(const DevGrid& G, int mol) { return G.mol_off ? G.mol_off[mol] : 0ll; }
__device__ __forceinline__ int mol_row(const DevGrid& G, int mol) { return G.mol_ao_off ? G.mol_ao_off[mol] : 0; }

struct EvalArgs {
  int mode;
  int xc;
  const double* Pa;   // density (RKS: total)
  const double* Pb;   // beta density (UKS)
  double* Va;         // output (lower triangle accumulated)
  double* Vb;
  double* rho_out;    // kModeRho: 4 per point
  const double* wv_in;  // kModeAccum: 4 per point
  double* batch_red;  // per batch: exc, nelec_a, nelec_b
  int* counter;       // work-queue head
  double* slab;       // per-CTA scratch
  size_t slab_stride; // doubles per CTA
  int max_m;
  // Optional per-point output of the fused RKS modes (nullptr: none): point_out[2 g] = w_g f_g and
  // point_out[2 g + 1] = w_g (v_rho rho + v_gamma |grad rho|^2), the point's share of Exc and of
  // tr(D Vxc).  Points below the density floor are not written (the caller zeroes the buffer).  The
  // tensor-core form sums grad rho with compensation in builds with point_out (the shares' accuracy)
  // and by FP32 FMAs without it.
  double* point_out;
  // With point_out in the closed-shell mode: nonzero skips the Vxc contraction (the per-point shares,
  // Exc and Nelec only; V is neither read nor written).
  int shares_only;
  // Tensor-core form: GEMM1 N chunk, 64 (two CTAs per SM) or 128 (one CTA per SM, 512 TMEM columns).
  int tile_n;
  // kModeFxc: n_trials matrices at Pa + b n^2, results at Va + b n^2; per-point kernel coefficients
  // fxc_coef[11 g ..] = (g_s x, y, z, singlet k_rr, k_rg, k_gg, u_iso, triplet k_rr, k_rg, k_gg, u_iso).
  int n_trials;
  int triplet;
  const double* fxc_coef;
  // Tensor-core form: the AO cache (nullptr: none).  Batch b's AO planes, packed GEMM1 operand and
  // row exponents live at ao_cache + ao_cache_off[b] (ao_cache_block_bytes; -1: the batch has no
  // block and is evaluated in the CTA's slab every time); ao_cache_ok[b] != 0 once a launch has
  // written them, and later launches read them instead of evaluating the AOs.
  unsigned char* ao_cache;
  const long long* ao_cache_off;
  int* ao_cache_ok;
};

// Bytes of one batch's AO-cache block for m AOs: with m_k = m rounded up to 64, four FP32 planes
// and four BF16 planes [m_k][128] (24 B per AO and point), the packed operand (m_k / 64 blocks of
// 64 KB) and 128 row exponents, rounded up to 1 KB.
inline size_t ao_cache_block_bytes(int m) {
  const size_t m_k = (size_t)(m + 63) / 64 * 64;
  return (m_k * 128 * 24 + m_k * 1024 + 512 + 1023) / 1024 * 1024;
}

// XC nuclear gradient (xc_grad.cu).  xc >= 0: fused form (densities, functional, AO and Becke
// terms); xc < 0: drop-in form, per-point coefficients wxc[8 g ..] = (w v_rho_a, w u_a, w v_rho_b,
// w u_b) from the caller and the AO term only.
constexpr int kMaxGradAtoms = 1024;

struct GradArgs {
  int xc;
  int closed;              // beta density = alpha density (Pb unused)
  const double* Pa;        // spin densities (n x n)
  const double* Pb;
  const double* wxc;       // drop-in form: 8 per point
  const double* raw_w;     // per point: weight before the Becke partition (fused form)
  const int* host;         // per point: host atom
  const int* ao_atom;      // per AO: atom of its shell
  const double* xyz;       // atoms, Bohr (3 n_atoms)
  const double* inv_r;     // n_atoms^2 inverse distances (0: coincident)
  const double* a_ij;      // n_atoms^2 Becke size adjustments
  const int2* pairs;       // the atom pairs (c, d), c < d
  int n_pairs;
  // per ordered pair (a, b), 5 float pairs (hi, lo): 1 / R_ab, a_ab, (R_a - R_b) / R_ab (the
  // double-float weight derivative of the tensor-core form)
  const float2* pair_df;
  // tensor-core form: when set, the quadrature kernel writes each point's energy density f here and
  // leaves the weight derivative to a separate kernel (becke_mixed_kernel)
  double* fx_out;
  int n_atoms;
  int max_m;
  double* part;            // [batch][atom][3] partial sums
  int* counter;            // work-queue head (zeroed by the caller)
  double* slab;            // per-CTA scratch
  size_t slab_stride;      // doubles per CTA
};

}  // namespace cxc
