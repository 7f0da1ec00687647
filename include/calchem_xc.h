/*
 * calchem_xc.h -- C ABI of the GB300 (sm_103a) exchange-correlation quadrature library
 * (libcalchem_xc.so).
 *
 * The library replaces CalChem's `calchem-cuda` Vxc path.  It keeps the reference's FFI
 * contract exactly, so CalChem's Rust `GpuVxcGrid` links against it unchanged, and it adds
 * fused entry points that compute (Exc, Nelec, Vxc) in one call with no CPU work in between.
 *
 * Conventions shared by every function (crates/calchem-cuda/src/cuda_kernels.cu:7354-7562):
 *   return 0 on success, otherwise
 *    -1  bad arguments (null pointer, non-positive size, unknown functional/precision code)
 *    -2  unknown grid id, size mismatch with the uploaded grid, or a size overflow
 *    -3  no usable CUDA device, or the request exceeds the caller's memory budget
 *    -4  device allocation failure
 *    -5  copy or kernel launch failure
 *    -6  device-side overflow flag (kept for compatibility; the kernels here never set it)
 *    -7  a device-side wait gave up (bounded spin expired); the result is not valid
 *   All matrices are dense row-major n_ao x n_ao doubles.  Every call is synchronous with
 *   respect to the host buffers it is given and is serialised by one process-wide mutex, as in
 *   the reference.  There is never a CPU fallback: a failure is reported, not recomputed.
 */
#ifndef CALCHEM_XC_H
#define CALCHEM_XC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Data layouts, identical to crates/calchem-cuda/src/lib.rs:46-84 (#[repr(C)]). ---- */
typedef struct AoShellGpu {
  double center[3];
  double r2_cutoff;
  int ao_offset;
  int n_funcs;
  int prim_start;
  int n_prims;
  int comp_start;
  int atom_index;
} AoShellGpu; /* 56 bytes */

typedef struct AoPrimGpu {
  double exponent;
  double weighted_norm;
} AoPrimGpu; /* 16 bytes */

typedef struct AoCompGpu {
  double scale;
  int lx, ly, lz, _pad;
} AoCompGpu; /* 24 bytes */

typedef struct GridPtGpu {
  double x, y, z;
  int batch_id;
  int host_atom;
} GridPtGpu; /* 32 bytes */

/* Functional codes, in the order of CalChem's XcFunctional enum (crates/calchem-dft/src/xc.rs:16-35). */
enum {
  CALCHEM_XC_SVWN5 = 0,
  CALCHEM_XC_BLYP = 1,
  CALCHEM_XC_PBE = 2,
  CALCHEM_XC_B3LYP = 3,  /* 0.80 Slater + 0.72 dB88 + 0.19 VWN_RPA + 0.81 LYP */
  CALCHEM_XC_B3LYP5 = 4, /* as B3LYP with VWN5 */
  CALCHEM_XC_PBE0 = 5,   /* 0.75 PBE_X + 1.00 PBE_C */
  CALCHEM_XC_CAMB3LYP = 6, /* ITYH-attenuated Slater + B88, 0.19 VWN5 + 0.81 LYP (exact exchange: caller) */
  CALCHEM_XC_WB97X = 7,    /* wB97X semilocal part (omega 0.30) */
  CALCHEM_XC_WB97XD = 8    /* wB97X-D semilocal part (omega 0.20) */
};

/* Precision of the two dense contractions (rho = Phi D Phi^T and V = Phi^T (w v) Phi). */
enum {
  CALCHEM_XC_FP64 = 0,  /* plain all-FP64 drop-in form (matches the reference to 1e-9 Eh / 1e-10) */
  CALCHEM_XC_MIXED = 1  /* tcgen05 tensor-core contractions, split operands, FP32 accumulation */
};

/* Grid levels (crates/calchem-dft/src/grid.rs:13-31). */
enum { CALCHEM_GRID_COARSE = 0, CALCHEM_GRID_MEDIUM = 1, CALCHEM_GRID_FINE = 2, CALCHEM_GRID_ULTRAFINE = 3 };

/* ======================================================================================
 * (1) Drop-in replacements of the reference's exports, same signatures and semantics.
 * ====================================================================================== */

/* Replaces calchem_cuda_is_available (crates/calchem-cuda/src/lib.rs:469-483 binding).
 * Returns 1 when a CUDA device of compute capability 10.3 is usable, else 0. */
int calchem_cuda_is_available(void);

/* Replaces calchem_cuda_vxc_upload_grid (cuda_kernels.cu:7354-7450; binding lib.rs:297-312).
 * Uploads the screened basis, the grid points (grouped by batch_id, batches in increasing
 * order) and the per-batch candidate-shell CSR lists.  Re-uploading an existing id with the same
 * (n_pts, n_ao) returns 0 and keeps the old data; different sizes return -2. */
int calchem_cuda_vxc_upload_grid(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                                 const AoCompGpu* h_comps, int n_comps, const GridPtGpu* h_pts, int n_pts,
                                 const int* h_cand_offsets, int n_cand_offsets, const int* h_cand_shells,
                                 int n_cand_shells, int n_ao, uint64_t grid_id, size_t memory_limit_bytes);

/* Replaces calchem_cuda_vxc_eval_rho (cuda_kernels.cu:7452-7494; binding lib.rs:313-319).
 * h_rho_grad_out[4*g + {0,1,2,3}] = rho, d/dx rho, d/dy rho, d/dz rho at point g for density P. */
int calchem_cuda_vxc_eval_rho(uint64_t grid_id, const double* h_p_mat, double* h_rho_grad_out, int n_pts, int n_ao);

/* Replaces calchem_cuda_vxc_accum (cuda_kernels.cu:7496-7545; binding lib.rs:320-326).
 * h_wv_in[4*g..] = (w v_rho / 2, w u_x, w u_y, w u_z).  h_vxc_out receives the LOWER triangle
 * of V (row >= col); the strict upper triangle is zero. */
int calchem_cuda_vxc_accum(uint64_t grid_id, const double* h_wv_in, double* h_vxc_out, int n_pts, int n_ao);

/* Replaces calchem_cuda_vxc_grad_force (cuda_kernels.cu:8277-8365, kernel 4351-4580; binding
 * lib.rs:394-405, caller GpuVxcGrid::eval_grad_force lib.rs:1308-1352).  The AO part of the XC
 * nuclear gradient for the caller's per-point coefficients h_wxc_in[8 g ..] = (w v_rho_a, w u_a,
 * w v_rho_b, w u_b) (u_a = 2 v_gamma_aa grad rho_a + v_gamma_ab grad rho_b) and spin densities
 * h_pa / h_pb (h_pb ignored when is_rks != 0: beta = alpha): h_grad_out[3 A + q] (n_atoms x 3,
 * overwritten) = -2 sum over points and spins of the AO force terms of the atoms' AOs, with every
 * point's total subtracted at its host atom (GridPtGpu.host_atom of the upload).  The Becke weight
 * term is the caller's, as in the reference.  memory_limit_bytes = 0: no limit.  Returns -1 (bad
 * arguments, host or shell atom outside [0, n_atoms), n_atoms > 1024), -2 (unknown grid or size
 * mismatch), -3 (memory limit), -4 (allocation), -5 (CUDA). */
int calchem_cuda_vxc_grad_force(uint64_t grid_id, const double* h_pa, const double* h_pb, int is_rks,
                                const double* h_wxc_in, double* h_grad_out, int n_pts, int n_ao, int n_atoms,
                                size_t memory_limit_bytes);

/* Replaces calchem_cuda_vxc_release (cuda_kernels.cu:7547-7562; binding lib.rs:327). */
int calchem_cuda_vxc_release(uint64_t grid_id);

/* ======================================================================================
 * (2) Host-side preparation (what RksVxcEngine::new_with_gpu does before uploading).
 * ====================================================================================== */

/* Contraction normalisation and screening data for Cartesian shells
 * (crates/calchem-basis/src/normalization.rs:20-97, lib.rs:462-573; ao_grid.rs:28-71).
 * Inputs per shell: angular momentum l (0..3), atom index, centre (Bohr), primitive count, and the
 * raw exponents / contraction coefficients concatenated over shells.  AO offsets follow shell
 * order.  Outputs: one AoShellGpu per shell, one AoPrimGpu per primitive, one AoCompGpu per
 * Cartesian component (sum over shells of (l+1)(l+2)/2 entries). */
int calchem_xc_prepare_shells(int n_shells, const int* l, const int* atom_index, const double* centers,
                              const int* n_prims, const double* exponents, const double* raw_coefs,
                              AoShellGpu* shells_out, AoPrimGpu* prims_out, AoCompGpu* comps_out, int* n_ao_out);

/* Overlap matrix S (n_ao x n_ao) of prepared shells (crates/calchem-int/src/one_electron.rs:7-31, 115-128). */
int calchem_xc_overlap(const AoShellGpu* shells, int n_shells, const AoPrimGpu* prims, const AoCompGpu* comps,
                       int n_ao, double* s_out);

/* Builds a Becke-partitioned Euler-Maclaurin x Lebedev molecular grid on the GPU
 * (crates/calchem-dft/src/grid.rs:732-828): atom-major, radial-shell-major, Lebedev order; points
 * with w <= 1e-18 dropped.  Becke weights are evaluated in FP64 on the device.  The grid stays on
 * the device under grid_handle until calchem_xc_grid_release. */
int calchem_xc_grid_build(int n_atoms, const int* z, const double* xyz_bohr, int level, int radial_min,
                          uint64_t grid_handle, int* n_pts_out);
/* Per-atom variant (no counterpart in the reference; the learned grid pruner's grids): atom a gets
 * n_rad[a] radial shells (<= 0: the Fine count); a shell at x = r / max(R_BS, 0.3 Bohr) takes
 * region_leb[5 a + k] Lebedev points in the Fine level's pruning region k (x < 0.18, 0.5, 0.95, 5,
 * beyond; each one of 26, 50, 110, 194, 302, 590, or <= 0 for the Fine choice 50 / 110 / 194 / 302 /
 * 194), and shells with x > x_max[a] are left out (x_max[a] <= 0: none).  All zeros reproduce
 * calchem_xc_grid_build(level = Fine). */
int calchem_xc_grid_build_atoms(int n_atoms, const int* z, const double* xyz_bohr, const int* n_rad,
                                const int* region_leb, const double* x_max, uint64_t grid_handle, int* n_pts_out);
/* Copies a built grid to the host: xyzw[4*g] = (x, y, z, weight); raw_w and host_atom may be NULL. */
int calchem_xc_grid_fetch(uint64_t grid_handle, double* xyzw, double* raw_w, int* host_atom);
int calchem_xc_grid_release(uint64_t grid_handle);

/* One-call engine construction: chunks the points into batches of 128 (points with |w| < 1e-24
 * skipped), computes each batch's bounding sphere and candidate shells (vxc.rs:443-493), and
 * uploads everything -- including the weights, which the fused evaluators need -- under grid_id.
 * The evaluation workspace (densities, Vxc, scratch) is allocated by the first evaluate, so a grid
 * uploaded only to become part of a group (below) holds none.  Returns -2 if grid_id exists. */
int calchem_xc_upload_points(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                             const AoCompGpu* h_comps, int n_comps, const double* h_xyzw, int n_pts, int n_ao,
                             uint64_t grid_id, size_t memory_limit_bytes);

/* As calchem_xc_upload_points with chunks of batch_pts (16..128) consecutive points instead of
 * 128: smaller chunks have smaller bounding spheres, hence fewer candidate AOs per point, at the cost
 * of more batches.  Results are the same up to summation order; the autotuner picks batch_pts. */
int calchem_xc_upload_points_ex(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims, int n_prims,
                                const AoCompGpu* h_comps, int n_comps, const double* h_xyzw, int n_pts, int n_ao,
                                int batch_pts, uint64_t grid_id, size_t memory_limit_bytes);

/* The batch plan of the two upload functions below, computed on the host only (no device): spatial = 0
 * CalChem's chunks (calchem_xc_upload_points_ex), 1 compact batches (calchem_xc_upload_points_spatial).
 * Outputs (each may be NULL): the number of batches, of kept points (|w| >= 1e-24, in a batch with a
 * candidate shell) and of candidate entries; sum over batches of m_b^2 n_b (m_b the batch's AO count)
 * and the largest m_b; h_order[k] = the caller's index of the k-th planned point and h_batch_of[k]
 * its batch (n_kept entries each: n_pts always suffice); h_cand_offsets (n_batches + 1 entries,
 * n_pts + 1 suffice) and h_cand_shells (n_cand entries, at most cand_capacity: -2 if more) the
 * candidate shells per batch.  Returns 0; -1 on bad arguments; -2 when h_cand_shells is given and
 * the plan has more than cand_capacity candidates (checked before any output is written, so a
 * failed call leaves every caller buffer as it was). */
int calchem_xc_plan_points(const AoShellGpu* h_shells, int n_shells, const double* h_xyzw, int n_pts, int batch_pts,
                           int spatial, int* n_batches, int* n_kept, int* n_cand, double* sum_m2n, int* max_m,
                           int* h_order, int* h_batch_of, int* h_cand_offsets, int* h_cand_shells, int cand_capacity);

/* As calchem_xc_upload_points_ex with spatially compact batches instead of consecutive chunks: the
 * points are ordered by recursive bisection along the longest axis of their box (leaves of batch_pts
 * points; ties broken by index, so the plan is the same on every machine) before chunking, and each
 * batch's candidate list (the reference's bounding-sphere rule) is narrowed to the shells whose
 * cut-off sphere holds at least one of its points.  A chunk of the reference's order spans whole
 * Lebedev spheres, so its candidates are nearly every shell; a compact batch has far fewer AOs.
 * Every point sees the same nonzero AO values as under the reference's batching, so the results are
 * the same up to summation order.  A candidate shell is also dropped from a batch when a bound on all
 * its components' |phi| and |grad phi| stays below 1e-17 at every point of the batch: those values are
 * zeroed by the reference's own screen (<= 1e-16, ao_grid.rs:182-230), so the results do not change.
 * (calchem_xc_plan_points, which has no primitives, does not apply this bound.) */
int calchem_xc_upload_points_spatial(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims,
                                     int n_prims, const AoCompGpu* h_comps, int n_comps, const double* h_xyzw,
                                     int n_pts, int n_ao, int batch_pts, uint64_t grid_id,
                                     size_t memory_limit_bytes);

/* As calchem_xc_upload_points_spatial with the value screen's floor chosen by the caller (no
 * counterpart in the reference): shells whose bound stays below ao_floor at every point of a batch are
 * left out of it.  ao_floor = 1e-17 is the exact screen above; larger floors (up to 1e-6) drop AO
 * contributions up to that size, an approximation traded for fewer AOs per batch.  -1 for ao_floor
 * outside [1e-17, 1e-6]. */
int calchem_xc_upload_points_screened(const AoShellGpu* h_shells, int n_shells, const AoPrimGpu* h_prims,
                                      int n_prims, const AoCompGpu* h_comps, int n_comps, const double* h_xyzw,
                                      int n_pts, int n_ao, int batch_pts, uint64_t grid_id,
                                      size_t memory_limit_bytes, double ao_floor);

/* Attaches quadrature weights to a grid uploaded with calchem_cuda_vxc_upload_grid
 * (weights in the uploaded point order). */
int calchem_xc_set_weights(uint64_t grid_id, const double* h_weights, int n_pts);

/* The AO cache of the tensor-core form.  AO values and gradients depend only on the grid and the
 * basis, so, as CalChem's RksVxcEngine caches them per batch for every SCF iteration
 * (crates/calchem-dft/src/vxc.rs:386-394, 600-716), the first tensor-core evaluation of a grid
 * allocates a cache of each batch's AO planes (FP32 + BF16 parts), packed GEMM1 operand and row
 * exponents (32 B per AO and point), the first launch to reach a batch fills its block, and later
 * evaluations read it instead of evaluating the AOs.  Its size is limited by
 * CALCHEM_MAX_AO_GRID_BYTES (the reference's variable for its AO cache; default here 32 GiB, since
 * the cache lives in HBM where the reference's 2560 MiB default sizes host memory), by the grid's
 * memory budget (memory_limit_bytes of its upload or group) and by the free device memory less
 * 1 GiB: the batches whose blocks fit within that limit, taken in batch order, are cached and the
 * others evaluate their AOs every time (the reference caches all or nothing).  enable = 0 waits for the device,
 * frees the cache, disables it and drops a captured graph; enable = 1 allows it again (a no-op when
 * allowed, the default); -1 only reports its size in *bytes_out (0 when none).  Results are the
 * same with and without the cache. */
int calchem_xc_set_ao_cache(uint64_t grid_id, int enable, size_t* bytes_out);

/* Number of batches and the sum over batches of m_b^2 * n_b (m_b AOs, n_b points): the
 * algorithmic contraction work is 4x (RKS) that sum in flops. */
int calchem_xc_plan_stats(uint64_t grid_id, int* n_batches, double* sum_m2n, double* sum_m2, int* max_m);

/* ======================================================================================
 * (3) Fused evaluators: D -> (Exc, Nelec, V) entirely on the device.
 * ====================================================================================== */

/* Closed shell.  d_total = P_total = 2 P_alpha (as RksVxcEngine::evaluate, vxc.rs:720-726).
 * exc_out = sum_g w_g f_xc; nelec_out = sum_g w_g rho_g (points with rho >= 1e-18);
 * v_out = full symmetric alpha-spin Vxc.
 * On a group (calchem_xc_group_create) the matrices are the members' blocks packed one after the
 * other (calchem_xc_group_layout gives the offsets) and exc_out / nelec_out hold one value per
 * member. */
int calchem_xc_evaluate_rks(uint64_t grid_id, int xc_code, int precision, const double* h_d_total,
                            double* exc_out, double* nelec_out, double* h_v_out);

/* Closed shell with per-point shares instead of V (no counterpart in the reference; used to measure
 * per-atom quadrature errors): point_out[2 g] = w_g f_g (summing to Exc) and point_out[2 g + 1] =
 * w_g (v_rho rho_g + v_gamma |grad rho_g|^2) (summing to tr(D Vxc)), for every point the caller
 * uploaded, in its order (2 x n_pts values); points below the density floor, and points no AO
 * reaches, get 0.  Single grids only (-2 for a group). */
int calchem_xc_evaluate_rks_points(uint64_t grid_id, int xc_code, int precision, const double* h_d_total,
                                   double* exc_out, double* nelec_out, double* h_point_out);

/* The tensor-core form's GEMM1 tile (no counterpart in the reference; chosen by the autotuner):
 * tile_n = 64 AOs per TMEM accumulator with two CTAs per SM (the default), or 128 with one CTA per SM
 * and all 512 TMEM columns (half the GEMM1 rounds and operand reloads per batch, no second CTA to
 * overlap with).  Results are identical up to the order of the Vxc atomics.  calchem_xc_set_tile
 * returns -1 for another value, -2 for an unknown id; calchem_xc_get_tile returns the tile or -2.  A
 * captured graph keeps the tile it was captured with. */
int calchem_xc_set_tile(uint64_t grid_id, int tile_n);
int calchem_xc_get_tile(uint64_t grid_id);

/* Per-atom quadrature shares for the learned grid's periodic full-grid judge (no counterpart in the
 * reference).  calchem_xc_set_point_atoms gives the host atom (0 .. n_atoms - 1) of every point the
 * caller uploaded, in its order (n_points = the uploaded count); the library groups the planned points
 * by atom once.  calchem_xc_evaluate_rks_atoms then evaluates the closed-shell per-point shares of
 * calchem_xc_evaluate_rks_points and sums them per atom on the device in a fixed order: atom_out[2 a] =
 * sum of w f over atom a's points (its share of Exc), atom_out[2 a + 1] = its share of tr(D Vxc);
 * exc_out / nelec_out as calchem_xc_evaluate_rks.  With h_v_out = NULL it skips the Vxc contraction
 * (the shares alone); with h_v_out it is the full build as well (Vxc as calchem_xc_evaluate_rks), so
 * an SCF iteration that runs the judge gets the pruned grid's shares from its own build.  The
 * _device variant takes device buffers (d_result: Exc, Nelec; d_v: n x n or NULL; d_atom_out: 2
 * n_atoms) and enqueues on `stream`.  Returns -2 for an unknown id, a group, a point count that
 * differs from the upload, or (evaluate) no atoms set. */
int calchem_xc_set_point_atoms(uint64_t grid_id, const int* h_host_atom, int n_points, int n_atoms);
int calchem_xc_evaluate_rks_atoms(uint64_t grid_id, int xc_code, int precision, const double* h_d_total,
                                  double* exc_out, double* nelec_out, double* h_atom_out, double* h_v_out);
int calchem_xc_evaluate_rks_atoms_device(uint64_t grid_id, int xc_code, int precision, const double* d_total,
                                         double* d_result, double* d_v, double* d_atom_out, void* stream);

/* The closed-shell point functional on the device (eval_xc_spin, crates/calchem-dft/src/xc.rs:159-175,
 * at rho_a = rho_b = h_rho[i], gamma_aa = gamma_ab = gamma_bb = h_gamma[i]): h_out[3 i ..] =
 * (f, v_rho_a, v_gamma_aa + v_gamma_ab / 2) for i < n.  precision CALCHEM_XC_FP64: the FP64 form of
 * the FP64 quadrature; CALCHEM_XC_MIXED: the form of the tensor-core quadrature (double-float
 * arithmetic on the FP32 pipe for xc codes 0-5 at total density >= 1e-12, FP64 otherwise). */
int calchem_xc_eval_closed_shell(int xc_code, int precision, int n, const double* h_rho, const double* h_gamma,
                                 double* h_out);

/* Open shell (UksVxcEngine::evaluate, vxc.rs:1662-1669).  nelec_out[0..1] = (N_alpha, N_beta);
 * on a group, exc_out[i] and nelec_out[2 i .. 2 i + 1] for member i. */
int calchem_xc_evaluate_uks(uint64_t grid_id, int xc_code, int precision, const double* h_pa, const double* h_pb,
                            double* exc_out, double* nelec_out, double* h_va_out, double* h_vb_out);

/* Device-pointer variants (inputs and outputs already in device memory; enqueued on `stream`,
 * a cudaStream_t, 0 for the legacy stream).  d_result receives (Exc, N_alpha + N_beta) for RKS and
 * (Exc, N_alpha, N_beta) for UKS, once per member of a group.  They return after enqueueing; the
 * caller synchronises and may then read the device status with calchem_xc_last_status. */
int calchem_xc_evaluate_rks_device(uint64_t grid_id, int xc_code, int precision, const double* d_total,
                                   double* d_result, double* d_v, void* stream);
int calchem_xc_evaluate_uks_device(uint64_t grid_id, int xc_code, int precision, const double* d_pa,
                                   const double* d_pb, double* d_result, double* d_va, double* d_vb, void* stream);

/* TD-DFT exchange-correlation kernel (FxcKernel, crates/calchem-dft/src/fxc.rs:176-647), batched over
 * trial matrices.  calchem_xc_fxc_prepare (FxcKernel::new) evaluates the ground-state density
 * d_total = P_total on the grid and stores 11 kernel coefficients per point (finite differences of
 * the FP64 functional, as the reference); calchem_xc_fxc_contract (contract_batch) returns, for each
 * of n_trials symmetric n x n matrices M_b packed one after the other in h_m, the full symmetric
 * dV_b = f_xc[M_b] (singlet, or triplet when triplet != 0) in h_v_out.  The grid's AOs are evaluated
 * once per batch for all trial matrices.  -1 when the kernel was not prepared; single grids only. */
int calchem_xc_fxc_prepare(uint64_t grid_id, int xc_code, const double* h_d_total);
int calchem_xc_fxc_contract(uint64_t grid_id, int triplet, const double* h_m, int n_trials, double* h_v_out);
/* As calchem_xc_fxc_contract with a precision: CALCHEM_XC_FP64 (the above) or CALCHEM_XC_MIXED, the
 * tensor-core form: per trial matrix the closed-shell tensor-core pipeline with M_b in place of the
 * density and the prepared kernel coefficients in place of the functional (the AO cache, filled by
 * the first launch, serves every trial); dV agrees with the FP64 form to ~1e-7 of its largest entry. */
int calchem_xc_fxc_contract_ex(uint64_t grid_id, int triplet, int precision, const double* h_m, int n_trials,
                               double* h_v_out);
/* Device-pointer variant of the contraction (enqueued on `stream`, not synchronised). */
int calchem_xc_fxc_contract_device(uint64_t grid_id, int triplet, const double* d_m, int n_trials, double* d_v_out,
                                   void* stream);
/* The device-pointer contraction with a precision (see calchem_xc_fxc_contract_ex). */
int calchem_xc_fxc_contract_device_ex(uint64_t grid_id, int triplet, int precision, const double* d_m, int n_trials,
                                      double* d_v_out, void* stream);

/* XC nuclear gradient dExc/dR at fixed densities (xc_nuclear_gradient, vxc.rs:1903-1912 and the
 * Becke weight derivative grid.rs:423-584), entirely on the device: densities, functional, AO force
 * terms with the host-atom term, and the weight derivative.  precision CALCHEM_XC_FP64: all FP64;
 * CALCHEM_XC_MIXED: the contractions P Phi and P Psi on the tensor cores (exact fixed-point split),
 * AO values, derivatives and the force terms in double-float, functional and weight derivative in
 * FP64; batches of more than 2048 AOs return -2 for it.  grid_id is a single grid
 * uploaded with its weights (calchem_xc_upload_points*); h_raw_w (weights before the Becke
 * partition) and h_host_atom hold the n_grid_pts points the caller uploaded, in its order (as
 * calchem_xc_grid_fetch returns them); the atoms (z, xyz_bohr) are the molecule the grid was built
 * for.  h_pa / h_pb are the spin densities; h_pb = NULL means a closed shell (beta = alpha, so an
 * RKS caller passes P_total / 2).  h_grad_out[3 A + q] = dExc/dR_Aq in Eh/Bohr.  Points that were
 * not uploaded (|w| < 1e-24) are left out.  One atom: zeros.  Returns -1 (bad arguments, host or
 * shell atom outside [0, n_atoms), n_atoms > 1024), -2 (unknown grid, a group, no weights, or
 * n_grid_pts not the uploaded count), -4 / -5 on allocation / CUDA failure, -7 when a device-side
 * wait of the tensor-core form expired. */
int calchem_xc_nuclear_gradient(uint64_t grid_id, int xc_code, int precision, int n_atoms, const int* z,
                                const double* xyz_bohr, const double* h_raw_w, const int* h_host_atom, int n_grid_pts,
                                const double* h_pa, const double* h_pb, double* h_grad_out);

/* ======================================================================================
 * (3b) Many molecules in one launch, and CUDA-graph replay.  No counterpart in the reference.
 * ====================================================================================== */

/* Concatenates already-uploaded grids (calchem_xc_upload_points, weights attached) into one group
 * under group_id: one work queue over every member's batches, processed by one persistent kernel
 * launch per evaluate.  The members' device data are copied, so they may be released afterwards.
 * Returns -2 for an unknown or grouped member id or an existing group_id, -1 for repeated ids,
 * -3 over memory_limit_bytes, -4 / -5 on allocation / copy failure. */
int calchem_xc_group_create(const uint64_t* member_ids, int n_members, uint64_t group_id, size_t memory_limit_bytes);

/* Layout of the packed matrices of a group (also valid for a single grid: one member at offset 0):
 * member i is the mol_n[i] x mol_n[i] block starting at element mol_off[i].  mol_n_out and
 * mol_off_out may be NULL; otherwise they hold n_mols entries. */
int calchem_xc_group_layout(uint64_t grid_id, int* n_mols_out, int* mol_n_out, long long* mol_off_out);

/* Captures one device evaluation of grid_id (a single grid or a group) into a CUDA graph held by
 * the library: mode 0 = RKS (d_pa = P_total, d_va), 1 = UKS (d_pa, d_pb, d_va, d_vb), arguments as
 * the _device evaluators.  The graph keeps these device pointers; calchem_xc_graph_launch replays
 * it on any stream (one kernel-launch latency for the whole sequence: density split, quadrature,
 * reductions, symmetrisation).  Capturing again replaces the graph. */
int calchem_xc_graph_capture(uint64_t grid_id, int mode, int xc_code, int precision, const double* d_pa,
                             const double* d_pb, double* d_result, double* d_va, double* d_vb);
int calchem_xc_graph_launch(uint64_t grid_id, void* stream);

/* Device status of the last evaluation or graph replay of grid_id (synchronous read): 0, or -7 when
 * a device-side wait expired. */
int calchem_xc_last_status(uint64_t grid_id);

/* Number of kernel launches the last evaluate on grid_id enqueued (for launch accounting). */
int calchem_xc_last_launch_count(uint64_t grid_id);

/* Kernel timing: when enabled, every evaluate on grid_id records CUDA events on its launch stream
 * around the main quadrature kernel; calchem_xc_last_kernel_ms synchronises on the end event and
 * returns that kernel's duration in milliseconds. */
int calchem_xc_set_profiling(uint64_t grid_id, int enable);
int calchem_xc_last_kernel_ms(uint64_t grid_id, float* ms_out);

/* ======================================================================================
 * (5) The learned grid pruner's network (no counterpart in the reference).  A fixed MLP
 * (16 inputs, two tanh layers of 64, 16 linear outputs; parameters one float buffer
 * W1 [16][64], b1, W2 [64][64], b2, W3 [64][16], b3) maps an atom's environment features to the
 * predicted log10 quadrature error of each candidate grid level.  All pointers are device
 * pointers; work is enqueued on `stream` (a cudaStream_t) and not synchronised.
 * ====================================================================================== */

int calchem_mlp_shape(int* n_in, int* n_hidden, int* n_out, int* n_params, int* work_per_sample);
/* y [n][16] = network(x [n][16]). */
int calchem_mlp_forward(const float* d_params, const float* d_x, int n, float* d_y, void* stream);
/* Masked mean squared error L = inv_count * sum mask (y - t)^2 over t, mask [n][16]:
 * d_grad [n_params] = dL/dparams (summed over samples in a fixed order), *d_loss = L;
 * d_work [n][work_per_sample] and d_loss_part [n] are scratch. */
int calchem_mlp_loss_grad(const float* d_params, const float* d_x, const float* d_t, const float* d_mask, int n,
                          float inv_count, float* d_work, float* d_loss_part, float* d_grad, float* d_loss,
                          void* stream);
/* One Adam update (bias-corrected, step >= 1) of d_params with moment buffers d_m, d_v. */
int calchem_mlp_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, int n_params, int step, float lr,
                     float beta1, float beta2, float eps, void* stream);

/* ======================================================================================
 * (6) Integrals for the SCF harness around the quadrature (host code, McMurchie-Davidson), over
 * the same prepared shells: crates/calchem-int/src/one_electron.rs, eri.rs, boys.rs provide these
 * to the reference's SCF.  Matrices are n_ao x n_ao row-major; the ERI tensor is dense n_ao^4
 * (chemists' order (pq|rs) at ((p n + q) n + r) n + s), for n_ao <= 400 (-3 beyond).
 * ====================================================================================== */

/* Boys function F_0 .. F_n_max at t (n_max <= 17). */
int calchem_scf_boys(int n_max, double t, double* f_out);
/* Overlap, kinetic and nuclear-attraction matrices (any output may be NULL); charges / xyz_bohr
 * give the nuclei. */
int calchem_scf_one_electron(const AoShellGpu* shells, int n_shells, const AoPrimGpu* prims, const AoCompGpu* comps,
                             int n_ao, int n_atoms, const double* charges, const double* xyz_bohr, double* s_out,
                             double* t_out, double* v_out);
int calchem_scf_eri(const AoShellGpu* shells, int n_shells, const AoPrimGpu* prims, const AoCompGpu* comps, int n_ao,
                    double* eri_out);

/* ======================================================================================
 * (4) Evaluation without device allocation.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc -- a framework that owns all device memory through its own
 * pool, or a serving loop that must not take cudaMalloc's implicit device synchronisation in the
 * middle of an SCF iteration.
 * ====================================================================================== */

/* Size of the library's fixed device working buffer (a static device array held by every GPU that
 * loads the library until the process exits). */
#define CALCHEM_XC_STATIC_SCRATCH_BYTES ((size_t)96 << 20)

/* Closed-shell FP64 evaluation (same results as calchem_xc_evaluate_rks with precision FP64) where
 * every input and output is a device buffer owned by the caller, in the reference's upload layout:
 * shells / prims / comps, points grouped by non-decreasing batch_id (<= 128 per batch) with their
 * quadrature weights, the per-batch candidate-shell CSR lists, max_batch_ao = the largest number of
 * AOs of any batch, d_total (n_ao x n_ao), d_result (Exc, Nelec) and d_v (n_ao x n_ao, full symmetric).
 * All working memory comes from the static buffer above; nothing is allocated.
 *   - The first call on a device looks up the buffer's device address (cudaGetSymbolAddress); make
 *     that first call before any stream capture on that device.  The address is kept for the life of
 *     the process, so do not call this entry point after a cudaDeviceReset.
 *   - Work on `stream` (a cudaStream_t, 0 for the legacy stream); returns after it completes.
 *   - Returns -3 when the points, tables and one CTA's working set do not fit in the buffer
 *     (large n_pts or max_batch_ao), -2 when the layout is inconsistent (a batch id outside
 *     [0, n_batches) or smaller than the previous point's, a batch of more than 128 points, a shell
 *     index or range out of bounds, a batch with more than max_batch_ao AOs), -1
 *     for null pointers or non-positive sizes, -5 for a launch or copy failure.
 *   - Every call shares the buffer and finds the previous call's contents in it (the work-queue head
 *     and status word are cleared on entry, the rest is overwritten before use).  Calls through this
 *     entry point are serialised and synchronous, so they never overlap; GPU work that did overlap
 *     on the buffer would race. */
int calchem_xc_evaluate_rks_static(const AoShellGpu* d_shells, int n_shells, const AoPrimGpu* d_prims, int n_prims,
                                   const AoCompGpu* d_comps, int n_comps, const GridPtGpu* d_pts,
                                   const double* d_weights, int n_pts, const int* d_cand_offsets,
                                   const int* d_cand_shells, int n_batches, int n_cand_shells, int n_ao,
                                   int max_batch_ao, int xc_code, const double* d_total, double* d_result,
                                   double* d_v, void* stream);

/* Library version string. */
const char* calchem_xc_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CALCHEM_XC_H */
