"""Kohn-Sham XC matrix engines (mirrors crates/calchem-dft/src/vxc.rs and the
``GpuVxcGrid`` wrapper of crates/calchem-cuda/src/lib.rs:1178-1306).

``RksVxcEngine`` / ``UksVxcEngine`` keep the reference call surface
(``new_with_gpu``, ``evaluate``, ``telemetry``) and run the whole Vxc build on the
GPU through the fused C ABI (``calchem_xc_evaluate_rks`` / ``_uks``).  There is no
CPU path: a device or library failure raises ``CalchemXcError`` instead of
falling back, so ``telemetry()`` never reports a fallback.

``GpuVxcGrid`` exposes the reference's own four-call FFI
(upload_grid / eval_rho / accum / release) for callers that evaluate the
functional themselves, as CalChem's Rust engine does (vxc.rs:728-799).
"""

import itertools
import os

import ctypes

import numpy as np

from . import _native
from .xc import XcFunctional

FP64 = 0
MIXED = 1
_PRECISION = {"fp64": FP64, "mixed": MIXED, FP64: FP64, MIXED: MIXED}

_ids = itertools.count(1 << 20)

MAX_GPU_MEMORY_BYTES = 64 << 30

# The tensor-core engines' value screen (calchem_xc_upload_points_screened): a shell is left out of a
# compact batch when a bound on its components' values and gradients stays below this at every point
# of the batch.  Those contributions are ~4 orders below the tensor-core form's own agreement with
# FP64 on Vxc (~1e-6); on the 61-water cluster the screen halves sum m^2 n and moves Exc by < 1e-10 Eh.
# The FP64 form keeps the exact screen (1e-17: only values the reference itself zeroes are left out).
MIXED_AO_FLOOR = 1e-12


def default_ao_floor(precision):
    """The value screen an engine of this precision uploads with: MIXED_AO_FLOOR for the tensor-core
    form, the exact screen (None) for FP64."""
    return MIXED_AO_FLOOR if _PRECISION[precision] == MIXED else None


def eval_closed_shell_gpu(func, rho_a, gamma, precision="fp64"):
    """The closed-shell point functional on the device: eval_xc_spin (xc.rs:159-175) at
    rho_a = rho_b = rho_a[i] and gamma_aa = gamma_ab = gamma_bb = gamma[i].  Returns an (n, 3) array
    of (f, v_rho_a, v_gamma_aa + v_gamma_ab / 2).  precision "fp64": the FP64 quadrature's form;
    "mixed": the tensor-core quadrature's form (double-float arithmetic for SVWN5..PBE0 at total
    density >= 1e-12)."""
    if isinstance(func, str):
        func = XcFunctional.from_name(func)
    r = np.ascontiguousarray(rho_a, dtype=np.float64).ravel()
    g = np.ascontiguousarray(gamma, dtype=np.float64).ravel()
    if r.shape != g.shape or r.size == 0:
        raise ValueError("rho_a and gamma must be non-empty and of equal size")
    out = np.empty((r.size, 3), dtype=np.float64)
    lib = _native.load()
    _native.check("calchem_xc_eval_closed_shell", lib.calchem_xc_eval_closed_shell(
        int(func), _PRECISION[precision], r.size, _native.ptr(r), _native.ptr(g), _native.ptr(out)))
    return out


def resolve_gpu_memory_limit() -> int:
    """CALCHEM_MAX_GPU_MEM_MB when set (as calchem-cuda's resolve_gpu_memory_limit, lib.rs:531-538);
    otherwise 64 GiB, since the reference's 5 GiB ceiling targets 8 GB cards."""
    v = os.environ.get("CALCHEM_MAX_GPU_MEM_MB")
    if v is not None:
        try:
            return min(int(v) << 20, MAX_GPU_MEMORY_BYTES)
        except ValueError:
            pass
    return MAX_GPU_MEMORY_BYTES


def is_cuda_available() -> bool:
    """calchem_cuda::is_cuda_available (lib.rs:469-483), including the CALCHEM_DISABLE_GPU switch."""
    if os.environ.get("CALCHEM_DISABLE_GPU") == "1":
        return False
    return _native.load().calchem_cuda_is_available() == 1


def _xc_code(func) -> int:
    if isinstance(func, str):
        return int(XcFunctional.from_name(func))
    return int(XcFunctional(func))


def _as_matrix(m, n):
    a = np.ascontiguousarray(m, dtype=np.float64)
    if a.shape != (n, n):
        raise ValueError(f"expected a {n}x{n} matrix, got {a.shape}")
    return a


class GpuVxcGrid:
    """The reference's device-resident grid (lib.rs:1178-1306) over the drop-in C ABI."""

    def __init__(self, grid_id, n_pts, n_ao):
        self.grid_id, self.n_pts, self.n_ao = grid_id, n_pts, n_ao

    @classmethod
    def upload(cls, shells, prims, comps, pts, cand_offsets, cand_shells, n_ao, memory_limit=None):
        lib = _native.load()
        gid = next(_ids)
        shells = np.ascontiguousarray(shells, dtype=_native.AO_SHELL)
        prims = np.ascontiguousarray(prims, dtype=_native.AO_PRIM)
        comps = np.ascontiguousarray(comps, dtype=_native.AO_COMP)
        pts = np.ascontiguousarray(pts, dtype=_native.GRID_PT)
        off = np.ascontiguousarray(cand_offsets, dtype=np.int32)
        cs = np.ascontiguousarray(cand_shells, dtype=np.int32)
        lim = resolve_gpu_memory_limit() if memory_limit is None else int(memory_limit)
        _native.check("calchem_cuda_vxc_upload_grid", lib.calchem_cuda_vxc_upload_grid(
            _native.ptr(shells), len(shells), _native.ptr(prims), len(prims), _native.ptr(comps), len(comps),
            _native.ptr(pts), len(pts), _native.ptr(off), len(off), _native.ptr(cs), len(cs), int(n_ao), gid, lim))
        return cls(gid, len(pts), int(n_ao))

    def eval_rho_grad(self, p_mat) -> np.ndarray:
        lib = _native.load()
        P = _as_matrix(p_mat, self.n_ao)
        out = np.zeros((self.n_pts, 4), dtype=np.float64)
        _native.check("calchem_cuda_vxc_eval_rho", lib.calchem_cuda_vxc_eval_rho(
            self.grid_id, _native.ptr(P), _native.ptr(out), self.n_pts, self.n_ao))
        return out

    def accumulate_vxc(self, wv) -> np.ndarray:
        lib = _native.load()
        w = np.ascontiguousarray(wv, dtype=np.float64).reshape(self.n_pts, 4)
        out = np.zeros((self.n_ao, self.n_ao), dtype=np.float64)
        _native.check("calchem_cuda_vxc_accum", lib.calchem_cuda_vxc_accum(
            self.grid_id, _native.ptr(w), _native.ptr(out), self.n_pts, self.n_ao))
        return out

    def eval_grad_force(self, pa, pb, is_rks, wxc, n_atoms, memory_limit=None) -> np.ndarray:
        """AO part of the XC nuclear gradient for per-point coefficients wxc [n_pts][8] =
        (w v_rho_a, w u_a, w v_rho_b, w u_b) (GpuVxcGrid::eval_grad_force, lib.rs:1308-1352);
        returns [n_atoms][3]."""
        lib = _native.load()
        Pa = _as_matrix(pa, self.n_ao)
        Pb = Pa if is_rks else _as_matrix(pb, self.n_ao)
        w = np.ascontiguousarray(wxc, dtype=np.float64).reshape(self.n_pts, 8)
        out = np.zeros((int(n_atoms), 3), dtype=np.float64)
        lim = resolve_gpu_memory_limit() if memory_limit is None else int(memory_limit)
        _native.check("calchem_cuda_vxc_grad_force", lib.calchem_cuda_vxc_grad_force(
            self.grid_id, _native.ptr(Pa), _native.ptr(Pb), int(bool(is_rks)), _native.ptr(w), _native.ptr(out),
            self.n_pts, self.n_ao, int(n_atoms), lim))
        return out

    def release(self):
        if self.grid_id:
            _native.load().calchem_cuda_vxc_release(self.grid_id)
            self.grid_id = 0

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


BATCHING = ("spatial", "reference")


def _upload_points(basis, grid, batch_pts: int = 128, batching: str = "spatial", ao_floor=None) -> int:
    """Batches and uploads one molecule's grid; returns its grid id.  batching "spatial": compact
    batches (calchem_xc_upload_points_spatial); "reference": chunks of consecutive points as CalChem
    forms them (calchem_xc_upload_points_ex).  The results agree up to summation order.  ao_floor
    (compact batches only): drop a shell from a batch when a bound on its components' values and
    gradients stays below this at every point of the batch (calchem_xc_upload_points_screened);
    None is the exact screen (1e-17, below the reference's own 1e-16 cut)."""
    if batching not in BATCHING:
        raise ValueError(f"batching must be one of {BATCHING}")
    lib = _native.load()
    sh, pr, co = basis.gpu_arrays()
    xyzw = np.ascontiguousarray(grid.xyzw, dtype=np.float64)
    if len(xyzw) == 0:
        raise ValueError("empty grid")
    gid = next(_ids)
    args = (_native.ptr(sh), len(sh), _native.ptr(pr), len(pr), _native.ptr(co), len(co), _native.ptr(xyzw),
            len(xyzw), basis.n_ao, int(batch_pts), gid, resolve_gpu_memory_limit())
    if ao_floor is not None:
        if batching != "spatial":
            raise ValueError("ao_floor applies to compact (spatial) batches")
        _native.check("calchem_xc_upload_points_screened", lib.calchem_xc_upload_points_screened(*args,
                                                                                                float(ao_floor)))
        return gid
    fn = "calchem_xc_upload_points_spatial" if batching == "spatial" else "calchem_xc_upload_points_ex"
    _native.check(fn, getattr(lib, fn)(*args))
    return gid


def plan_points(basis, xyzw, batch_pts: int = 128, batching: str = "spatial") -> dict:
    """The batch plan an engine would upload for these points, computed on the host alone
    (calchem_xc_plan_points): "order" (the caller's index of each planned point), "batch_of" (its
    batch), "cand_offsets"/"cand_shells" (candidate shells per batch), "sum_m2n" (sum over batches
    of m_b^2 n_b, the contraction work), "max_m" (the largest batch's AO count)."""
    if batching not in BATCHING:
        raise ValueError(f"batching must be one of {BATCHING}")
    lib = _native.load()
    sh, _, _ = basis.gpu_arrays()
    xyzw = np.ascontiguousarray(getattr(xyzw, "xyzw", xyzw), dtype=np.float64).reshape(-1, 4)
    n = len(xyzw)
    if n == 0:
        raise ValueError("empty grid")
    nb, nk, nc, mm = (np.zeros(1, np.int32) for _ in range(4))
    s2 = np.zeros(1)
    spatial = int(batching == "spatial")
    args = (_native.ptr(sh), len(sh), _native.ptr(xyzw), n, int(batch_pts), spatial)
    _native.check("calchem_xc_plan_points", lib.calchem_xc_plan_points(
        *args, _native.ptr(nb), _native.ptr(nk), _native.ptr(nc), None, None, None, None, None, None, 0))
    order, batch_of = np.zeros(n, np.int32), np.zeros(n, np.int32)
    offs, cand = np.zeros(int(nb[0]) + 1, np.int32), np.zeros(max(int(nc[0]), 1), np.int32)
    _native.check("calchem_xc_plan_points", lib.calchem_xc_plan_points(
        *args, None, None, None, _native.ptr(s2), _native.ptr(mm), _native.ptr(order), _native.ptr(batch_of),
        _native.ptr(offs), _native.ptr(cand), len(cand)))
    k = int(nk[0])
    return {"order": order[:k], "batch_of": batch_of[:k], "cand_offsets": offs, "cand_shells": cand[:int(nc[0])],
            "sum_m2n": float(s2[0]), "max_m": int(mm[0])}


class _TileMixin:
    """The tensor-core form's GEMM1 tile (calchem_xc_set_tile): 64 or 128, or "auto" to take the
    autotuner's choice for the workload, measured at the first tensor-core evaluation (and cached)."""

    def _init_tile(self, tile, basis, grid, spin):
        self._tile_src = (basis, grid, spin)
        self.tile = None
        if tile != "auto":
            self.set_tile(int(tile))

    def set_tile(self, tile_n: int):
        _native.check("calchem_xc_set_tile", _native.load().calchem_xc_set_tile(self.grid_id, int(tile_n)))
        self.tile = int(tile_n)

    def _tune_tile(self, func, run):
        """Picks the tile on the first tensor-core evaluation: every tile is timed on this workload (or
        the cached choice for its signature is taken)."""
        from . import autotune
        basis, grid, spin = self._tile_src
        key = autotune.signature(basis, grid, func, "mixed", spin)
        lib = _native.load()

        def measure():
            _native.check("calchem_xc_set_profiling", lib.calchem_xc_set_profiling(self.grid_id, 1))
            try:
                return autotune.time_tiles(self, run)
            finally:
                _native.check("calchem_xc_set_profiling", lib.calchem_xc_set_profiling(self.grid_id,
                                                                                      int(self._profiling)))
        self.set_tile(autotune.choose_tile(key, measure))

    def last_kernel_ms(self) -> float:
        """Duration of the quadrature kernel of the last evaluate (profiling enabled)."""
        ms = (ctypes.c_float * 1)()
        _native.check("calchem_xc_last_kernel_ms", _native.load().calchem_xc_last_kernel_ms(self.grid_id, ms))
        return float(ms[0])


class _EngineBase(_TileMixin):
    """batch_pts: points per batch (16..128; the reference's 128 by default), or "auto" to take
    the autotuner's choice for this workload (tuned on first use, then cached).  batching:
    "spatial" (compact batches, the default) or "reference" (CalChem's chunks of consecutive
    points); the results agree up to summation order.  tile: the tensor-core GEMM1 tile, 64, 128 or
    "auto" (the default: tuned at the first tensor-core evaluation; results do not depend on it).
    ao_floor: the compact plan's value screen ("auto": MIXED_AO_FLOOR for a tensor-core engine, the
    exact screen for FP64; None: exact; a number: that floor)."""

    def __init__(self, basis, grid, use_gpu=True, precision="fp64", batch_pts=128, func="b3lyp",
                 batching="spatial", tile="auto", ao_floor="auto"):
        if not use_gpu:
            raise NotImplementedError("calchem_gb300 evaluates Vxc on the GPU only; there is no CPU engine")
        self.n_ao = basis.n_ao
        self.precision = _PRECISION[precision]
        self.gpu_kernel_invocations = 0
        self.gpu_fallback_invocations = 0
        self.grid_id = 0
        self.last_nelec = None
        self._profiling = False
        spin = "uks" if isinstance(self, UksVxcEngine) else "rks"
        if batch_pts == "auto":
            from . import autotune
            plan = autotune.choose_plan(basis, grid, func, precision, spin=spin)
            batch_pts = plan["batch_pts"]
            if tile == "auto" and precision == "mixed":
                tile = plan["tile_n"]
        self.batch_pts = int(batch_pts)
        self.batching = batching
        if ao_floor == "auto":
            ao_floor = default_ao_floor(precision) if batching == "spatial" else None
        self.ao_floor = ao_floor
        self.grid_id = _upload_points(basis, grid, self.batch_pts, batching, ao_floor)
        self._init_tile(tile, basis, grid, spin)

    @classmethod
    def new_with_gpu(cls, basis, grid, use_gpu=True, precision="fp64", batch_pts=128, batching="spatial",
                     tile="auto"):
        return cls(basis, grid, use_gpu, precision, batch_pts, batching=batching, tile=tile)

    def set_profiling(self, enable: bool = True):
        _native.check("calchem_xc_set_profiling", _native.load().calchem_xc_set_profiling(self.grid_id, int(enable)))
        self._profiling = bool(enable)

    def telemetry(self):
        """(gpu_kernel_invocations, gpu_fallback_invocations) as in vxc.rs:420-425."""
        return self.gpu_kernel_invocations, self.gpu_fallback_invocations

    def plan_stats(self):
        """(n_batches, sum m^2 n, sum m^2, max m) of the batch plan."""
        lib = _native.load()
        nb = np.zeros(1, np.int32)
        s1 = np.zeros(1)
        s2 = np.zeros(1)
        mm = np.zeros(1, np.int32)
        _native.check("calchem_xc_plan_stats", lib.calchem_xc_plan_stats(
            self.grid_id, _native.ptr(nb), _native.ptr(s1), _native.ptr(s2), _native.ptr(mm)))
        return int(nb[0]), float(s1[0]), float(s2[0]), int(mm[0])

    def set_ao_cache(self, enable: bool = True):
        """Allows (default) or frees and disables the tensor-core form's AO cache
        (calchem_xc_set_ao_cache): per-batch AO values, gradients and the packed operand kept in
        device memory across evaluations, as CalChem's engine keeps its AO cache across SCF
        iterations.  Results are the same either way."""
        _native.check("calchem_xc_set_ao_cache", _native.load().calchem_xc_set_ao_cache(
            self.grid_id, 1 if enable else 0, None))

    def ao_cache_bytes(self) -> int:
        """Bytes of the AO cache (0 before the first tensor-core evaluation, or when off)."""
        out = (ctypes.c_size_t * 1)()
        _native.check("calchem_xc_set_ao_cache", _native.load().calchem_xc_set_ao_cache(self.grid_id, -1, out))
        return int(out[0])

    def last_launch_count(self) -> int:
        return int(_native.load().calchem_xc_last_launch_count(self.grid_id))

    def nuclear_gradient(self, mol, grid, func, pa, pb=None, precision=None) -> np.ndarray:
        """dExc/dR [n_atoms][3] (Eh/Bohr) at fixed spin densities on this engine's grid, which must be
        the grid it was built from (calchem_xc_nuclear_gradient).  pb = None: closed shell (beta =
        alpha; pass P_total / 2).  precision: "fp64" or "mixed" (default: the engine's)."""
        lib = _native.load()
        Pa = _as_matrix(pa, self.n_ao)
        Pb = None if pb is None else _as_matrix(pb, self.n_ao)
        z = np.ascontiguousarray(mol.z, dtype=np.int32)
        xyz = np.ascontiguousarray(mol.coords_bohr, dtype=np.float64)
        raw = np.ascontiguousarray(grid.raw_weight, dtype=np.float64)
        host = np.ascontiguousarray(grid.host_atom, dtype=np.int32)
        out = np.zeros((len(z), 3), dtype=np.float64)
        prec = self.precision if precision is None else _PRECISION[precision]
        _native.check("calchem_xc_nuclear_gradient", lib.calchem_xc_nuclear_gradient(
            self.grid_id, _xc_code(func), prec, len(z), _native.ptr(z), _native.ptr(xyz), _native.ptr(raw),
            _native.ptr(host), len(raw), _native.ptr(Pa), None if Pb is None else _native.ptr(Pb), _native.ptr(out)))
        self.gpu_kernel_invocations += self.last_launch_count()
        return out

    def close(self):
        if self.grid_id:
            _native.load().calchem_cuda_vxc_release(self.grid_id)
            self.grid_id = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RksVxcEngine(_EngineBase):
    """Closed-shell engine: evaluate(basis, grid, func, P_total) -> (Exc, Vxc) (vxc.rs:720-726)."""

    def evaluate(self, basis, grid, func, density_total, precision=None):
        lib = _native.load()
        P = _as_matrix(density_total, self.n_ao)
        V = np.zeros((self.n_ao, self.n_ao), dtype=np.float64)
        exc = np.zeros(1)
        ne = np.zeros(1)
        prec = self.precision if precision is None else _PRECISION[precision]
        run = lambda: _native.check("calchem_xc_evaluate_rks", lib.calchem_xc_evaluate_rks(
            self.grid_id, _xc_code(func), prec, _native.ptr(P), _native.ptr(exc), _native.ptr(ne),
            _native.ptr(V)))
        if prec == MIXED and self.tile is None:
            self._tune_tile(func, run)
        run()
        self.gpu_kernel_invocations += self.last_launch_count()
        self.last_nelec = float(ne[0])
        return float(exc[0]), V


    def set_point_atoms(self, host_atom, n_atoms):
        """Host atom of every grid point (the grid's order), for evaluate_with_shares."""
        host = np.ascontiguousarray(host_atom, dtype=np.int32)
        _native.check("calchem_xc_set_point_atoms", _native.load().calchem_xc_set_point_atoms(
            self.grid_id, _native.ptr(host), len(host), int(n_atoms)))
        self._share_atoms = int(n_atoms)

    def evaluate_with_shares(self, basis, grid, func, density_total, precision=None):
        """evaluate() plus every atom's share of Exc and of tr(D Vxc) from the same build
        (calchem_xc_evaluate_rks_atoms): (Exc, Vxc, E_A, T_A).  set_point_atoms must come first."""
        lib = _native.load()
        n_at = getattr(self, "_share_atoms", 0)
        if n_at <= 0:
            raise ValueError("set_point_atoms first")
        P = _as_matrix(density_total, self.n_ao)
        V = np.zeros((self.n_ao, self.n_ao), dtype=np.float64)
        out = np.zeros(2 * n_at)
        exc, ne = np.zeros(1), np.zeros(1)
        prec = self.precision if precision is None else _PRECISION[precision]
        if prec == MIXED and self.tile is None:
            self.evaluate(basis, grid, func, density_total, precision)  # tunes the tile
        _native.check("calchem_xc_evaluate_rks_atoms", lib.calchem_xc_evaluate_rks_atoms(
            self.grid_id, _xc_code(func), prec, _native.ptr(P), _native.ptr(exc), _native.ptr(ne), _native.ptr(out),
            _native.ptr(V)))
        self.gpu_kernel_invocations += self.last_launch_count()
        self.last_nelec = float(ne[0])
        return float(exc[0]), V, out[0::2].copy(), out[1::2].copy()


class UksVxcEngine(_EngineBase):
    """Open-shell engine: evaluate(basis, grid, func, Pa, Pb) -> (Exc, Va, Vb) (vxc.rs:1662-1669)."""

    def evaluate(self, basis, grid, func, pa, pb, precision=None):
        lib = _native.load()
        Pa = _as_matrix(pa, self.n_ao)
        Pb = _as_matrix(pb, self.n_ao)
        Va = np.zeros((self.n_ao, self.n_ao), dtype=np.float64)
        Vb = np.zeros((self.n_ao, self.n_ao), dtype=np.float64)
        exc = np.zeros(1)
        ne = np.zeros(2)
        prec = self.precision if precision is None else _PRECISION[precision]
        run = lambda: _native.check("calchem_xc_evaluate_uks", lib.calchem_xc_evaluate_uks(
            self.grid_id, _xc_code(func), prec, _native.ptr(Pa), _native.ptr(Pb), _native.ptr(exc),
            _native.ptr(ne), _native.ptr(Va), _native.ptr(Vb)))
        if prec == MIXED and self.tile is None:
            self._tune_tile(func, run)
        run()
        self.gpu_kernel_invocations += self.last_launch_count()
        self.last_nelec = (float(ne[0]), float(ne[1]))
        return float(exc[0]), Va, Vb


def evaluate_vxc_rks(basis, grid, func, density_total, precision="fp64"):
    """evaluate_vxc_rks (vxc.rs:280-285): one-shot engine build + evaluate."""
    eng = RksVxcEngine(basis, grid, True, precision)
    try:
        return eng.evaluate(basis, grid, func, density_total)
    finally:
        eng.close()


def evaluate_vxc_uks(basis, grid, func, pa, pb, precision="fp64"):
    """evaluate_vxc_uks (vxc.rs:1352-1358)."""
    eng = UksVxcEngine(basis, grid, True, precision)
    try:
        return eng.evaluate(basis, grid, func, pa, pb)
    finally:
        eng.close()


def xc_nuclear_gradient_with_gpu(mol, basis, grid, func, pa, pb, use_gpu=True, precision="fp64"):
    """xc_nuclear_gradient_with_gpu (vxc.rs:2030-2333): (grad [n_atoms][3], gpu_kernel_invocations,
    gpu_fallback_invocations).  Equal pa and pb are treated as a closed shell, as the reference does
    (is_rks = pa == pb).  There is no CPU path: use_gpu=False raises."""
    if not use_gpu:
        raise NotImplementedError("calchem_gb300 evaluates the XC gradient on the GPU only; there is no CPU path")
    n_atoms = len(mol.z)
    if n_atoms <= 1 or basis.n_ao == 0 or len(grid.xyzw) == 0:
        return np.zeros((n_atoms, 3)), 0, 0
    pa = _as_matrix(pa, basis.n_ao)
    pb = _as_matrix(pb, basis.n_ao)
    closed = pa is pb or np.array_equal(pa, pb)
    eng = UksVxcEngine(basis, grid, True, precision)
    try:
        g = eng.nuclear_gradient(mol, grid, func, pa, None if closed else pb)
        return g, eng.gpu_kernel_invocations, 0
    finally:
        eng.close()


def xc_nuclear_gradient(mol, basis, grid, func, pa, pb, precision="fp64"):
    """xc_nuclear_gradient (vxc.rs:1903-1912): dExc/dR_A at fixed spin densities pa, pb (closed
    shell: pa = pb = P_total / 2), in Eh/Bohr, [n_atoms][3]; precision "mixed" runs the density
    contractions on the tensor cores."""
    return xc_nuclear_gradient_with_gpu(mol, basis, grid, func, pa, pb, True, precision)[0]


class _GroupGrid:
    """Point count of a group's members together (the autotuner's workload signature)."""

    def __init__(self, n):
        self.xyzw = np.empty((n, 0))


class VxcGroup(_TileMixin):
    """Many molecules, one persistent kernel launch per evaluation (calchem_xc_group_create).

    ``members`` is a sequence of (basis, grid) pairs.  Every member's grid is batched as a single
    engine would batch it, then all batches join one device work queue, so the per-member Exc and
    Nelec equal a single engine's bit for bit and the members share the GPU without a launch each.
    Densities and Vxc are exchanged as lists of per-member matrices (host) or as one packed device
    vector whose member blocks start at ``offsets`` (device and graph paths).
    """

    def __init__(self, members, precision="fp64", batch_pts=128, batching="spatial", tile="auto", ao_floor="auto"):
        lib = _native.load()
        self.precision = _PRECISION[precision]
        self.grid_id = 0
        self._profiling = False
        if ao_floor == "auto":
            ao_floor = default_ao_floor(precision) if batching == "spatial" else None
        self.ao_floor = ao_floor
        ids = []
        try:
            for basis, grid in members:
                ids.append(_upload_points(basis, grid, batch_pts, batching, ao_floor))
            gid = next(_ids)
            arr = np.array(ids, dtype=np.uint64)
            _native.check("calchem_xc_group_create", lib.calchem_xc_group_create(
                _native.ptr(arr), len(ids), gid, resolve_gpu_memory_limit()))
            self.grid_id = gid
        finally:
            for i in ids:
                lib.calchem_cuda_vxc_release(i)
        nm = np.zeros(1, np.int32)
        _native.check("calchem_xc_group_layout", lib.calchem_xc_group_layout(self.grid_id, _native.ptr(nm), None,
                                                                              None))
        self.n_mols = int(nm[0])
        self.sizes = np.zeros(self.n_mols, np.int32)
        self.offsets = np.zeros(self.n_mols, np.int64)
        _native.check("calchem_xc_group_layout", lib.calchem_xc_group_layout(
            self.grid_id, _native.ptr(nm), _native.ptr(self.sizes), _native.ptr(self.offsets)))
        self.packed_size = int(np.sum(self.sizes.astype(np.int64) ** 2))
        # the tile is tuned on the whole group (its members' first basis names the signature)
        self._init_tile(tile, members[0][0], _GroupGrid(sum(len(g.xyzw) for _, g in members)),
                        f"group{self.n_mols}")

    def set_profiling(self, enable: bool = True):
        _native.check("calchem_xc_set_profiling", _native.load().calchem_xc_set_profiling(self.grid_id, int(enable)))
        self._profiling = bool(enable)

    def pack(self, mats) -> np.ndarray:
        if len(mats) != self.n_mols:
            raise ValueError(f"expected {self.n_mols} matrices")
        out = np.empty(self.packed_size, dtype=np.float64)
        for i, m in enumerate(mats):
            n = int(self.sizes[i])
            out[self.offsets[i]:self.offsets[i] + n * n] = _as_matrix(m, n).ravel()
        return out

    def unpack(self, packed):
        return [np.array(packed[o:o + int(n) * int(n)]).reshape(int(n), int(n)) for n, o in zip(self.sizes, self.offsets)]

    def plan_stats(self):
        lib = _native.load()
        nb = np.zeros(1, np.int32)
        s1 = np.zeros(1)
        s2 = np.zeros(1)
        mm = np.zeros(1, np.int32)
        _native.check("calchem_xc_plan_stats", lib.calchem_xc_plan_stats(
            self.grid_id, _native.ptr(nb), _native.ptr(s1), _native.ptr(s2), _native.ptr(mm)))
        return int(nb[0]), float(s1[0]), float(s2[0]), int(mm[0])

    def set_ao_cache(self, enable: bool = True):
        """Allows (default) or frees and disables the tensor-core form's AO cache
        (calchem_xc_set_ao_cache): per-batch AO values, gradients and the packed operand kept in
        device memory across evaluations, as CalChem's engine keeps its AO cache across SCF
        iterations.  Results are the same either way."""
        _native.check("calchem_xc_set_ao_cache", _native.load().calchem_xc_set_ao_cache(
            self.grid_id, 1 if enable else 0, None))

    def ao_cache_bytes(self) -> int:
        """Bytes of the AO cache (0 before the first tensor-core evaluation, or when off)."""
        out = (ctypes.c_size_t * 1)()
        _native.check("calchem_xc_set_ao_cache", _native.load().calchem_xc_set_ao_cache(self.grid_id, -1, out))
        return int(out[0])

    def evaluate_rks(self, func, densities, precision=None):
        """-> (exc[n_mols], nelec[n_mols], [Vxc per member])."""
        lib = _native.load()
        P = self.pack(densities)
        V = np.zeros(self.packed_size)
        exc = np.zeros(self.n_mols)
        ne = np.zeros(self.n_mols)
        prec = self.precision if precision is None else _PRECISION[precision]
        run = lambda: _native.check("calchem_xc_evaluate_rks", lib.calchem_xc_evaluate_rks(
            self.grid_id, _xc_code(func), prec, _native.ptr(P), _native.ptr(exc), _native.ptr(ne), _native.ptr(V)))
        if prec == MIXED and self.tile is None:
            self._tune_tile(func, run)
        run()
        return exc, ne, self.unpack(V)

    def evaluate_uks(self, func, pas, pbs, precision=None):
        """-> (exc[n_mols], nelec[n_mols, 2], [Va], [Vb])."""
        lib = _native.load()
        Pa = self.pack(pas)
        Pb = self.pack(pbs)
        Va = np.zeros(self.packed_size)
        Vb = np.zeros(self.packed_size)
        exc = np.zeros(self.n_mols)
        ne = np.zeros(2 * self.n_mols)
        prec = self.precision if precision is None else _PRECISION[precision]
        run = lambda: _native.check("calchem_xc_evaluate_uks", lib.calchem_xc_evaluate_uks(
            self.grid_id, _xc_code(func), prec, _native.ptr(Pa), _native.ptr(Pb), _native.ptr(exc), _native.ptr(ne),
            _native.ptr(Va), _native.ptr(Vb)))
        if prec == MIXED and self.tile is None:
            self._tune_tile(func, run)
        run()
        return exc, ne.reshape(self.n_mols, 2), self.unpack(Va), self.unpack(Vb)

    def capture_rks(self, func, d_total: int, d_result: int, d_v: int, precision=None):
        """Captures one RKS evaluation on device buffers (addresses) into a CUDA graph."""
        prec = self.precision if precision is None else _PRECISION[precision]
        _native.check("calchem_xc_graph_capture", _native.load().calchem_xc_graph_capture(
            self.grid_id, 0, _xc_code(func), prec, d_total, None, d_result, d_v, None))

    def replay(self, stream: int = 0):
        _native.check("calchem_xc_graph_launch", _native.load().calchem_xc_graph_launch(self.grid_id, stream))

    def status(self) -> int:
        return int(_native.load().calchem_xc_last_status(self.grid_id))

    def close(self):
        if self.grid_id:
            _native.load().calchem_cuda_vxc_release(self.grid_id)
            self.grid_id = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FxcKernel:
    """TD-DFT exchange-correlation kernel (FxcKernel, fxc.rs:176-647): built from the ground-state
    total density, then contracted with batches of symmetric trial matrices on the GPU.  precision
    "fp64" (default) or "mixed" (the tensor-core contraction, calchem_xc_fxc_contract_ex)."""

    def __init__(self, basis, grid, func, density_total, precision="fp64"):
        lib = _native.load()
        self.n_ao = basis.n_ao
        self.precision = _PRECISION[precision]
        self.func = XcFunctional.from_name(func) if isinstance(func, str) else XcFunctional(func)
        self.grid_id = _upload_points(basis, grid)
        P = _as_matrix(density_total, self.n_ao)
        try:
            _native.check("calchem_xc_fxc_prepare", lib.calchem_xc_fxc_prepare(self.grid_id, _xc_code(func),
                                                                                _native.ptr(P)))
        except Exception:
            self.close()
            raise

    @classmethod
    def new(cls, basis, grid, func, density_total, precision="fp64"):
        return cls(basis, grid, func, density_total, precision)

    def functional(self):
        return self.func

    def contract_batch(self, d_sym_list, triplet=False, precision=None):
        """[dV_b] for the symmetric trial matrices (contract_batch, fxc.rs:374)."""
        if len(d_sym_list) == 0:
            return []
        n = self.n_ao
        M = np.ascontiguousarray(np.stack([_as_matrix(m, n) for m in d_sym_list]))
        out = np.zeros_like(M)
        prec = self.precision if precision is None else _PRECISION[precision]
        _native.check("calchem_xc_fxc_contract_ex", _native.load().calchem_xc_fxc_contract_ex(
            self.grid_id, int(bool(triplet)), prec, _native.ptr(M), len(d_sym_list), _native.ptr(out)))
        return [out[b] for b in range(len(d_sym_list))]

    def contract(self, m_sym, triplet=False, precision=None):
        return self.contract_batch([m_sym], triplet, precision)[0]

    def close(self):
        if self.grid_id:
            _native.load().calchem_cuda_vxc_release(self.grid_id)
            self.grid_id = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
