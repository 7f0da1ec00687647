"""Autotuner for the tensor-core quadrature's tile shape and the batch plan.

Two knobs are tuned by timing the quadrature kernel on the workload itself (CUDA events the library
records around the kernel, the minimum of a few repetitions after a warm-up that also fills the AO
cache), and the choice is cached under a signature of the workload (device, basis, element, AO and
point counts, functional, precision, spin):

* the GEMM1 tile (``TILES``): 64 AOs per TMEM accumulator with two CTAs per SM, or 128 AOs with one
  CTA per SM and all 512 TMEM columns.  The wider tile halves the GEMM1 rounds and the reloads of the
  packed AO operand per batch, which pays for batches with many AOs; the narrow one keeps two CTAs
  per SM, whose phases overlap each other.  Results do not depend on it (the same products are
  accumulated in the same order), so the tensor-core engines tune it by default, on their first
  evaluation.  The K block (64 AOs, one 128-byte swizzle atom of BF16) is fixed by the operand
  layout;
* the points per batch (``CANDIDATES``): smaller batches have smaller bounding spheres, so each
  point meets fewer candidate AOs (the work per batch is ~ m_b^2 n_b), but they mean more batches,
  more per-batch overhead and, on the tensor-core path, idle rows of the 128-row MMA tiles.  This
  changes the batch plan, and with it the summation order, so it is opt-in (``batch_pts="auto"``).

The cache is a JSON file, by default ``~/.cache/calchem_gb300/autotune.json``
(``CALCHEM_AUTOTUNE_CACHE`` overrides it).
"""

import json
import os
import threading

import numpy as np

CANDIDATES = (128, 96, 64)
TILES = (64, 128)
_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get("CALCHEM_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "calchem_gb300", "autotune.json")


def _device_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "cuda"


def signature(basis, grid, func, precision, spin) -> str:
    """Workload key: device, basis name, atom / AO / point counts (points to 3 significant digits),
    functional, precision and spin."""
    n_atoms = 1 + max((s.atom_index for s in basis.shells), default=0)
    n_pts = len(grid.xyzw)
    return (f"{_device_name()}|{basis.name}|atoms={n_atoms}|nao={basis.n_ao}|npts={n_pts:.3g}|"
            f"{str(func).lower()}|{precision}|{spin}")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value: dict) -> None:
    path = cache_path()
    data = _load()
    data[key] = value
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def best_of(times: dict, prefer) -> object:
    """The fastest candidate; ties go to the one ``prefer`` ranks first (smallest key)."""
    return min(times, key=lambda k: (times[k], prefer(k)))


def time_tiles(engine, run, reps=3, tiles=TILES) -> dict:
    """{tile: ms} of the quadrature kernel for each tile on an engine (``run()`` evaluates once)."""
    out = {}
    for t in tiles:
        engine.set_tile(t)
        run()  # warm-up (and the AO cache fill on the first)
        best = float("inf")
        for _ in range(reps):
            run()
            best = min(best, engine.last_kernel_ms())
        out[int(t)] = best
    return out


def choose_tile(key, measure) -> int:
    """The cached tile for a workload key, measuring first (``measure() -> {tile: ms}``) if there is
    none.  Ties go to the narrow tile."""
    tkey = key + "|tile"
    with _lock:
        hit = _load().get(tkey)
        if hit is not None and int(hit.get("tile_n", 0)) in TILES:
            return int(hit["tile_n"])
        times = {int(k): float(v) for k, v in measure().items()}
        best = best_of(times, lambda t: t)
        _store(tkey, {"tile_n": int(best), "ms": {str(k): v for k, v in times.items()}})
        return int(best)


def _kernel_ms(basis, grid, func, precision, spin, batch_pts, reps, tile=64) -> float:
    from . import workloads
    from .vxc import RksVxcEngine, UksVxcEngine
    S = basis.overlap()
    n_occ = max(1, basis.n_ao // 4)
    if spin == "rks":
        eng = RksVxcEngine(basis, grid, precision=precision, batch_pts=batch_pts, tile=tile)
        D = workloads.seeded_density_rks(S, n_occ, 7)
        run = lambda: eng.evaluate(basis, grid, func, D)
    else:
        eng = UksVxcEngine(basis, grid, precision=precision, batch_pts=batch_pts, tile=tile)
        Pa, Pb = workloads.seeded_density_uks(S, n_occ, max(1, n_occ - 1), 7, 8)
        run = lambda: eng.evaluate(basis, grid, func, Pa, Pb)
    try:
        eng.set_profiling(True)
        run()
        best = float("inf")
        for _ in range(reps):
            run()
            best = min(best, eng.last_kernel_ms())
        return best
    finally:
        eng.close()


def tune(basis, grid, func, precision="fp64", spin="rks", candidates=CANDIDATES, reps=3, measure=None,
         tiles=None) -> dict:
    """Times every (points per batch, tile) candidate; returns {"batch_pts": best, "tile_n": best,
    "ms": {"bp/tile": ms}}.  The FP64 form has one tile; the tensor-core form is timed with both.

    ``measure(batch_pts, tile) -> ms`` replaces the GPU timing (used to test the selection logic)."""
    if tiles is None:
        tiles = TILES if precision == "mixed" else (64,)
    if measure is None:
        measure = lambda bp, t: _kernel_ms(basis, grid, func, precision, spin, bp, reps, t)
    times = {(int(bp), int(t)): float(measure(int(bp), int(t))) for bp in candidates for t in tiles}
    best = best_of(times, lambda k: (-k[0], k[1]))  # ties go to the larger batch, then the narrow tile
    return {"batch_pts": best[0], "tile_n": best[1], "ms": {f"{k[0]}/{k[1]}": v for k, v in times.items()}}


def choose_plan(basis, grid, func, precision="fp64", spin="rks", measure=None) -> dict:
    """The cached (batch_pts, tile_n) for this workload, tuning it first if there is none."""
    key = signature(basis, grid, func, precision, spin)
    with _lock:
        hit = _load().get(key)
        if hit is not None and int(hit.get("batch_pts", 0)) in CANDIDATES and int(hit.get("tile_n", 0)) in TILES:
            return {"batch_pts": int(hit["batch_pts"]), "tile_n": int(hit["tile_n"])}
        res = tune(basis, grid, func, precision, spin, measure=measure)
        _store(key, res)
        return {"batch_pts": int(res["batch_pts"]), "tile_n": int(res["tile_n"])}


def choose_batch_pts(basis, grid, func, precision="fp64", spin="rks", measure=None) -> int:
    """The cached points per batch for this workload (``choose_plan``)."""
    return choose_plan(basis, grid, func, precision, spin, measure)["batch_pts"]
