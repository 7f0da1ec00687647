"""Autotuner for the batch plan: picks the points per batch (the block size of the persistent
kernels' work items) by timing the quadrature kernel on the workload itself, and caches the choice.

Smaller batches have smaller bounding spheres, so each point meets fewer candidate AOs (the work
per batch is ~ m_b^2 n_b), but they also mean more batches, more per-batch overhead and, on the
tensor-core path, idle rows of the 128-row MMA tiles.  Which wins depends on the molecule, the basis
and the grid, so it is measured: every candidate is planned, uploaded and timed with CUDA events
around the quadrature kernel (the minimum of a few repetitions after one warm-up), and the fastest
is stored under a signature of the workload (device, element counts, AO and point counts,
functional, precision, spin).  The cache is a JSON file, by default
``~/.cache/calchem_gb300/autotune.json`` (``CALCHEM_AUTOTUNE_CACHE`` overrides it).
"""

import json
import os
import threading

import numpy as np

CANDIDATES = (128, 96, 64)
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


def _kernel_ms(basis, grid, func, precision, spin, batch_pts, reps) -> float:
    from . import workloads
    from .vxc import RksVxcEngine, UksVxcEngine
    S = basis.overlap()
    n_occ = max(1, basis.n_ao // 4)
    if spin == "rks":
        eng = RksVxcEngine(basis, grid, precision=precision, batch_pts=batch_pts)
        D = workloads.seeded_density_rks(S, n_occ, 7)
        run = lambda: eng.evaluate(basis, grid, func, D)
    else:
        eng = UksVxcEngine(basis, grid, precision=precision, batch_pts=batch_pts)
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


def tune(basis, grid, func, precision="fp64", spin="rks", candidates=CANDIDATES, reps=3, measure=None) -> dict:
    """Times every candidate batch size; returns {"batch_pts": best, "ms": {candidate: ms}}.

    ``measure(batch_pts) -> ms`` replaces the GPU timing (used to test the selection logic)."""
    if measure is None:
        measure = lambda bp: _kernel_ms(basis, grid, func, precision, spin, bp, reps)
    times = {int(bp): float(measure(int(bp))) for bp in candidates}
    best = min(times, key=lambda k: (times[k], -k))  # ties go to the larger batch
    return {"batch_pts": best, "ms": {str(k): v for k, v in times.items()}}


def choose_batch_pts(basis, grid, func, precision="fp64", spin="rks", measure=None) -> int:
    """The cached choice for this workload, tuning it first if there is none."""
    key = signature(basis, grid, func, precision, spin)
    with _lock:
        hit = _load().get(key)
        if hit is not None and int(hit.get("batch_pts", 0)) in CANDIDATES:
            return int(hit["batch_pts"])
        res = tune(basis, grid, func, precision, spin, measure=measure)
        _store(key, res)
        return int(res["batch_pts"])
