"""Benchmark: Vxc build time per SCF iteration on one GB300.

Workload (the configuration the headline metric is quoted on): the 61-molecule water cluster
(H2O)61, 183 atoms, rigid waters at 1 g/cm^3 with O-O >= 2.6 Angstrom (PCG64 seed 61), B3LYP
(VWN_RPA), 6-31G(d) Cartesian (1159 AOs), seeded S-orthonormal density (244 occupied orbitals, seed
7).  One step = one SCF iteration's XC work on a built engine: the Vxc build (D -> Exc, Nelec, Vxc)
in the tensor-core form on the MLP-pruned grid with spatially compact batches, plus, on every
JUDGE_EVERY-th iteration, the periodic full-grid judge (per-atom shares of the pruned atoms on their
Fine and pruned points, tensor-core form, resident uploads), so the mean step is the per-iteration
cost with the judge amortised.  The FP64-plain comparison runs CalChem's batching (chunks of
consecutive points) on the full Fine grid.  The AO caches (per-batch AO values, gradients and packed
operand, kept across iterations as CalChem's RksVxcEngine keeps its AO cache) are filled before the
timed steps; the line reports the build without them as well.  ``--workload octane_b3lyp`` runs the
same line on n-octane C8H18 / 6-31G(d,p).

* value: mean device time of one step with D already resident in HBM, CUDA events on the launch
  stream, L2 flushed (256 MiB write) before every step.
* e2e: the same step through the host-buffer C ABI calls (calchem_xc_evaluate_rks, and
  calchem_xc_evaluate_rks_atoms for the judge), host<->device copies inside the timed region.
* roofline: the quadrature kernel of the build, algorithmic work 4 * sum_b m_b^2 n_b flops (RKS
  contractions) and 16 * sum_b m_b^2 + 32 N + 16 n^2 bytes, timed by CUDA events around that kernel.
* cpu_baseline: the oracle's restatement of CalChem's RksVxcEngine cached-AO CPU path (two
  contractions per batch by a register-blocked FMA GEMM, as CalChem's faer GEMM) on this host's
  cores, timed on a strided sample of CalChem's 128-point chunks of the Fine grid and scaled to the
  whole grid (the reference's Rust cannot be built offline).

``--impl reference`` times that CPU restatement as the reference arm (oracle only: the molecule,
basis, overlap, density and grid all come from the oracle and numpy).  With N > 1 GPUs (torchrun)
every rank runs an independent replica (the path is one GPU by design), and the reported value is
the maximum over ranks.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Vxc build ms/SCF iter on 1 GB300: mixed+pruned vs FP64 plain at dExc<=1e-6 Eh"
SEED = 7
PRUNE_TOL = 5e-7  # per-molecule quadrature tolerance of the learned grid against the Fine grid (Eh)
JUDGE_EVERY = 5   # SCF iterations between full-grid checks (calchem_gb300.scf's default)
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# The learned-grid RKS workloads: (molecule builder name and argument, basis, functional, description)
RKS_WORKLOADS = {
    "water61_b3lyp": (("water_cluster", (61, 61)), "6-31g(d)", "b3lyp",
                      "(H2O)61 water cluster, 183 atoms (rigid waters, 1 g/cm^3, O-O >= 2.6 A, PCG64 seed 61), "
                      "B3LYP (VWN_RPA), 6-31G(d) Cartesian 1159 AOs, CalChem Fine grid (99 radial shells, pruned "
                      "Lebedev, Becke) as judge, seeded S-orthonormal D (244 occ, seed 7)"),
    "water12_b3lyp": (("water_cluster", (12, 12)), "6-31g(d)", "b3lyp",
                      "(H2O)12 water cluster (rigid waters, 1 g/cm^3, O-O >= 2.6 A, PCG64 seed 12), B3LYP (VWN_RPA), "
                      "6-31G(d) Cartesian 228 AOs, CalChem Fine grid as judge, seeded S-orthonormal D (seed 7); "
                      "the profiling stand-in for the 61-water build (a few GB on the device)"),
    "octane_b3lyp": (("octane", ()), "6-31g(d,p)", "b3lyp",
                     "C8H18 all-trans, B3LYP (VWN_RPA), 6-31G(d,p) Cartesian 210 AOs, CalChem Fine grid "
                     "(99 radial shells, pruned Lebedev, Becke) as judge, seeded S-orthonormal D (33 occ, seed 7)"),
}
CLUSTERS_AO_CACHE_CAP = 60 << 30  # the 64-cluster group's AO-cache cap (bytes)
# DRAM bytes (read + write) per launch of the quadrature kernel from one ncu capture of the workload's
# timed build (profiles/); absent until a capture exists for the workload and precision.  The 61-water
# build is too large for a full capture: its figure is the 12-water capture (1.229 GB, 1.325 GB of AO
# cache) scaled by the AO-cache bytes (10.069 GB), the data that traffic grows with.
NCU_TRAFFIC_BYTES = {("octane_b3lyp", "mixed"): 1.925e9, ("water12_b3lyp", "mixed"): 1.229e9,
                     ("water61_b3lyp", "mixed"): 9.34e9}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", default="learned", choices=["learned", "fine"],
                    help="learned: the MLP-pruned grid with the periodic Fine-grid judge (RKS workloads)")
    ap.add_argument("--profile-case", action="store_true",
                    help="profiling case for ncu: the learned-grid build of an RKS workload on a fresh engine, "
                         "twice (the first fills the AO cache), tile 64, no judge, tuning, graph or baselines; "
                         "capture the second launch of the quadrature kernel")
    ap.add_argument("--workload", default="water61_b3lyp",
                    choices=["water61_b3lyp", "water12_b3lyp", "octane_b3lyp", "c54h18_pbe0_uks",
                             "water_clusters_pbe", "octane_b3lyp_gradient", "octane_b3lyp_fxc"],
                    help="water61_b3lyp is the headline; octane_b3lyp, the UKS flake and the 64-cluster batched "
                         "launch report the same line; octane_b3lyp_gradient times the XC nuclear gradient and "
                         "octane_b3lyp_fxc the TD-DFT kernel contraction (each its own metric)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(dist, value, device):
    """The largest of every rank's value (N replicas: the job takes as long as its slowest rank);
    the value itself with no process group."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rks_molecule(name):
    """(molecule, basis name, functional, description) of a learned-grid RKS workload (pure Python:
    no native library is loaded)."""
    from calchem_gb300 import workloads

    (builder, args), bname, func, desc = RKS_WORKLOADS[name]
    return getattr(workloads, builder)(*args), bname, func, desc


def build_inputs(name="octane_b3lyp"):
    """(molecule, basis, D) of an RKS workload with the product's basis and overlap."""
    from calchem_gb300 import BasisSet, workloads

    mol, bname, _, _ = rks_molecule(name)
    basis = BasisSet.from_name(bname, mol)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, SEED)
    return mol, basis, D


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_peak_tflops(torch, dev):
    """FP64 matmul throughput on this GPU (cuBLAS DGEMM 4096^3, best of 5): the FP64 roofline."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2 * 4096 ** 3 / (best * 1e-3) / 1e12


def roofline(flops, bytes_alg, kms, tc_peak, tc_unit_note, traffic, kernel, work):
    """Roofline of one launch after the definition used for this path: the contractions' flops at the
    tensor (or FP64) peak and the algorithmic HBM bytes at the measured copy bandwidth; the larger of
    the two times is the bound, and achieved / peak are given in that resource's unit."""
    pk, pk_kind = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    t_c = flops / (tc_peak * 1e12)
    t_m = bytes_alg / (hbm * 1e9)
    if t_m >= t_c:
        bound, achieved, peak, unit = "hbm", bytes_alg / (kms * 1e-3) / 1e9, hbm, "GB/s"
        note = f"measured copy bandwidth, {pk_kind}"
    else:
        bound, achieved, peak, unit = "tensor", flops / (kms * 1e-3) / 1e12, tc_peak, "TFLOP/s"
        note = tc_unit_note
    return {"bound": bound, "achieved": round(achieved, 4), "peak": round(peak, 3), "unit": unit,
            "frac": round(achieved / peak, 5), "traffic": traffic, "kernel": kernel, "kernel_ms": round(kms, 4),
            "work": work, "algorithmic_bytes": float(bytes_alg), "algorithmic_flop": float(flops),
            "roofline_ms": {"contractions": round(t_c * 1e3, 5), "hbm": round(t_m * 1e3, 5)},
            "peak_source": note}


def cpu_reference_run(name, steps, warmup, budget_s=20.0, fine_xyzw=None):
    """Times the oracle's restatement of CalChem's RksVxcEngine CPU path (cached-AO, both contractions
    by the register-blocked FMA GEMM, all host threads) on a strided sample of CalChem's 128-point
    chunks of the Fine grid, scaled to the whole grid.  Everything comes from the oracle and numpy
    (fine_xyzw: the Fine grid's points when the caller already has them; the oracle builds the same
    grid bit for bit otherwise).  Returns (ms per build, threads, sample description)."""
    from calchem_gb300 import workloads
    from oracle import oracle as O

    mol, bname, func, _ = rks_molecule(name)
    ob = O.Basis.from_name(bname, [a.symbol for a in mol.atoms], mol.coords_bohr)
    D = workloads.seeded_density_rks(ob.overlap(), mol.nelectron() // 2, SEED)
    if fine_xyzw is None:
        fine_xyzw = O.Grid.build(mol.z, mol.coords_bohr, "fine").points()[0]
    threads = O.max_threads()
    n_chunks = (len(fine_xyzw) + 127) // 128

    def sample(stride):
        idx = np.concatenate([np.arange(c * 128, min(c * 128 + 128, len(fine_xyzw)))
                              for c in range(0, n_chunks, stride)])
        eng = O.RksEngine(ob, O.Grid.from_points(fine_xyzw[idx]), cap_bytes=1e12)
        return eng, len(range(0, n_chunks, stride))

    # probe with a sparse sample, then size the sample so that (warmup + steps) builds take ~budget_s
    stride = max(1, n_chunks // 48)
    eng, k = sample(stride)
    t0 = time.perf_counter()
    eng.evaluate(D, func, blocked=True)
    per_chunk = (time.perf_counter() - t0) / k
    want = max(1, int(budget_s / ((warmup + steps) * per_chunk)))
    if want > k:
        stride = max(1, n_chunks // want)
        eng, k = sample(stride)
    for _ in range(warmup):
        eng.evaluate(D, func, blocked=True)
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        eng.evaluate(D, func, blocked=True)
        ts.append(time.perf_counter() - t0)
    scale = n_chunks / k
    ms = statistics.mean(ts) * 1e3 * scale
    desc = (f"CalChem RksVxcEngine::evaluate cached-AO path restated in C++ (oracle), both contractions by a "
            f"register-blocked FMA GEMM, {threads} threads; {steps} timed builds over every {stride}-th of "
            f"CalChem's {n_chunks} 128-point chunks of the Fine grid ({k} chunks, {len(fine_xyzw)} points in "
            f"all), scaled by {scale:.2f} to a full build")
    return ms, threads, desc


def cpu_group_run(mols, xyzws, dens, func, steps=3, n_sample=4, seed=5):
    """The oracle's restatement of CalChem's RksVxcEngine CPU path (cached-AO, register-blocked FMA
    GEMM, all host threads) for a batch of molecules, one engine per molecule as CalChem runs them:
    n_sample seeded molecules are timed and the total is scaled by the contraction work
    sum_b m_b^2 n_b of CalChem's batches over all molecules against the sampled ones."""
    from oracle import oracle as O

    total = 0.0
    bases = []
    for mol, xyzw in zip(mols, xyzws):
        ob = O.Basis.from_name("6-31g(d)", [a.symbol for a in mol.atoms], mol.coords_bohr)
        bases.append(ob)
        total += O.RksEngine(ob, O.Grid.from_points(xyzw), cap_bytes=0.0).work
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = sorted(rng.choice(len(mols), size=min(n_sample, len(mols)), replace=False).tolist())
    ms, work = 0.0, 0.0
    for i in pick:
        eng = O.RksEngine(bases[i], O.Grid.from_points(xyzws[i]), cap_bytes=1e12)
        work += eng.work
        eng.evaluate(dens[i], func, blocked=True)
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            eng.evaluate(dens[i], func, blocked=True)
            ts.append(time.perf_counter() - t0)
        ms += statistics.mean(ts) * 1e3
    threads = O.max_threads()
    scale = total / work
    desc = (f"CalChem RksVxcEngine::evaluate cached-AO path restated in C++ (oracle), both contractions by a "
            f"register-blocked FMA GEMM, {threads} threads, one engine per molecule; molecules {pick} of "
            f"{len(mols)} timed ({steps} builds each), scaled by the contraction work sum m^2 n of CalChem's "
            f"batches over all molecules ({scale:.2f}x the sample)")
    return ms * scale, threads, desc


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    name = getattr(args, "workload", "water61_b3lyp")
    if name not in RKS_WORKLOADS:
        name = "water61_b3lyp"
    ms, threads, sample = cpu_reference_run(name, args.steps, args.warmup, budget_s=60.0)
    line = {"metric": METRIC, "value": round(ms, 4), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": RKS_WORKLOADS[name][3], "name": name,
                       "path": "CPU, all host threads, Fine grid, CalChem's batching"},
            "cpu_baseline": {"value": round(ms, 4), "unit": "ms", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(ms, 4), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


class _Work:
    """One benchmark workload: the GPU objects, device buffers and the ways to run one step (device
    step, host-buffer step, FP64 plain comparison)."""

    def __init__(self, name, torch, dev, prec_name, grid_kind="fine"):
        from calchem_gb300 import (BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, VxcGroup,
                                   _native, pruner, workloads)
        from calchem_gb300.vxc import default_ao_floor
        self.name = name
        self.torch = torch
        self.dev = dev
        self.lib = _native.load()
        self.prec = 1 if prec_name == "mixed" else 0
        self.prec_name = prec_name
        self.graph = False
        self.lg = None       # learned grid with its resident judge
        self.judge = None
        # the FP64-plain comparison: CalChem's batching (chunks of consecutive points) on the Fine grid
        self.plain = None
        self.grid_info = {"grid": "Fine"}
        self.fine_xyzw = None
        if name in RKS_WORKLOADS:
            mol, basis, D = build_inputs(name)
            _, _, self.func, self.description = rks_molecule(name)
            grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
            self.fine_xyzw = grid.xyzw
            self.kind, self.xc = "rks", 3
            self.mats = [D]
            self.mol, self.basis = mol, basis
            if grid_kind == "learned":
                t0 = time.perf_counter()
                lg = pruner.LearnedGrid(mol, basis, tol=PRUNE_TOL)
                picked = lg.levels.copy()
                reverted, _ = lg.check(D, self.func, precision=prec_name)
                self.lg = lg
                self.judge = lg.fine_judge()
                self.grid_info = {"grid": f"MLP-pruned (per-atom tolerance {lg.tol_atom:.2e}, molecule {PRUNE_TOL:g}), "
                                          f"Fine-grid judge every {JUDGE_EVERY} iterations (timed, amortised into "
                                          f"value and e2e): the pruned atoms' Fine points evaluated for their "
                                          f"shares, the pruned grid's shares taken from that iteration's build",
                                  "grid_points_fine": len(grid), "grid_points_pruned": len(lg.grid),
                                  "atoms_pruned": int(len(lg.pruned_atoms())),
                                  "atoms_reverted_by_judge": len(reverted),
                                  "judge_points": int(lg.judge_points(with_pruned=False)),
                                  "judge_every": JUDGE_EVERY,
                                  "levels_picked": np.bincount(picked, minlength=len(pruner.LEVELS)).tolist(),
                                  "pruner_setup_s": round(time.perf_counter() - t0, 3)}
                grid_fine = grid
                grid = lg.grid
            else:
                grid_fine = grid
            self.plain = RksVxcEngine(basis, grid_fine, batching="reference")
            # the timed engine's plan: the tensor-core form's value screen (vxc.MIXED_AO_FLOOR)
            self.ao_floor = default_ao_floor(prec_name)
            self.obj = RksVxcEngine(basis, grid, ao_floor=self.ao_floor)
            self.grid_info["ao_floor"] = self.ao_floor
            if self.lg is not None:
                self.obj.set_point_atoms(grid.host_atom, len(mol.atoms))
            self.grid_obj = grid
            self.n_points = len(grid)
        elif name == "c54h18_pbe0_uks":
            mol, basis, func, (Pa, Pb) = workloads.build_workload("c54h18_pbe0_uks", SEED)
            grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
            self.kind, self.func, self.xc = "uks", "pbe0", 5
            self.obj = UksVxcEngine(basis, grid, ao_floor=default_ao_floor(prec_name))
            self.grid_info["ao_floor"] = default_ao_floor(prec_name)
            self.plain = UksVxcEngine(basis, grid, batching="reference")
            self.basis_obj, self.grid_obj = basis, grid
            self.mats = [Pa, Pb]
            self.n_points = len(grid)
            na, nb = mol.n_alpha_beta()
            self.description = (f"C54H18 circumcoronene flake (C-C 1.42, C-H 1.09 A, planar), UKS PBE0, 6-31G(d) "
                                f"Cartesian {basis.n_ao} AOs, Fine grid, seeded D (n_alpha {na}, n_beta {nb}, "
                                f"seeds {SEED}/{SEED + 1})")
        elif name == "water_clusters_pbe":
            # the group's AO cache would take ~150 GB at 32 B per AO and point: on a dedicated GB300
            # the cap is raised to 60 GiB (within the grid's 64 GiB budget), and the batches whose
            # blocks fit are cached (CALCHEM_MAX_AO_GRID_BYTES, read at the first tensor-core build)
            os.environ.setdefault("CALCHEM_MAX_AO_GRID_BYTES", str(CLUSTERS_AO_CACHE_CAP))
            self.grid_info["ao_cache_cap_bytes"] = int(os.environ["CALCHEM_MAX_AO_GRID_BYTES"])
            sizes = workloads.cluster_batch_sizes()
            members, dens, self.cluster_mols = [], [], []
            for i, k in enumerate(sizes):
                mol = workloads.water_cluster(k, 1000 + i)
                basis = BasisSet.from_name("6-31g(d)", mol)
                grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
                members.append((basis, grid))
                self.cluster_mols.append(mol)
                dens.append(workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, SEED + i))
            self.cluster_xyzw = [g.xyzw for _, g in members]
            self.kind, self.func, self.xc = "group", "pbe", 2
            self.obj = VxcGroup(members, precision=prec_name)
            self.grid_info["ao_floor"] = self.obj.ao_floor
            self.plain = VxcGroup(members, precision="fp64", batching="reference")
            self.mats = dens
            self.n_points = sum(len(g) for _, g in members)
            self.description = (f"{len(sizes)} water clusters of 1-32 rigid waters (sizes PCG64 seed 2024, total "
                                f"{sum(sizes)} waters, 1 g/cm^3, O-O >= 2.6 A, placement seeds 1000+i), PBE, "
                                f"6-31G(d) Cartesian, Fine grid, seeded D; one persistent launch per build, "
                                f"replayed as a CUDA graph")
        else:
            raise ValueError(name)
        self.n_batches, self.sum_m2n, self.sum_m2, self.max_m = self.obj.plan_stats()
        self.flops = (8.0 if self.kind == "uks" else 4.0) * self.sum_m2n
        # packed device buffers
        if self.kind == "group":
            self.packed = [self.obj.pack(self.mats)]
            self.n_mols = self.obj.n_mols
            nn = self.obj.packed_size
        else:
            self.packed = [np.ascontiguousarray(m).ravel() for m in self.mats]
            self.n_mols = 1
            nn = self.packed[0].size
        self.nn = nn
        self.dP = [torch.from_numpy(p).to(dev) for p in self.packed]
        self.dV = [torch.zeros(nn, dtype=torch.float64, device=dev) for _ in self.packed]
        self.dres = torch.zeros(3 * self.n_mols + 1, dtype=torch.float64, device=dev)
        if self.judge is not None:
            n_at = len(self.mol.atoms)
            self.djudge_res = torch.zeros(4, dtype=torch.float64, device=dev)
            # [the Fine judge's shares | the build's shares], 2 n_atoms each
            self.djudge_atoms = torch.zeros(4 * n_at, dtype=torch.float64, device=dev)

    @property
    def gid(self):
        return self.obj.grid_id

    def tune(self):
        """The autotuner's tile choice for this workload (timed on its first tensor-core evaluation,
        or taken from the cache), applied to the build and the judge uploads before the capture."""
        from calchem_gb300 import autotune
        if self.prec != 1:
            return None
        if self.kind == "group":
            self.obj.evaluate_rks(self.func, self.mats)
            sig = autotune.signature(self.obj._tile_src[0], self.obj._tile_src[1], self.func, "mixed",
                                     self.obj._tile_src[2])
        elif self.kind == "uks":
            self.obj.evaluate(self.basis_obj, self.grid_obj, self.func, *self.mats, precision="mixed")
            sig = autotune.signature(self.basis_obj, self.grid_obj, self.func, "mixed", "uks")
        else:
            self.obj.evaluate(self.basis, self.grid_obj, self.func, self.mats[0], precision="mixed")
            sig = autotune.signature(self.basis, self.grid_obj, self.func, "mixed", "rks")
        if self.judge is not None:
            self.judge.set_tile(self.obj.tile)
        rec = autotune._load().get(sig + "|tile", {})
        return {"tile_n": self.obj.tile, "ctas_per_sm": 1 if self.obj.tile == 128 else 2,
                "autotuned": True, "kernel_ms_by_tile": rec.get("ms")}

    def n_ao(self):
        return int(np.sqrt(self.nn)) if self.kind != "group" else int(self.obj.sizes.max())

    def enable_profiling(self):
        from calchem_gb300 import _native
        _native.check("calchem_xc_set_profiling", self.lib.calchem_xc_set_profiling(self.gid, 1))

    def capture(self):
        """Each timed build is replayed from a CUDA graph (device buffers fixed): split, quadrature,
        reductions and symmetrisation in one launch."""
        from calchem_gb300 import _native
        uks = self.kind == "uks"
        _native.check("calchem_xc_graph_capture", self.lib.calchem_xc_graph_capture(
            self.gid, 1 if uks else 0, self.xc, self.prec, self.dP[0].data_ptr(),
            self.dP[1].data_ptr() if uks else None, self.dres.data_ptr(), self.dV[0].data_ptr(),
            self.dV[1].data_ptr() if uks else None))
        self.graph = True

    def device_step(self, stream, prec=None, plain=False, direct=False):
        """plain: the FP64-plain comparison object (prec is then FP64 unless given); direct: enqueue
        the calls instead of replaying the captured graph."""
        prec = (0 if plain else self.prec) if prec is None else prec
        gid = self.plain.grid_id if plain else self.gid
        if self.graph and prec == self.prec and not plain and not direct:
            return self.lib.calchem_xc_graph_launch(self.gid, stream.cuda_stream)
        if self.kind == "uks":
            return self.lib.calchem_xc_evaluate_uks_device(
                gid, self.xc, prec, self.dP[0].data_ptr(), self.dP[1].data_ptr(), self.dres.data_ptr(),
                self.dV[0].data_ptr(), self.dV[1].data_ptr(), stream.cuda_stream)
        return self.lib.calchem_xc_evaluate_rks_device(gid, self.xc, prec, self.dP[0].data_ptr(),
                                                       self.dres.data_ptr(), self.dV[0].data_ptr(),
                                                       stream.cuda_stream)

    def judge_step(self, stream):
        """An SCF iteration that runs the periodic full-grid check, on the device: the build with every
        atom's shares (direct launches: calchem_xc_evaluate_rks_atoms_device with Vxc), then the shares
        of the pruned atoms' Fine points (resident upload, D already on the device)."""
        n_at = len(self.mol.atoms)
        rc = self.lib.calchem_xc_evaluate_rks_atoms_device(
            self.gid, self.xc, self.prec, self.dP[0].data_ptr(), self.dres.data_ptr(), self.dV[0].data_ptr(),
            self.djudge_atoms.data_ptr() + 16 * n_at, stream.cuda_stream)
        if rc:
            return rc
        return self.judge.enqueue(self.dP[0].data_ptr(), self.djudge_res.data_ptr(), self.djudge_atoms.data_ptr(),
                                  stream.cuda_stream, self.func, self.prec_name)

    def judge_launches(self):
        """Kernels of the last judge iteration (its build and the Fine judge)."""
        return (self.lib.calchem_xc_last_launch_count(self.gid) +
                self.lib.calchem_xc_last_launch_count(self.judge.grid_id)) if self.judge else 0

    def host_step(self, prec=None, plain=False):
        """The reference-facing host-buffer call (copies inside); returns (exc[], nelec[], [V...])."""
        from calchem_gb300 import _native
        prec = self.prec if prec is None else prec
        gid = self.plain.grid_id if plain else self.gid
        exc = np.zeros(self.n_mols)
        if self.kind == "uks":
            ne = np.zeros(2)
            Va, Vb = np.zeros(self.nn), np.zeros(self.nn)
            _native.check("calchem_xc_evaluate_uks", self.lib.calchem_xc_evaluate_uks(
                gid, self.xc, prec, _native.ptr(self.packed[0]), _native.ptr(self.packed[1]), _native.ptr(exc),
                _native.ptr(ne), _native.ptr(Va), _native.ptr(Vb)))
            return exc, ne, [Va, Vb]
        ne = np.zeros(self.n_mols)
        V = np.zeros(self.nn)
        _native.check("calchem_xc_evaluate_rks", self.lib.calchem_xc_evaluate_rks(
            gid, self.xc, prec, _native.ptr(self.packed[0]), _native.ptr(exc), _native.ptr(ne), _native.ptr(V)))
        return exc, ne, [V]

    def host_judge_step(self):
        """A judge iteration through the host-buffer calls, as the SCF loop runs it: the build with its
        per-atom shares (D in; Exc, Nelec, Vxc and the shares out), the Fine judge's shares, and the
        comparison on the host."""
        exc, V, E, T = self.obj.evaluate_with_shares(self.basis, self.grid_obj, self.func, self.mats[0],
                                                     precision=self.prec_name)
        E0, T0 = self.judge.shares(self.mats[0], self.func, self.prec_name)
        at = self.lg.pruned_atoms()
        err = np.maximum(np.abs(E - E0), np.abs(T - T0))[at]
        return exc, V, int(np.sum(err > self.lg.tol_atom))

    def io_bytes(self):
        k = len(self.packed)
        return k * self.nn * 8, k * self.nn * 8 + (3 if self.kind == "uks" else 2) * 8 * self.n_mols

    def judge_io_bytes(self):
        """Extra copies of a judge iteration: D in for the Fine judge, its (Exc, Nelec) and per-atom
        shares out, and the build's per-atom shares out."""
        n_at = len(self.mol.atoms)
        return self.nn * 8, 2 * 8 + 2 * (2 * n_at * 8)

    def close(self):
        self.obj.close()
        if self.plain is not None:
            self.plain.close()
        if self.lg is not None:
            self.lg.close()


def run_ours(args):
    import torch

    from calchem_gb300 import _native

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    dev = torch.device("cuda", torch.cuda.current_device())
    prec_name = "mixed" if args.precision == "auto" else args.precision
    W = _Work(args.workload, torch, dev, prec_name, args.grid if args.workload in RKS_WORKLOADS else "fine")
    lib = W.lib
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    t_first = time.perf_counter()
    W.host_step()  # allocates the workspace (and fills the AO cache) outside the capture
    torch.cuda.synchronize()
    first_ms = (time.perf_counter() - t_first) * 1e3
    if W.judge is not None:
        # the judge's first check fills its own AO cache and the build's per-point share buffers,
        # once per geometry as the build's first evaluation does: set-up, not a timed iteration
        W.host_judge_step()
        torch.cuda.synchronize()
    tile = W.tune()  # the tile is chosen before the capture, which keeps it
    if tile:
        W.grid_info["tile"] = tile
    W.enable_profiling()
    W.capture()
    torch.cuda.synchronize()
    judged = W.judge is not None

    def step(i, direct=False):
        if judged and i % JUDGE_EVERY == JUDGE_EVERY - 1:
            _native.check("judge iteration", W.judge_step(stream))
        else:
            _native.check("evaluate", W.device_step(stream, direct=direct))

    for i in range(max(3, args.warmup)):
        with torch.cuda.stream(stream):
            flush.zero_()
        step(i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    step_ms, kern_ms = [], []
    launches = 0
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        step(i)
        e.record(stream)
        e.synchronize()
        step_ms.append(s.elapsed_time(e))
        if judged and i % JUDGE_EVERY == JUDGE_EVERY - 1:
            launches += W.judge_launches()
        else:
            launches += lib.calchem_xc_last_launch_count(W.gid)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    _native.check("device status", lib.calchem_xc_last_status(W.gid))
    res_dev = W.dres.cpu().numpy()
    ms = statistics.mean(step_ms)
    # a plain iteration (the build) and a judge iteration, each on the device
    build_ms, judge_ms = [], []
    for _ in range(5):
        for which in ("build", "judge") if judged else ("build",):
            with torch.cuda.stream(stream):
                flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            _native.check(which, W.device_step(stream) if which == "build" else W.judge_step(stream))
            e.record(stream)
            e.synchronize()
            (build_ms if which == "build" else judge_ms).append(s.elapsed_time(e))
    for _ in range(3):  # graph replays: time the quadrature kernel outside the graph
        with torch.cuda.stream(stream):
            flush.zero_()
        _native.check("evaluate", W.device_step(stream, direct=True))
        km = np.zeros(1, np.float32)
        _native.check("last_kernel_ms", lib.calchem_xc_last_kernel_ms(W.gid, _native.ptr(km)))
        kern_ms.append(float(km[0]))
    kms = statistics.mean(kern_ms)
    ms = max_over_ranks(dist, ms, dev)
    # ---- e2e through the host-buffer C ABI calls (copies inside the timed region)
    e2e = []
    host = None
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if judged and i % JUDGE_EVERY == JUDGE_EVERY - 1:
            W.host_judge_step()
        else:
            host = W.host_step()
        if i >= args.warmup:
            e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.mean(e2e)
    # ---- the FP64 plain form (CalChem's batching, Fine grid), for the timed-vs-plain comparison
    ref_fp64 = {}
    if W.plain is not None:
        ef, nf, Vf = W.host_step(prec=0, plain=True)

        def timed(fn, reps=3):
            ts = []
            for _ in range(reps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                torch.cuda.synchronize()
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record(stream)
                _native.check("evaluate", fn())
                e.record(stream)
                e.synchronize()
                ts.append(s.elapsed_time(e))
            return statistics.mean(ts)

        fts = timed(lambda: W.device_step(stream, prec=0, plain=True))
        # the gains one at a time: FP64 on the timed build's own grid and batches, and (learned grid)
        # the timed precision on the Fine grid with CalChem's batching
        W.grid_info["fp64_same_plan_ms"] = round(timed(lambda: W.device_step(stream, prec=0)), 4)
        if judged:
            W.grid_info["mixed_on_fine_grid_reference_batching_ms"] = round(timed(
                lambda: W.device_step(stream, prec=W.prec, plain=True)), 4)
        dexc = host[0] - ef
        ref_fp64 = {"fp64_plain_ms": round(fts, 4),
                    "speedup_vs_fp64_plain": round(fts / ms, 3),
                    "dExc_vs_fp64": float(dexc[np.argmax(np.abs(dexc))]),
                    "dNelec_vs_fp64": float(np.max(np.abs(host[1] - nf))),
                    "max_abs_dV_vs_fp64": float(max(np.max(np.abs(a - b)) for a, b in zip(host[2], Vf)))}
        if W.n_mols > 1:
            ref_fp64["dExc_vs_fp64_is"] = "largest |dExc| over the molecules"
    if W.prec == 1:
        # the AO cache: its size, the first build (which fills it) and a build with it off
        W.grid_info["ao_cache_bytes"] = W.obj.ao_cache_bytes()
        if judged:
            W.grid_info["judge_ao_cache_bytes"] = int(W.judge.ao_cache_bytes())
        W.grid_info["first_build_wall_ms"] = round(first_ms, 4)  # host call: workspace and cache allocation, fill
        W.obj.set_ao_cache(False)
        nts = []
        for _ in range(3):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            _native.check("evaluate", W.device_step(stream, direct=True))
            e.record(stream)
            e.synchronize()
            nts.append(s.elapsed_time(e))
        W.grid_info["no_ao_cache_ms"] = round(statistics.mean(nts), 4)
    pk, pk_kind = peaks()
    if W.prec == 1:
        tc_peak, peak_note = pk.get("bf16_tflops", 1900.0), f"dense bf16 burst, {pk_kind}"
    else:
        tc_peak = fp64_peak_tflops(torch, dev)
        peak_note = "FP64 pipe: cuBLAS DGEMM 4096^3 measured in this run (no FP64 figure in the measured peaks)"
    traffic = NCU_TRAFFIC_BYTES.get((W.name, prec_name)) if judged else None
    nspin = 2 if W.kind == "uks" else 1
    # algorithmic bytes per build: D_sub gathered and V_sub scattered per batch and spin (8 B each per
    # AO pair), the points (x, y, z, w), and D in and V out once
    bytes_alg = nspin * 16.0 * W.sum_m2 + 32.0 * W.n_points + nspin * 16.0 * W.nn
    h2d, d2h = W.io_bytes()
    if judged:
        jh, jd = W.judge_io_bytes()
        h2d += jh / JUDGE_EVERY
        d2h += jd / JUDGE_EVERY
    line = {
        "metric": METRIC, "value": round(ms, 4), "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if W.prec == 0 else "bf16x3 split (f32 accumulate) contractions, f64 functional/sums",
        "data": "synthetic",
        "config": {"workload": W.description, "name": W.name, "precision": prec_name, **W.grid_info, "n_ao": W.n_ao(),
                   "molecules": W.n_mols, "grid_points": W.n_points, "batches": W.n_batches, "max_m": W.max_m,
                   "l2": "flushed before every timed step (256 MiB write)",
                   "graph": "CUDA-graph replay of the build per step" if W.graph else "direct launches",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "build_ms": round(statistics.mean(build_ms), 4),
        "grid_points_per_s": round(W.n_points / (statistics.mean(build_ms) * 1e-3), 1),
        "median_ms_per_step": round(statistics.median(step_ms), 4),
        "exc": float(res_dev[0]), "nelec": float(res_dev[1]),
        "roofline": roofline(W.flops, bytes_alg, kms, tc_peak, peak_note, traffic, "vxc quadrature kernel",
                             f"{'8' if W.kind == 'uks' else '4'}*sum(m^2 n) = {W.flops:.4e} flop; "
                             f"{16 * nspin}*sum(m^2) + 32 N + {16 * nspin} n^2 = {bytes_alg:.4e} B per launch"),
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "wall_s_timed": round(t_wall, 3),
        "clocks": clk,
    }
    if judged:
        extra = statistics.mean(judge_ms) - statistics.mean(build_ms)
        line["judge_iteration_ms"] = round(statistics.mean(judge_ms), 4)
        line["judge_ms"] = round(extra, 4)  # what a judge iteration costs beyond a plain one
        line["judge_ms_per_iteration"] = round(extra / JUDGE_EVERY, 4)
    line.update(ref_fp64)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline and W.name in RKS_WORKLOADS:
        cms, threads, sample = cpu_reference_run(W.name, 3, 1, budget_s=20.0, fine_xyzw=W.fine_xyzw)
        line["cpu_baseline"] = {"value": round(cms, 3), "unit": "ms", "cores": threads, "kind": "port",
                                "sample": sample}
    elif rank == 0 and ws == 1 and not args.no_cpu_baseline and W.name == "water_clusters_pbe":
        cms, threads, sample = cpu_group_run(W.cluster_mols, W.cluster_xyzw, W.mats, W.func)
        line["cpu_baseline"] = {"value": round(cms, 3), "unit": "ms", "cores": threads, "kind": "port",
                                "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    W.close()
    if dist:
        dist.destroy_process_group()
    return 0


GRADIENT_METRIC = "XC nuclear gradient dExc/dR ms on 1 GB300: tensor-core form vs FP64 plain (fixed density)"


def cpu_gradient_sample(mol, basis, grid, Pa, func, n_sample=4000):
    """The oracle's restatement of xc_nuclear_gradient_cpu (vxc.rs:1914-2024) on every k-th point of
    the grid, scaled to the whole grid: (ms, sample description)."""
    from oracle import oracle as O

    stride = max(1, len(grid) // n_sample)
    idx = np.arange(0, len(grid), stride)
    og = O.Grid.from_points(grid.xyzw[idx], grid.host_atom[idx], grid.raw_weight[idx])
    ob = O.Basis.from_name("6-31g(d,p)", [a.symbol for a in mol.atoms], mol.coords_bohr)
    O.xc_gradient(ob, og, mol.z, mol.coords_bohr, Pa, Pa, func)  # warm-up (tables)
    t0 = time.perf_counter()
    O.xc_gradient(ob, og, mol.z, mol.coords_bohr, Pa, Pa, func)
    t = time.perf_counter() - t0
    ms = t * 1e3 * len(grid) / len(idx)
    return ms, (f"oracle xc_gradient (per point: AO Hessians, P contractions, functional, Becke derivative; "
                f"1 thread) on every {stride}-th point ({len(idx)} of {len(grid)}), scaled to the full grid")


def run_gradient(args):
    """One step = one XC nuclear gradient (calchem_xc_nuclear_gradient) of the headline workload on
    its Fine grid at the seeded closed-shell density (P_alpha = D / 2); the tensor-core form unless
    --precision fp64, with the FP64 form timed beside it."""
    import torch

    from calchem_gb300 import GridLevel, MolecularGrid, RksVxcEngine

    ws, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    prec = "fp64" if args.precision == "fp64" else "mixed"
    mol, basis, D = build_inputs("octane_b3lyp")
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    eng = RksVxcEngine(basis, grid)
    eng.set_profiling(True)
    # the FP64-plain comparison on CalChem's batching of consecutive points
    plain = RksVxcEngine(basis, grid, batching="reference")
    plain.set_profiling(True)
    Pa = 0.5 * D
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(precision, steps, e=eng):
        kern, wall, g = [], [], None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g = e.nuclear_gradient(mol, grid, "b3lyp", Pa, precision=precision)
            wall.append((time.perf_counter() - t0) * 1e3)
            kern.append(e.last_kernel_ms())
        return kern, wall, g

    timed(prec, max(3, args.warmup))
    n0 = eng.gpu_kernel_invocations
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    kern, wall, g = timed(prec, args.steps)
    clk = clocks.stop()
    launches = eng.gpu_kernel_invocations - n0
    k64, _, g64 = timed("fp64", 2, plain)
    k64_same, _, _ = timed("fp64", 2)
    n_batches, sum_m2n, _, max_m = eng.plan_stats()
    flops = 4.0 * sum_m2n  # T = P Phi and Y = P Psi, 2 m^2 n each (closed shell)
    kms = statistics.mean(kern)
    if prec == "mixed":
        pk, pk_kind = peaks()
        tc_peak, peak_note = pk.get("bf16_tflops", 1900.0), f"dense bf16 burst, {pk_kind}"
    else:
        tc_peak, peak_note = fp64_peak_tflops(torch, dev), "FP64 pipe: cuBLAS DGEMM 4096^3 measured in this run"
    sum_m2 = eng.plan_stats()[2]
    # D_sub gathered for T and for Y per batch, the points (x, y, z, w, raw w, host), D in
    bytes_alg = 16.0 * sum_m2 + 44.0 * len(grid) + 8.0 * basis.n_ao ** 2
    n = basis.n_ao
    line = {
        "metric": GRADIENT_METRIC, "value": round(kms, 4), "unit": "ms", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(kms, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if prec == "fp64" else "bf16x4 fixed-point split contractions, df32 AO/forces/weights, f64 functional",
        "data": "synthetic",
        "config": {"workload": RKS_WORKLOADS["octane_b3lyp"][3] + "; XC nuclear gradient at P_alpha = D / 2", "name": args.workload,
                   "precision": prec, "grid_points": len(grid), "batches": n_batches, "max_m": max_m,
                   "atoms": len(mol.z), "l2": "flushed before every timed step (256 MiB write)"},
        "roofline": roofline(flops, bytes_alg, kms, tc_peak, peak_note, None, "gradient kernels + split + reduce",
                             f"4*sum(m^2 n) = {flops:.4e} flop of AO contractions (weight derivative not counted); "
                             f"16*sum(m^2) + 44 N + 8 n^2 = {bytes_alg:.4e} B per gradient"),
        "e2e": {"value": round(statistics.mean(wall), 4), "unit": "ms",
                "h2d_bytes_per_step": n * n * 8 + len(grid) * 12, "d2h_bytes_per_step": len(mol.z) * 24},
        "gpu_launches": launches, "clocks": clk,
        "fp64_plain_ms": round(statistics.mean(k64), 4),
        "speedup_vs_fp64_plain": round(statistics.mean(k64) / kms, 3),
        "fp64_same_plan_ms": round(statistics.mean(k64_same), 4),
        "max_abs_dgrad_vs_fp64": float(np.max(np.abs(g - g64))),
        "max_abs_grad": float(np.max(np.abs(g))), "sum_over_atoms": float(np.max(np.abs(g.sum(axis=0)))),
    }
    if not args.no_cpu_baseline:
        cms, sample = cpu_gradient_sample(mol, basis, grid, Pa, "b3lyp")
        line["cpu_baseline"] = {"value": round(cms, 2), "unit": "ms", "cores": 1, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    plain.close()
    return 0


FXC_METRIC = "TD-DFT kernel contraction ms per batch of 16 trial matrices on 1 GB300: tensor-core vs FP64"
FXC_TRIALS = 16


def run_fxc(args):
    """One step = one FxcKernel.contract_batch of 16 seeded symmetric trial matrices (host buffers in
    and out, calchem_xc_fxc_contract_ex) on the headline molecule's Fine grid at its ground-state
    density; the tensor-core form unless --precision fp64, with the FP64 form timed beside it."""
    import torch

    from calchem_gb300 import FxcKernel, GridLevel, MolecularGrid

    ws, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    prec = "fp64" if args.precision == "fp64" else "mixed"
    mol, basis, D = build_inputs("octane_b3lyp")
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    ker = FxcKernel(basis, grid, "b3lyp", D, precision=prec)
    rng = np.random.default_rng(SEED)
    mats = [0.01 * (lambda a: a + a.T)(rng.normal(size=D.shape)) for _ in range(FXC_TRIALS)]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(precision, steps):
        ts, out = [], None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = ker.contract_batch(mats, precision=precision)
            ts.append((time.perf_counter() - t0) * 1e3)
        return ts, out

    timed(prec, max(3, args.warmup))
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ts, out = timed(prec, args.steps)
    clk = clocks.stop()
    t64, ref = timed("fp64", 2)
    ms = statistics.mean(ts)
    n = basis.n_ao
    rel = max(float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(out, ref))
    line = {
        "metric": FXC_METRIC, "value": round(ms, 4), "unit": "ms", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "bf16x4 fixed-point / bf16x3 split contractions",
        "data": "synthetic",
        "config": {"workload": RKS_WORKLOADS["octane_b3lyp"][3] + f"; TD-DFT kernel contraction of {FXC_TRIALS} seeded symmetric trial "
                                          "matrices (singlet) at the ground-state density",
                   "name": args.workload, "precision": prec, "grid_points": len(grid), "trials": FXC_TRIALS,
                   "l2": "flushed before every timed step (256 MiB write)", "timing": "host wall clock of the "
                   "host-buffer call, copies included"},
        "e2e": {"value": round(ms, 4), "unit": "ms", "h2d_bytes_per_step": FXC_TRIALS * n * n * 8,
                "d2h_bytes_per_step": FXC_TRIALS * n * n * 8},
        "gpu_launches": 3 * FXC_TRIALS if prec == "mixed" else 1 + FXC_TRIALS,
        "clocks": clk,
        "fp64_plain_ms": round(statistics.mean(t64), 4),
        "speedup_vs_fp64_plain": round(statistics.mean(t64) / ms, 3),
        "max_rel_dV_vs_fp64": rel,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ker.close()
    return 0


def run_profile_case(args):
    """Two builds of the workload's learned-grid engine (tensor-core form unless --precision fp64); the
    second reads the AO cache, as every timed build does.  Prints the kernel times."""
    from calchem_gb300 import RksVxcEngine, pruner

    mol, basis, D = build_inputs(args.workload)
    _, _, func, _ = rks_molecule(args.workload)
    lg = pruner.LearnedGrid(mol, basis, tol=PRUNE_TOL)
    prec = "fp64" if args.precision == "fp64" else "mixed"
    eng = RksVxcEngine(basis, lg.grid, precision=prec, tile=64)
    eng.set_profiling(True)
    ms = []
    for _ in range(2):
        eng.evaluate(basis, lg.grid, func, D)
        ms.append(eng.last_kernel_ms())
    n_batches, sum_m2n, sum_m2, max_m = eng.plan_stats()
    print(json.dumps({"profile_case": args.workload, "precision": prec, "grid_points": len(lg.grid),
                      "batches": n_batches, "sum_m2n": sum_m2n, "sum_m2": sum_m2, "max_m": max_m,
                      "ao_cache_bytes": eng.ao_cache_bytes(), "kernel_ms": ms}), flush=True)
    eng.close()
    lg.close()
    return 0


def main():
    args = parse()
    if args.profile_case:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "octane_b3lyp_gradient":
        return run_gradient(args)
    if args.workload == "octane_b3lyp_fxc":
        return run_fxc(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
