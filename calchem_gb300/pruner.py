"""Learned grid pruning: per-atom radial and angular orders chosen by a small MLP, with the Fine
grid as fallback and judge.

The quadrature of a Becke-partitioned grid is a sum of atomic-cell integrals, so every atom's share
of Exc (and of tr(D Vxc)) can be taken from its own points alone, and changing one atom's grid
changes only that atom's share.  For an atom A and a candidate grid level l (a radial shell count
the Lebedev rules of the Fine level's pruning regions and a radial cut-off) the quadrature error is

    err_A(l) = max(|E_A(l) - E_A(Fine)|, |T_A(l) - T_A(Fine)|),
    E_A = sum over A's points of w f,   T_A = sum over A's points of w (v_rho rho + v_gamma |grad rho|^2).

The method generates its own training data: for seeded synthetic molecules (water clusters, alkanes,
benzene) with seeded S-orthonormal densities it evaluates every level and the Fine grid on the GPU
(calchem_xc_grid_build_atoms + calchem_xc_evaluate_rks_points, FP64) and records log10 err_A(l)
against 16 features of the atom's environment.  The network (csrc/mlp.cu) is trained on the GPU with
the library's own forward / backward / Adam kernels.

At use, every atom takes the cheapest level whose predicted error is below log10(tol_atom) - margin,
with tol_atom = tol / n_atoms (so that the per-atom errors, even if they all had one sign, stay
within tol).  The judge (``LearnedGrid.check``) evaluates the per-atom shares on the Fine grid and on
the pruned grid for the current density; every atom whose error exceeds tol_atom reverts to Fine.
"""

import json
import math
import os

import numpy as np

from . import _native
from .grid import MolecularGrid

# Candidate levels, cheapest first: (radial shells, Lebedev points of the five Fine pruning regions
# x = r / R_BS < 0.18, 0.5, 0.95, 5, beyond, radial cut-off x_max).  Zeros mean the Fine choice
# (99 shells; 50 / 110 / 194 / 302 / 194; no cut-off); the last level is the Fine grid itself.
# Measured on water clusters, octane and benzene (FP64, B3LYP / PBE): shells beyond x = 12 change an
# atom's share by < 1e-9 and beyond x = 20 by nothing; the innermost region's 50-point rule can drop
# to 26 at ~1e-10 - 1e-8; hydrogen (no core) also tolerates 50 / 110 points in the next two regions
# (~1e-10 - 1e-9) where heavy atoms do not (~1e-7 - 1e-6); the 302-point valence region, the outer
# region's 194 points and the radial count cannot be reduced at this accuracy.
LEVELS = [
    (0, (26, 50, 110, 0, 0), 8.0),
    (0, (26, 50, 110, 0, 0), 12.0),
    (0, (26, 50, 0, 0, 0), 12.0),
    (0, (26, 0, 0, 0, 0), 12.0),
    (0, (0, 0, 0, 0, 0), 12.0),
    (0, (26, 0, 0, 0, 0), 20.0),
    (0, (0, 0, 0, 0, 0), 20.0),
    (0, (0, 0, 0, 0, 0), 0.0),
]
FINE = len(LEVELS) - 1
N_FEATURES = 16
N_OUTPUTS = 16
MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "pruner_mlp.json")
ERR_FLOOR = 1e-14


# ----------------------------------------------------------------------------------------- features
def atom_features(mol) -> np.ndarray:
    """[n_atoms, 16] environment features: element one-hot (H, C, N, O, other), Z / 10, neighbour
    count within 12 Bohr / 10, the two nearest-neighbour distances, neighbour counts within 2.5 / 4 /
    6 / 9 Bohr, sum of Z_B exp(-r_AB) / 10, sum of exp(-r_AB^2 / 8), mean neighbour Z within
    4 Bohr / 8 (distances in Bohr)."""
    z = np.asarray(mol.z, dtype=np.int64)
    xyz = np.asarray(mol.coords_bohr, dtype=np.float64)
    n = len(z)
    F = np.zeros((n, N_FEATURES))
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    np.fill_diagonal(d, np.inf)
    for a in range(n):
        za = int(z[a])
        F[a, {1: 0, 6: 1, 7: 2, 8: 3}.get(za, 4)] = 1.0
        F[a, 5] = za / 10.0
        F[a, 6] = np.sum(d[a] < 12.0) / 10.0
        r = np.sort(d[a])
        F[a, 7] = r[0] if n > 1 else 20.0
        F[a, 8] = r[1] if n > 2 else 20.0
        F[a, 9] = np.sum(d[a] < 2.5)
        F[a, 10] = np.sum(d[a] < 4.0)
        F[a, 11] = np.sum(d[a] < 6.0)
        F[a, 12] = np.sum(d[a] < 9.0)
        fin = np.isfinite(d[a])
        F[a, 13] = np.sum(z[fin] * np.exp(-d[a][fin])) / 10.0
        F[a, 14] = np.sum(np.exp(-d[a][fin] ** 2 / 8.0))
        near = d[a] < 4.0
        F[a, 15] = (np.mean(z[near]) / 8.0) if np.any(near) else 0.0
    F[:, 7:9] = np.minimum(F[:, 7:9], 20.0)
    return F


# ------------------------------------------------------------------------- per-atom quadrature shares
def _level_arrays(levels_per_atom):
    nr = np.array([LEVELS[l][0] for l in levels_per_atom], dtype=np.int32)
    leb = np.array([LEVELS[l][1] for l in levels_per_atom], dtype=np.int32).reshape(-1, 5)
    xm = np.array([LEVELS[l][2] for l in levels_per_atom], dtype=np.float64)
    return nr, leb, xm


def grid_for_levels(mol, levels_per_atom) -> MolecularGrid:
    return MolecularGrid.build_atoms(mol, *_level_arrays(levels_per_atom))


def atom_shares(mol, basis, grid, func, D, precision="fp64"):
    """(E_A, T_A) per atom of one grid: each atom's share of Exc and of tr(D Vxc)."""
    from .vxc import _upload_points, _xc_code, _PRECISION
    lib = _native.load()
    gid = _upload_points(basis, grid)
    try:
        pts = np.zeros(2 * len(grid))
        exc, ne = np.zeros(1), np.zeros(1)
        P = np.ascontiguousarray(D, dtype=np.float64)
        _native.check("calchem_xc_evaluate_rks_points", lib.calchem_xc_evaluate_rks_points(
            gid, _xc_code(func), _PRECISION[precision], _native.ptr(P), _native.ptr(exc), _native.ptr(ne),
            _native.ptr(pts)))
    finally:
        lib.calchem_cuda_vxc_release(gid)
    n = len(mol.atoms)
    E = np.bincount(grid.host_atom, weights=pts[0::2], minlength=n)
    T = np.bincount(grid.host_atom, weights=pts[1::2], minlength=n)
    return E, T


def level_errors(mol, basis, func, D, levels=None):
    """[n_atoms, n_levels] per-atom errors err_A(l) against the Fine grid (FP64 evaluation)."""
    levels = range(len(LEVELS)) if levels is None else levels
    n = len(mol.atoms)
    fine = grid_for_levels(mol, [FINE] * n)
    E0, T0 = atom_shares(mol, basis, fine, func, D)
    out = np.zeros((n, len(LEVELS)))
    for l in levels:
        if l == FINE:
            continue
        g = grid_for_levels(mol, [l] * n)
        E, T = atom_shares(mol, basis, g, func, D)
        out[:, l] = np.maximum(np.abs(E - E0), np.abs(T - T0))
    return out


# ------------------------------------------------------------------------------ training molecules
def benzene(seed: int):
    from .molecule import Atom, Molecule
    rng = np.random.Generator(np.random.PCG64(seed))
    atoms = []
    for k in range(6):
        ang = k * math.pi / 3
        c = np.array([1.39 * math.cos(ang), 1.39 * math.sin(ang), 0.0])
        atoms.append(("C", c + rng.normal(0, 0.02, 3)))
        atoms.append(("H", c * (1.39 + 1.09) / 1.39 + rng.normal(0, 0.02, 3)))
    return Molecule([Atom.from_angstrom(s, p) for s, p in atoms], 0, 1)


def perturbed(mol, seed: int, sigma_ang: float = 0.03):
    from .molecule import ANGSTROM_TO_BOHR, Atom, Molecule
    rng = np.random.Generator(np.random.PCG64(seed))
    atoms = [Atom(a.symbol, np.asarray(a.position_bohr) + rng.normal(0, sigma_ang * ANGSTROM_TO_BOHR, 3))
             for a in mol.atoms]
    return Molecule(atoms, mol.charge, mol.multiplicity)


def training_set():
    """Seeded synthetic molecules with their basis name, functional and density seed."""
    from . import workloads
    funcs = ["pbe", "b3lyp", "svwn5", "blyp"]
    out = []
    i = 0
    for k in (1, 2, 3, 4, 6, 8, 12, 16):
        for s in (0, 1):
            out.append((workloads.water_cluster(k, 500 + 10 * k + s), "6-31g(d)", funcs[i % 4], 900 + i))
            i += 1
    for nc in range(2, 11):
        for s in (0, 1):
            out.append((perturbed(workloads.alkane(nc), 700 + 10 * nc + s), "6-31g(d,p)", funcs[i % 4], 900 + i))
            i += 1
    for s in range(3):
        out.append((benzene(800 + s), "6-31g(d)", funcs[i % 4], 900 + i))
        i += 1
    return out


def generate_samples(molecules=None, log=None):
    """(X [n, 16], Y [n, n_levels] log10 errors, molecule index per sample) from the GPU."""
    from . import workloads
    from .basis import BasisSet
    molecules = training_set() if molecules is None else molecules
    X, Y, M = [], [], []
    for mi, (mol, bname, func, seed) in enumerate(molecules):
        basis = BasisSet.from_name(bname, mol)
        D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, seed)
        err = level_errors(mol, basis, func, D)
        X.append(atom_features(mol))
        Y.append(np.log10(err + ERR_FLOOR))
        M.extend([mi] * len(mol.atoms))
        if log:
            log(f"  molecule {mi}: {len(mol.atoms)} atoms, {func}, max log10 err per level "
                f"{np.round(Y[-1].max(axis=0), 2).tolist()}")
    return np.vstack(X), np.vstack(Y), np.array(M)


# ----------------------------------------------------------------------------------------- network
class Network:
    """The MLP of csrc/mlp.cu with its normalisation; GPU forward, backward and Adam through the
    library's kernels (device buffers are torch tensors)."""

    def __init__(self, params=None, feature_mean=None, feature_std=None, target_shift=8.0, target_scale=3.0,
                 seed=0):
        lib = _native.load()
        dims = [np.zeros(1, np.int32) for _ in range(5)]
        _native.check("calchem_mlp_shape", lib.calchem_mlp_shape(*[_native.ptr(d) for d in dims]))
        self.n_in, self.n_hid, self.n_out, self.n_params, self.work = (int(d[0]) for d in dims)
        assert self.n_in == N_FEATURES and self.n_out == N_OUTPUTS
        if params is None:
            rng = np.random.Generator(np.random.PCG64(seed))
            parts = []
            for fan_in, fan_out in ((self.n_in, self.n_hid), (self.n_hid, self.n_hid), (self.n_hid, self.n_out)):
                parts.append(rng.normal(0, 1.0 / math.sqrt(fan_in), (fan_in, fan_out)).ravel())
                parts.append(np.zeros(fan_out))
            params = np.concatenate(parts)
        self.params = np.asarray(params, dtype=np.float32)
        assert self.params.size == self.n_params
        self.feature_mean = np.zeros(N_FEATURES) if feature_mean is None else np.asarray(feature_mean, float)
        self.feature_std = np.ones(N_FEATURES) if feature_std is None else np.asarray(feature_std, float)
        self.target_shift = float(target_shift)
        self.target_scale = float(target_scale)

    # normalisation: x' = (x - mean) / std;  y' = (log10 err + shift) / scale
    def norm_x(self, X):
        return ((np.asarray(X, float) - self.feature_mean) / self.feature_std).astype(np.float32)

    def norm_y(self, Y):
        return ((np.asarray(Y, float) + self.target_shift) / self.target_scale).astype(np.float32)

    def denorm_y(self, Yn):
        return np.asarray(Yn, float) * self.target_scale - self.target_shift

    def predict(self, X) -> np.ndarray:
        """log10 error per level, [n, n_levels] (GPU forward kernel)."""
        import torch
        lib = _native.load()
        dev = torch.device("cuda:0")
        x = torch.from_numpy(self.norm_x(X)).to(dev)
        p = torch.from_numpy(self.params).to(dev)
        y = torch.zeros((len(x), self.n_out), dtype=torch.float32, device=dev)
        _native.check("calchem_mlp_forward", lib.calchem_mlp_forward(p.data_ptr(), x.data_ptr(), len(x), y.data_ptr(),
                                                                     torch.cuda.current_stream(dev).cuda_stream))
        torch.cuda.synchronize(dev)
        return self.denorm_y(y.cpu().numpy())[:, :len(LEVELS)]

    def fit(self, X, Y, steps=4000, lr=3e-3, log=None, X_val=None, Y_val=None):
        """Full-batch Adam on the masked MSE, all on the GPU; returns the loss history."""
        import torch
        lib = _native.load()
        dev = torch.device("cuda:0")
        st = torch.cuda.current_stream(dev).cuda_stream
        n = len(X)
        T = np.zeros((n, self.n_out), np.float32)
        Mk = np.zeros((n, self.n_out), np.float32)
        T[:, :len(LEVELS)] = self.norm_y(Y)
        Mk[:, :len(LEVELS)] = 1.0
        Mk[:, FINE] = 0.0  # the Fine level's error is zero by definition
        inv = float(1.0 / Mk.sum())
        x = torch.from_numpy(self.norm_x(X)).to(dev)
        t = torch.from_numpy(T).to(dev)
        mk = torch.from_numpy(Mk).to(dev)
        p = torch.from_numpy(self.params.copy()).to(dev)
        g = torch.zeros_like(p)
        m = torch.zeros_like(p)
        v = torch.zeros_like(p)
        work = torch.zeros(n * self.work, dtype=torch.float32, device=dev)
        lp = torch.zeros(n, dtype=torch.float32, device=dev)
        loss = torch.zeros(1, dtype=torch.float32, device=dev)
        hist = []
        for step in range(1, steps + 1):
            _native.check("calchem_mlp_loss_grad", lib.calchem_mlp_loss_grad(
                p.data_ptr(), x.data_ptr(), t.data_ptr(), mk.data_ptr(), n, inv, work.data_ptr(), lp.data_ptr(),
                g.data_ptr(), loss.data_ptr(), st))
            _native.check("calchem_mlp_adam", lib.calchem_mlp_adam(p.data_ptr(), g.data_ptr(), m.data_ptr(),
                                                                   v.data_ptr(), self.n_params, step, lr, 0.9, 0.999,
                                                                   1e-8, st))
            if step == 1 or step % 200 == 0 or step == steps:
                hist.append((step, float(loss.item())))
                if log:
                    log(f"  step {step}: loss {hist[-1][1]:.5f}")
        torch.cuda.synchronize(dev)
        self.params = p.cpu().numpy()
        return hist

    def to_json(self, **extra) -> dict:
        d = {"levels": LEVELS, "n_features": N_FEATURES, "feature_mean": self.feature_mean.tolist(),
             "feature_std": self.feature_std.tolist(), "target_shift": self.target_shift,
             "target_scale": self.target_scale, "params": [float(v) for v in self.params]}
        d.update(extra)
        return d

    @classmethod
    def from_json(cls, d):
        if [(l[0], tuple(l[1]), l[2]) for l in d["levels"]] != LEVELS:
            raise ValueError("model was trained for other grid levels")
        return cls(np.array(d["params"], np.float32), d["feature_mean"], d["feature_std"], d["target_shift"],
                   d["target_scale"])

    @classmethod
    def load(cls, path=MODEL_PATH):
        with open(path) as f:
            return cls.from_json(json.load(f))


def train(samples=None, steps=4000, lr=3e-3, log=None, seed=0):
    """Trains a network on (X, Y, molecule ids); molecules with id % 5 == 4 are held out."""
    X, Y, mol_id = generate_samples(log=log) if samples is None else samples
    val = (mol_id % 5) == 4
    mean = X[~val].mean(axis=0)
    std = X[~val].std(axis=0)
    std[std < 1e-6] = 1.0
    net = Network(feature_mean=mean, feature_std=std, seed=seed)
    hist = net.fit(X[~val], Y[~val], steps=steps, lr=lr, log=log)
    rmse = lambda A, B: float(np.sqrt(np.mean((A[:, :FINE] - B[:, :FINE]) ** 2)))
    stats = {"train_atoms": int((~val).sum()), "val_atoms": int(val.sum()),
             "train_rmse_log10": rmse(net.predict(X[~val]), Y[~val]),
             "val_rmse_log10": rmse(net.predict(X[val]), Y[val]) if val.any() else None,
             "loss_history": hist}
    return net, stats


# ------------------------------------------------------------------------------ choice and judge
def choose_levels(net, mol, tol_atom, margin=0.5) -> np.ndarray:
    """Cheapest level per atom whose predicted log10 error is below log10(tol_atom) - margin."""
    pred = net.predict(atom_features(mol))
    lim = math.log10(tol_atom) - margin
    out = np.full(len(mol.atoms), FINE, dtype=np.int64)
    for a in range(len(mol.atoms)):
        ok = np.nonzero(pred[a, :FINE] <= lim)[0]
        if len(ok):
            out[a] = int(ok[0])
    return out


class ShareEngine:
    """A resident upload of a set of grid points with their host atoms, evaluated for per-atom shares
    of Exc and tr(D Vxc) without the Vxc contraction (calchem_xc_set_point_atoms,
    calchem_xc_evaluate_rks_atoms[_device]).  The points stay on the device, with the tensor-core
    form's AO cache, across evaluations."""

    def __init__(self, basis, grid, n_atoms, ao_floor=None):
        from .vxc import _upload_points
        lib = _native.load()
        self.n_atoms = int(n_atoms)
        self.n_points = len(grid)
        self.grid_id = _upload_points(basis, grid, ao_floor=ao_floor)
        host = np.ascontiguousarray(grid.host_atom, dtype=np.int32)
        _native.check("calchem_xc_set_point_atoms",
                      lib.calchem_xc_set_point_atoms(self.grid_id, _native.ptr(host), len(host), self.n_atoms))

    def shares(self, D, func, precision="mixed"):
        """(E_A, T_A) per atom from a host density."""
        from .vxc import _xc_code, _PRECISION
        lib = _native.load()
        P = np.ascontiguousarray(D, dtype=np.float64)
        out = np.zeros(2 * self.n_atoms)
        exc, ne = np.zeros(1), np.zeros(1)
        _native.check("calchem_xc_evaluate_rks_atoms", lib.calchem_xc_evaluate_rks_atoms(
            self.grid_id, _xc_code(func), _PRECISION[precision], _native.ptr(P), _native.ptr(exc), _native.ptr(ne),
            _native.ptr(out), None))
        return out[0::2].copy(), out[1::2].copy()

    def enqueue(self, d_total, d_result, d_atom_out, stream, func, precision="mixed"):
        """Device-buffer form (addresses; d_atom_out holds 2 n_atoms doubles), enqueued on stream."""
        from .vxc import _xc_code, _PRECISION
        return _native.load().calchem_xc_evaluate_rks_atoms_device(
            self.grid_id, _xc_code(func), _PRECISION[precision], d_total, d_result, None, d_atom_out, stream)

    def set_profiling(self, enable=True):
        _native.check("calchem_xc_set_profiling", _native.load().calchem_xc_set_profiling(self.grid_id, int(enable)))

    def set_tile(self, tile_n):
        """The tensor-core GEMM1 tile (64 or 128, calchem_xc_set_tile); results do not depend on it."""
        _native.check("calchem_xc_set_tile", _native.load().calchem_xc_set_tile(self.grid_id, int(tile_n)))

    def ao_cache_bytes(self) -> int:
        import ctypes
        out = (ctypes.c_size_t * 1)()
        _native.check("calchem_xc_set_ao_cache", _native.load().calchem_xc_set_ao_cache(self.grid_id, -1, out))
        return int(out[0])

    def last_kernel_ms(self):
        import ctypes
        ms = (ctypes.c_float * 1)()
        _native.check("calchem_xc_last_kernel_ms", _native.load().calchem_xc_last_kernel_ms(self.grid_id, ms))
        return float(ms[0])

    def close(self):
        if self.grid_id:
            _native.load().calchem_cuda_vxc_release(self.grid_id)
            self.grid_id = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _subgrid(grid, keep):
    return MolecularGrid(grid.xyzw[keep], grid.raw_weight[keep], grid.host_atom[keep], grid.level)


class LearnedGrid:
    """A molecule's MLP-pruned grid with the Fine grid as fallback and judge.

    ``tol`` bounds the total (per molecule) Exc and tr(D Vxc) quadrature error against the Fine grid;
    every atom is held to tol / n_atoms.  ``check(D, func)`` is the periodic full-grid check: it
    compares every atom's shares on the pruned and Fine grids for the density D and reverts the
    atoms that exceed their tolerance to Fine (rebuilding the grid).

    Becke partitioning makes an atom's share depend on its own points only, and an atom kept at the
    Fine level has the same points on both grids, so the judge evaluates just the pruned atoms'
    points: their Fine points and their pruned points, two resident uploads (``judge_engines``) kept
    with their AO caches between checks and rebuilt only when an atom reverts.  The pruned grid's
    shares can come from the iteration's own build instead (``pruned_shares``, from
    ``RksVxcEngine.evaluate_with_shares``), which leaves only the Fine points to evaluate.  The shares
    need no Vxc contraction, and the check runs in the tensor-core form by default (the difference
    it judges is within ~2e-10 Eh of the FP64 form's on water clusters and octane, against per-atom
    tolerances of ~3e-9 and above)."""

    def __init__(self, mol, basis, net=None, tol=5e-7, margin=0.5, ao_floor="auto"):
        """ao_floor: the value screen of the judge's uploads ("auto": the tensor-core engines' floor,
        so that the judge's shares and a tensor-core build's shares come from the same plan rule)."""
        from .vxc import MIXED_AO_FLOOR
        self.mol = mol
        self.basis = basis
        self.ao_floor = MIXED_AO_FLOOR if ao_floor == "auto" else ao_floor
        self.net = Network.load() if net is None else net
        self.tol_atom = tol / len(mol.atoms)
        self.levels = choose_levels(self.net, mol, self.tol_atom, margin)
        self.grid = grid_for_levels(mol, self.levels)
        self._fine = None
        self._judge = None
        self.reverted = []

    @property
    def fine_grid(self):
        if self._fine is None:
            self._fine = grid_for_levels(self.mol, [FINE] * len(self.mol.atoms))
        return self._fine

    def pruned_atoms(self):
        return np.nonzero(self.levels != FINE)[0]

    def fine_judge(self):
        """The Fine-grid points of the pruned atoms as a resident ShareEngine; None when no atom is
        pruned."""
        atoms = self.pruned_atoms()
        if len(atoms) == 0:
            return None
        if self._judge is None:
            self._judge = [None, None]
        if self._judge[0] is None:
            fine = _subgrid(self.fine_grid, np.isin(self.fine_grid.host_atom, atoms))
            self._judge[0] = ShareEngine(self.basis, fine, len(self.mol.atoms), self.ao_floor)
        return self._judge[0]

    def judge_engines(self):
        """(Fine-grid points of the pruned atoms, pruned-grid points of the same atoms) as resident
        ShareEngines; None when no atom is pruned."""
        if self.fine_judge() is None:
            return None
        if self._judge[1] is None:
            pruned = _subgrid(self.grid, np.isin(self.grid.host_atom, self.pruned_atoms()))
            self._judge[1] = ShareEngine(self.basis, pruned, len(self.mol.atoms), self.ao_floor)
        return tuple(self._judge)

    def judge_points(self, with_pruned=True):
        """Points the judge evaluates (the Fine upload, and the pruned one unless the build supplies
        the pruned shares)."""
        j = self.fine_judge()
        if j is None:
            return 0
        return j.n_points + (self.judge_engines()[1].n_points if with_pruned else 0)

    def _close_judge(self):
        if self._judge is not None:
            for e in self._judge:
                if e is not None:
                    e.close()
            self._judge = None

    def check(self, D, func, precision="mixed", pruned_shares=None):
        """Full-grid check; returns (atoms reverted to Fine, per-atom errors).  pruned_shares: the
        pruned grid's per-atom (E_A, T_A) from the iteration's own build (all atoms; only the pruned
        ones are read), in place of evaluating them here.  The grid and the judge uploads are rebuilt
        if any atom reverts."""
        n = len(self.mol.atoms)
        judge = self.fine_judge()
        if judge is None:
            return [], np.zeros(n)
        E0, T0 = judge.shares(D, func, precision)
        if pruned_shares is None:
            E, T = self.judge_engines()[1].shares(D, func, precision)
        else:
            E, T = (np.asarray(x, dtype=np.float64) for x in pruned_shares)
        err = np.maximum(np.abs(E - E0), np.abs(T - T0))
        bad = [int(a) for a in np.nonzero((err > self.tol_atom) & (self.levels != FINE))[0]]
        if bad:
            self.levels[bad] = FINE
            self.grid = grid_for_levels(self.mol, self.levels)
            self.reverted.extend(bad)
            self._close_judge()
        return bad, err

    def close(self):
        self._close_judge()
