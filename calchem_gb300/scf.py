"""SCF harness around the GPU XC quadrature: restricted and unrestricted Kohn-Sham (and Hartree-Fock
when no functional is given), mirroring the entry points of calchem-scf (``rks`` / ``uks``,
crates/calchem-scf/src/rks.rs:255-300, uks.rs).

Integrals come from the library's host code (McMurchie-Davidson, ``calchem_scf_one_electron`` /
``calchem_scf_eri``) over the same shells the quadrature uses; J and K are contracted from the dense
ERI tensor (small molecules).  Every iteration calls the GPU Vxc engine once.  Convergence is
accelerated by DIIS on the orbital gradient F D S - S D F (Pulay).  With ``learned=True`` the grid
is the MLP-pruned grid, checked against the Fine grid every ``judge_every`` iterations on the current
density (atoms over tolerance revert to Fine, and the engine is rebuilt).
"""

from dataclasses import dataclass, field

import numpy as np

from . import _native
from .grid import GridLevel, MolecularGrid
from .vxc import RksVxcEngine, UksVxcEngine
from .xc import XcFunctional

_EXACT_EXCHANGE = {XcFunctional.B3LYP: 0.20, XcFunctional.B3LYP5: 0.20, XcFunctional.PBE0: 0.25}


def exact_exchange_fraction(func) -> float:
    """exact_exchange_fraction (xc.rs:116-125); Hartree-Fock (func None) is 1."""
    if func is None:
        return 1.0
    f = XcFunctional.from_name(func) if isinstance(func, str) else XcFunctional(func)
    if f.is_range_separated():
        raise NotImplementedError("range-separated exact exchange (erf-attenuated K) is not in this SCF harness; "
                                  "their semilocal XC part is evaluated by the engines")
    return _EXACT_EXCHANGE.get(f, 0.0)


def nuclear_repulsion(mol) -> float:
    z = np.asarray(mol.z, float)
    x = np.asarray(mol.coords_bohr)
    e = 0.0
    for i in range(len(z)):
        for j in range(i):
            e += z[i] * z[j] / np.linalg.norm(x[i] - x[j])
    return float(e)


def core_matrices(basis, mol):
    """(S, T, V) over the basis (calchem_scf_one_electron)."""
    lib = _native.load()
    sh, pr, co = basis.gpu_arrays()
    n = basis.n_ao
    S, T, V = (np.zeros((n, n)) for _ in range(3))
    z = np.ascontiguousarray(mol.z, dtype=np.float64)
    xyz = np.ascontiguousarray(mol.coords_bohr)
    _native.check("calchem_scf_one_electron", lib.calchem_scf_one_electron(
        _native.ptr(sh), len(sh), _native.ptr(pr), _native.ptr(co), n, len(z), _native.ptr(z), _native.ptr(xyz),
        _native.ptr(S), _native.ptr(T), _native.ptr(V)))
    return S, T, V


def eri_tensor(basis) -> np.ndarray:
    """Dense (pq|rs) tensor (calchem_scf_eri)."""
    lib = _native.load()
    sh, pr, co = basis.gpu_arrays()
    n = basis.n_ao
    eri = np.zeros((n, n, n, n))
    _native.check("calchem_scf_eri", lib.calchem_scf_eri(_native.ptr(sh), len(sh), _native.ptr(pr), _native.ptr(co),
                                                         n, _native.ptr(eri)))
    return eri


class _JK:
    """Coulomb and exchange matrices J_pq = sum_rs (pq|rs) D_rs and K_pq = sum_rs (pr|qs) D_rs from the
    dense ERI tensor: numpy contractions, or (device given) two matrix-vector products on the GPU with
    the tensor resident in device memory (large bases, where the host contractions would dominate)."""

    def __init__(self, eri, device=None):
        self.n = eri.shape[0]
        self.eri = eri
        self.dev = device
        if device is not None:
            import torch
            t = torch.from_numpy(eri).to(device)
            n2 = self.n * self.n
            self.Jm = t.view(n2, n2)
            self.Km = t.permute(0, 2, 1, 3).reshape(n2, n2)  # (pq|rs) -> [(p,q), (r,s)] of (pr|qs)

    def _apply(self, M, D, spec):
        if self.dev is None:
            return np.einsum(spec, self.eri, D, optimize=True)
        import torch
        d = torch.from_numpy(np.ascontiguousarray(D, dtype=np.float64).ravel()).to(self.dev)
        return (M @ d).view(self.n, self.n).cpu().numpy()

    def J(self, D):
        return self._apply(getattr(self, "Jm", None), D, "pqrs,rs->pq")

    def K(self, D):
        return self._apply(getattr(self, "Km", None), D, "prqs,rs->pq")


def integrals(mol, basis):
    """The SCF's integrals once per geometry: {"S", "T", "V", "eri"} (pass to rks / uks as ints)."""
    S, T, V = core_matrices(basis, mol)
    return {"S": S, "T": T, "V": V, "eri": eri_tensor(basis)}


def _jk_device(eri, jk):
    if jk == "host":
        return None
    if jk not in ("auto", "gpu"):
        raise ValueError("jk must be 'auto', 'host' or 'gpu'")
    try:
        import torch
        ok = torch.cuda.is_available()
    except ImportError:
        ok = False
    if jk == "gpu" and not ok:
        raise RuntimeError("jk='gpu' needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device()) if ok and (jk == "gpu" or eri.nbytes > (1 << 30)) else None


class _Diis:
    def __init__(self, size=8):
        self.size = size
        self.F, self.E = [], []

    def push(self, F, err):
        self.F.append(F)
        self.E.append(err)
        if len(self.F) > self.size:
            self.F.pop(0)
            self.E.pop(0)

    def extrapolate(self):
        k = len(self.F)
        if k < 2:
            return self.F[-1]
        B = -np.ones((k + 1, k + 1))
        B[k, k] = 0.0
        for i in range(k):
            for j in range(k):
                B[i, j] = sum(np.vdot(a, b) for a, b in zip(self.E[i], self.E[j]))
        rhs = np.zeros(k + 1)
        rhs[k] = -1.0
        try:
            c = np.linalg.solve(B, rhs)[:k]
        except np.linalg.LinAlgError:
            return self.F[-1]
        return tuple(sum(ci * Fi[s] for ci, Fi in zip(c, self.F)) for s in range(len(self.F[-1])))


@dataclass
class ScfResult:
    total_energy_hartree: float
    converged: bool
    iterations: int
    mo_energies: np.ndarray
    densities: tuple
    exc: float = 0.0
    nuclear_repulsion: float = 0.0
    s_squared: float = 0.0          # <S^2> - S(S+1) (UKS spin contamination)
    grid_points: int = 0
    energies: list = field(default_factory=list)
    reverted_atoms: list = field(default_factory=list)
    first_exc: float = 0.0            # Exc of the first iteration (at the core-Hamiltonian guess density)
    first_density: np.ndarray = None  # total density of the first iteration


def _orthogonaliser(S):
    w, U = np.linalg.eigh(S)
    keep = w > 1e-8
    return U[:, keep] / np.sqrt(w[keep])


def _diag(F, X):
    e, C = np.linalg.eigh(X.T @ F @ X)
    return e, X @ C


def _grid_and_engine(mol, basis, func, level, precision, learned, tol, spin):
    if func is None:
        return None, None, None
    if learned:
        from . import pruner
        from .vxc import default_ao_floor
        lg = pruner.LearnedGrid(mol, basis, tol=tol, ao_floor=default_ao_floor(precision))
        grid = lg.grid
    else:
        lg = None
        grid = MolecularGrid.build_for_basis(mol, basis, level)
    return lg, grid, _engine(mol, basis, grid, precision, spin, learned)


def _engine(mol, basis, grid, precision, spin, learned):
    if spin == "uks":
        return UksVxcEngine(basis, grid, precision=precision)
    eng = RksVxcEngine(basis, grid, precision=precision)
    if learned:  # the judge takes the pruned grid's per-atom shares from the build
        eng.set_point_atoms(grid.host_atom, len(mol.atoms))
    return eng


def _run(mol, basis, func, level, precision, learned, tol, judge_every, max_iter, e_tol, g_tol, spin, ints=None,
         jk="auto"):
    ints = integrals(mol, basis) if ints is None else ints
    S, T, Vn, eri = ints["S"], ints["T"], ints["V"], ints["eri"]
    H = T + Vn
    jk_op = _JK(eri, _jk_device(eri, jk))
    X = _orthogonaliser(S)
    ax = exact_exchange_fraction(func)
    e_nuc = nuclear_repulsion(mol)
    n_a, n_b = mol.n_alpha_beta()
    lg, grid, eng = _grid_and_engine(mol, basis, func, level, precision, learned, tol, spin)
    diis = _Diis()
    e_orb, C = _diag(H, X)
    Ca = Cb = C
    Da = Ca[:, :n_a] @ Ca[:, :n_a].T
    Db = Cb[:, :n_b] @ Cb[:, :n_b].T
    energies, reverted = [], []
    e_old = None
    converged = False
    exc = 0.0
    it = 0
    for it in range(1, max_iter + 1):
        judge_now = lg is not None and judge_every and it % judge_every == 0
        if judge_now and spin == "uks":
            bad, _ = lg.check(Da + Db, func, precision=precision)
            if bad:
                reverted.extend(bad)
                eng.close()
                grid = lg.grid
                eng = _engine(mol, basis, grid, precision, spin, True)
        Dt = Da + Db
        J = jk_op.J(Dt)
        Ka = jk_op.K(Da) if ax != 0.0 else np.zeros_like(Dt)
        Kb = Ka if spin == "rks" else (jk_op.K(Db) if ax != 0.0 else Ka)
        if func is None:
            exc, Va, Vb = 0.0, 0.0, 0.0
        elif spin == "rks":
            if judge_now:
                # the periodic full-grid check, with the pruned grid's shares from this build
                exc, Va, E, T = eng.evaluate_with_shares(basis, grid, func, Dt)
                bad, _ = lg.check(Dt, func, precision=precision, pruned_shares=(E, T))
                if bad:
                    reverted.extend(bad)
                    eng.close()
                    grid = lg.grid
                    eng = _engine(mol, basis, grid, precision, spin, True)
                    exc, Va = eng.evaluate(basis, grid, func, Dt)
            else:
                exc, Va = eng.evaluate(basis, grid, func, Dt)
            Vb = Va
        else:
            exc, Va, Vb = eng.evaluate(basis, grid, func, Da, Db)
        Fa = H + J - ax * Ka + Va
        Fb = H + J - ax * Kb + Vb
        e = (np.sum(Dt * H) + 0.5 * np.sum(Dt * J) - 0.5 * ax * (np.sum(Da * Ka) + np.sum(Db * Kb)) + exc + e_nuc)
        energies.append(float(e))
        if it == 1:
            first = (float(exc), Dt.copy())
        errs = (X.T @ (Fa @ Da @ S - S @ Da @ Fa) @ X, X.T @ (Fb @ Db @ S - S @ Db @ Fb) @ X)
        g = max(float(np.max(np.abs(errs[0]))), float(np.max(np.abs(errs[1]))))
        if e_old is not None and abs(e - e_old) < e_tol and g < g_tol:
            converged = True
            break
        e_old = e
        diis.push((Fa, Fb), errs)
        Fa_x, Fb_x = diis.extrapolate()
        ea, Ca = _diag(Fa_x, X)
        if spin == "rks":
            eb, Cb = ea, Ca
        else:
            eb, Cb = _diag(Fb_x, X)
        Da = Ca[:, :n_a] @ Ca[:, :n_a].T
        Db = Cb[:, :n_b] @ Cb[:, :n_b].T
        e_orb = ea
    s2 = 0.0
    if spin == "uks":
        ov = Ca[:, :n_a].T @ S @ Cb[:, :n_b]
        sz = 0.5 * (n_a - n_b)
        s2 = float(sz * (sz + 1) + n_b - np.sum(ov * ov) - sz * (sz + 1))
    if eng is not None:
        eng.close()
    if lg is not None:
        lg.close()
    dens = (Da + Db,) if spin == "rks" else (Da, Db)
    return ScfResult(energies[-1], converged, it, e_orb, dens, float(exc), e_nuc, s2,
                     0 if grid is None else len(grid), energies, reverted, first_exc=first[0], first_density=first[1])


def rks(mol, basis, func="b3lyp", level=GridLevel.FINE, precision="fp64", learned=False, tol=5e-7, judge_every=5,
        max_iter=128, e_tol=1e-10, g_tol=1e-7, ints=None, jk="auto"):
    """Restricted Kohn-Sham (restricted Hartree-Fock for func=None) to tight convergence.  ints: the
    integrals() of this geometry, to share them between runs; jk: "auto" (J and K on the GPU for dense
    ERI tensors over 1 GiB), "host" or "gpu"."""
    return _run(mol, basis, func, level, precision, learned, tol, judge_every, max_iter, e_tol, g_tol, "rks",
                ints, jk)


def uks(mol, basis, func="b3lyp", level=GridLevel.FINE, precision="fp64", learned=False, tol=5e-7, judge_every=5,
        max_iter=128, e_tol=1e-10, g_tol=1e-7, ints=None, jk="auto"):
    """Unrestricted Kohn-Sham (unrestricted Hartree-Fock for func=None)."""
    return _run(mol, basis, func, level, precision, learned, tol, judge_every, max_iter, e_tol, g_tol, "uks",
                ints, jk)


def rhf(mol, basis, **kw):
    return rks(mol, basis, None, **kw)
