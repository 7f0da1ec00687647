"""Molecular integration grids (mirrors crates/calchem-dft/src/grid.rs).

``MolecularGrid.build`` / ``build_for_basis`` run on the GPU: the native library
expands the Euler-Maclaurin radial shells and pruned Lebedev rules of every atom
and evaluates the screened Becke partition weights in FP64 on the device
(``calchem_xc_grid_build``).  Point order, pruning and the w > 1e-18 cut follow
grid.rs:732-828.
"""

import enum
import itertools
import math

import numpy as np

from . import _native
from .molecule import Molecule


class GridLevel(enum.IntEnum):
    COARSE = 0
    MEDIUM = 1
    FINE = 2
    ULTRAFINE = 3

    @classmethod
    def from_name(cls, name: str) -> "GridLevel":
        """GridLevel::from_name (grid.rs:22-31)."""
        n = name.strip().lower()
        if n in ("coarse", "small", "1"):
            return cls.COARSE
        if n in ("fine", "3"):
            return cls.FINE
        if n in ("ultrafine", "ultra_fine", "4"):
            return cls.ULTRAFINE
        return cls.MEDIUM


_handles = itertools.count(1)


class MolecularGrid:
    """Grid points (x, y, z, w) in Bohr, with raw (pre-Becke) weights and host atoms."""

    def __init__(self, xyzw: np.ndarray, raw_weight: np.ndarray, host_atom: np.ndarray, level: GridLevel):
        self.xyzw = np.ascontiguousarray(xyzw, dtype=np.float64).reshape(-1, 4)
        self.raw_weight = np.asarray(raw_weight, dtype=np.float64)
        self.host_atom = np.asarray(host_atom, dtype=np.int32)
        self.level = GridLevel(level)

    def __len__(self):
        return self.xyzw.shape[0]

    @property
    def coords(self) -> np.ndarray:
        return self.xyzw[:, :3]

    @property
    def weights(self) -> np.ndarray:
        return self.xyzw[:, 3]

    @staticmethod
    def radial_min_for_basis(basis) -> int:
        """Extra radial shells for diffuse exponents (grid.rs:650-663)."""
        alpha = basis.min_exponent()
        extra = math.ceil(180.0 * (1e-4 / max(alpha, 1e-12)) ** 0.25) if alpha < 1e-3 else 0
        return min(extra, 4096)

    @classmethod
    def build(cls, mol: Molecule, level: GridLevel, radial_min: int = 0) -> "MolecularGrid":
        lib = _native.load()
        z = np.ascontiguousarray(mol.z, dtype=np.int32)
        xyz = np.ascontiguousarray(mol.coords_bohr)
        h = next(_handles)
        n = np.zeros(1, dtype=np.int32)
        _native.check("calchem_xc_grid_build",
                      lib.calchem_xc_grid_build(len(z), _native.ptr(z), _native.ptr(xyz), int(level), int(radial_min),
                                                h, _native.ptr(n)))
        try:
            npts = int(n[0])
            xyzw = np.zeros((npts, 4), dtype=np.float64)
            raw = np.zeros(npts, dtype=np.float64)
            host = np.zeros(npts, dtype=np.int32)
            if npts:
                _native.check("calchem_xc_grid_fetch",
                              lib.calchem_xc_grid_fetch(h, _native.ptr(xyzw), _native.ptr(raw), _native.ptr(host)))
        finally:
            lib.calchem_xc_grid_release(h)
        return cls(xyzw, raw, host, level)

    @classmethod
    def build_atoms(cls, mol: Molecule, n_rad, region_leb, x_max) -> "MolecularGrid":
        """Per-atom grid (calchem_xc_grid_build_atoms): atom a gets n_rad[a] radial shells,
        region_leb[a][k] Lebedev points in the Fine pruning region k and no shells beyond
        x = r / R_BS > x_max[a] (zeros: the Fine choices)."""
        lib = _native.load()
        z = np.ascontiguousarray(mol.z, dtype=np.int32)
        xyz = np.ascontiguousarray(mol.coords_bohr)
        nr = np.ascontiguousarray(n_rad, dtype=np.int32)
        leb = np.ascontiguousarray(region_leb, dtype=np.int32).reshape(-1, 5)
        xm = np.ascontiguousarray(x_max, dtype=np.float64)
        if nr.shape != z.shape or leb.shape[0] != len(z) or xm.shape != z.shape:
            raise ValueError("one radial count, five region rules and one cut-off per atom")
        h = next(_handles)
        n = np.zeros(1, dtype=np.int32)
        _native.check("calchem_xc_grid_build_atoms",
                      lib.calchem_xc_grid_build_atoms(len(z), _native.ptr(z), _native.ptr(xyz), _native.ptr(nr),
                                                      _native.ptr(leb), _native.ptr(xm), h, _native.ptr(n)))
        try:
            npts = int(n[0])
            xyzw = np.zeros((npts, 4), dtype=np.float64)
            raw = np.zeros(npts, dtype=np.float64)
            host = np.zeros(npts, dtype=np.int32)
            if npts:
                _native.check("calchem_xc_grid_fetch",
                              lib.calchem_xc_grid_fetch(h, _native.ptr(xyzw), _native.ptr(raw), _native.ptr(host)))
        finally:
            lib.calchem_xc_grid_release(h)
        return cls(xyzw, raw, host, GridLevel.FINE)

    @classmethod
    def build_for_basis(cls, mol: Molecule, basis, level: GridLevel) -> "MolecularGrid":
        """MolecularGrid::build_for_basis (grid.rs:623-634), materialised."""
        return cls.build(mol, level, cls.radial_min_for_basis(basis))
