"""Cartesian Gaussian basis sets (mirrors crates/calchem-basis/src/lib.rs).

The basis data (MolSSI-BSE-derived, H..Ar) live in ``data/basis/*.json``.  Shell
normalisation and the GPU-layout arrays (AoShellGpu / AoPrimGpu / AoCompGpu,
crates/calchem-cuda/src/lib.rs:46-84) are produced by the native library
(``calchem_xc_prepare_shells``), as the reference engine does before uploading
(crates/calchem-dft/src/vxc.rs:497-545).
"""

import json
import os

import numpy as np

from . import _native
from .molecule import Molecule

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis")
_FILES = {"sto-3g": "sto-3g.json", "6-31g": "6-31g.json", "6-31g(d)": "6-31gd.json", "6-31g(d,p)": "6-31gdp.json"}
_L = {"s": 0, "p": 1, "d": 2, "f": 3}
_CACHE = {}


def canonical_name(name: str):
    """BasisSet::canonical_name (calchem-basis/src/lib.rs:268-278), for the sets shipped here."""
    n = name.strip().lower()
    if n in ("sto-3g", "sto3g"):
        return "sto-3g"
    if n in ("6-31g", "631g"):
        return "6-31g"
    if n in ("6-31g(d)", "6-31g*", "631gd", "631g*", "6-31gd"):
        return "6-31g(d)"
    if n in ("6-31g(d,p)", "6-31g**", "631gdp", "631g**", "6-31gdp"):
        return "6-31g(d,p)"
    return None


def _load(canon: str):
    if canon not in _CACHE:
        with open(os.path.join(_DATA, _FILES[canon])) as f:
            _CACHE[canon] = json.load(f)
    return _CACHE[canon]


class Shell:
    __slots__ = ("atom_index", "center", "l", "exponents", "raw_coefs", "ao_offset")

    def __init__(self, atom_index, center, l, exponents, raw_coefs, ao_offset):
        self.atom_index = atom_index
        self.center = np.asarray(center, dtype=np.float64)
        self.l = l
        self.exponents = np.asarray(exponents, dtype=np.float64)
        self.raw_coefs = np.asarray(raw_coefs, dtype=np.float64)
        self.ao_offset = ao_offset

    @property
    def n_functions(self) -> int:
        return (self.l + 1) * (self.l + 2) // 2


class BasisSet:
    """Shells in atom-major order; AO offsets follow shell order (lib.rs:462-518)."""

    def __init__(self, name: str, shells):
        self.name = name
        self.shells = list(shells)
        self.n_ao = sum(s.n_functions for s in self.shells)
        self._gpu = None

    @classmethod
    def from_name(cls, name: str, mol: Molecule) -> "BasisSet":
        canon = canonical_name(name)
        if canon is None:
            raise ValueError(f"unsupported basis set: {name!r}")
        data = _load(canon)["elements"]
        shells = []
        ao = 0
        for ia, atom in enumerate(mol.atoms):
            if atom.symbol not in data:
                raise ValueError(f"element {atom.symbol} not in basis {canon}")
            for st, exps, coefs in data[atom.symbol]:
                sh = Shell(ia, atom.position_bohr, _L[st], exps, coefs, ao)
                shells.append(sh)
                ao += sh.n_functions
        return cls(canon, shells)

    def min_exponent(self) -> float:
        return float(min(np.min(s.exponents) for s in self.shells))

    def gpu_arrays(self):
        """(shells, prims, comps) structured arrays in the reference GPU layout."""
        if self._gpu is None:
            lib = _native.load()
            ns = len(self.shells)
            ls = np.array([s.l for s in self.shells], dtype=np.int32)
            atoms = np.array([s.atom_index for s in self.shells], dtype=np.int32)
            centers = np.ascontiguousarray(np.array([s.center for s in self.shells], dtype=np.float64))
            nprim = np.array([len(s.exponents) for s in self.shells], dtype=np.int32)
            exps = np.ascontiguousarray(np.concatenate([s.exponents for s in self.shells]))
            coefs = np.ascontiguousarray(np.concatenate([s.raw_coefs for s in self.shells]))
            sh = np.zeros(ns, dtype=_native.AO_SHELL)
            pr = np.zeros(int(nprim.sum()), dtype=_native.AO_PRIM)
            co = np.zeros(self.n_ao, dtype=_native.AO_COMP)
            n_ao = np.zeros(1, dtype=np.int32)
            _native.check("calchem_xc_prepare_shells", lib.calchem_xc_prepare_shells(
                ns, _native.ptr(ls), _native.ptr(atoms), _native.ptr(centers), _native.ptr(nprim),
                _native.ptr(exps), _native.ptr(coefs), _native.ptr(sh), _native.ptr(pr), _native.ptr(co),
                _native.ptr(n_ao)))
            assert int(n_ao[0]) == self.n_ao
            self._gpu = (sh, pr, co)
        return self._gpu

    def overlap(self) -> np.ndarray:
        """Overlap matrix S (compute_overlap, calchem-int/src/one_electron.rs:115-128)."""
        lib = _native.load()
        sh, pr, co = self.gpu_arrays()
        S = np.zeros((self.n_ao, self.n_ao), dtype=np.float64)
        _native.check("calchem_xc_overlap", lib.calchem_xc_overlap(
            _native.ptr(sh), len(sh), _native.ptr(pr), _native.ptr(co), self.n_ao, _native.ptr(S)))
        return S
