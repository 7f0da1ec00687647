"""Atoms and molecules (mirrors crates/calchem-model/src/lib.rs:4, 32-126)."""

import numpy as np

ANGSTROM_TO_BOHR = 1.8897261245650618  # calchem-model/src/lib.rs:4
BOHR_TO_ANGSTROM = 1.0 / ANGSTROM_TO_BOHR

PERIODIC_TABLE = [
    "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl",
    "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As",
    "Se", "Br", "Kr", "Rb", "Sr", "Y", "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In",
    "Sn", "Sb", "Te", "I", "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb",
    "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W", "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl",
    "Pb", "Bi", "Po", "At", "Rn",
]


def atomic_number(symbol: str) -> int:
    s = symbol.strip()
    if not s:
        raise ValueError("empty element symbol")
    norm = s[0].upper() + s[1:].lower()
    if norm not in PERIODIC_TABLE:
        raise ValueError(f"unsupported element symbol: {symbol}")
    return PERIODIC_TABLE.index(norm) + 1


class Atom:
    __slots__ = ("symbol", "z", "position_bohr")

    def __init__(self, symbol: str, position_bohr):
        self.symbol = symbol.strip()
        self.z = atomic_number(symbol)
        p = np.asarray(position_bohr, dtype=np.float64).reshape(3)
        if not np.all(np.isfinite(p)):
            raise ValueError(f"atom {symbol} has non-finite coordinates")
        self.position_bohr = p

    @classmethod
    def from_angstrom(cls, symbol: str, pos):
        p = np.asarray(pos, dtype=np.float64)
        return cls(symbol, [p[0] * ANGSTROM_TO_BOHR, p[1] * ANGSTROM_TO_BOHR, p[2] * ANGSTROM_TO_BOHR])

    @classmethod
    def from_bohr(cls, symbol: str, pos):
        return cls(symbol, pos)


class Molecule:
    def __init__(self, atoms, charge: int = 0, multiplicity: int = 1):
        self.atoms = list(atoms)
        self.charge = int(charge)
        self.multiplicity = int(multiplicity)

    @property
    def z(self) -> np.ndarray:
        return np.array([a.z for a in self.atoms], dtype=np.int32)

    @property
    def coords_bohr(self) -> np.ndarray:
        return np.array([a.position_bohr for a in self.atoms], dtype=np.float64).reshape(-1, 3)

    def nelectron(self) -> int:
        ne = int(sum(a.z for a in self.atoms)) - self.charge
        if ne <= 0:
            raise ValueError("non-positive electron count")
        return ne

    def n_alpha_beta(self):
        ne = self.nelectron()
        unpaired = self.multiplicity - 1
        if unpaired > ne or (ne - unpaired) % 2:
            raise ValueError("incompatible electron count and multiplicity")
        nb = (ne - unpaired) // 2
        return nb + unpaired, nb

    def __len__(self):
        return len(self.atoms)
