"""XC functional selection (mirrors crates/calchem-dft/src/xc.rs:16-134).

Codes follow the reference enum order and the ``CALCHEM_XC_*`` constants of
include/calchem_xc.h.
"""

import enum


class XcFunctional(enum.IntEnum):
    SVWN5 = 0
    BLYP = 1
    PBE = 2
    B3LYP = 3   # 0.20 HF + 0.80 Slater + 0.72 dB88 + 0.19 VWN_RPA + 0.81 LYP
    B3LYP5 = 4  # as B3LYP with VWN5
    PBE0 = 5    # 0.25 HF + 0.75 PBE_X + 1.00 PBE_C

    @classmethod
    def from_name(cls, name: str) -> "XcFunctional":
        """XcFunctional::from_name (xc.rs:51-72) for the functionals this library evaluates."""
        norm = "".join(c for c in name.strip().lower() if not c.isspace() and c not in "-_")
        table = {"svwn": cls.SVWN5, "svwn5": cls.SVWN5, "lda": cls.SVWN5, "slatervwn5": cls.SVWN5,
                 "blyp": cls.BLYP, "pbe": cls.PBE, "pbepbe": cls.PBE, "b3lyp": cls.B3LYP,
                 "b3lyp5": cls.B3LYP5, "pbe0": cls.PBE0, "pbe1pbe": cls.PBE0}
        if norm not in table:
            raise ValueError(f"unsupported DFT XC functional {name!r} (supported: SVWN5, BLYP, PBE, B3LYP, "
                             "B3LYP5, PBE0)")
        return table[norm]

    def exact_exchange_fraction(self) -> float:
        """xc.rs:116-125 (handled by the J/K builder, not by the quadrature)."""
        return {0: 0.0, 1: 0.0, 2: 0.0, 3: 0.20, 4: 0.20, 5: 0.25}[int(self)]

    def is_gga(self) -> bool:
        return self != XcFunctional.SVWN5

    def canonical_name(self) -> str:
        return ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"][int(self)]
