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
    CAMB3LYP = 6  # range-separated: ITYH-attenuated B88 exchange + 0.19 VWN5 + 0.81 LYP
    WB97X = 7     # range-separated (omega 0.30)
    WB97XD = 8    # range-separated (omega 0.20)

    @classmethod
    def from_name(cls, name: str) -> "XcFunctional":
        """XcFunctional::from_name (xc.rs:51-72) for the functionals this library evaluates."""
        norm = "".join(c for c in name.strip().lower() if not c.isspace() and c not in "-_")
        table = {"svwn": cls.SVWN5, "svwn5": cls.SVWN5, "lda": cls.SVWN5, "slatervwn5": cls.SVWN5,
                 "blyp": cls.BLYP, "pbe": cls.PBE, "pbepbe": cls.PBE, "b3lyp": cls.B3LYP,
                 "b3lyp5": cls.B3LYP5, "pbe0": cls.PBE0, "pbe1pbe": cls.PBE0, "camb3lyp": cls.CAMB3LYP,
                 "wb97x": cls.WB97X, "wb97xd": cls.WB97XD}
        if norm not in table:
            raise ValueError(f"unsupported DFT XC functional {name!r} (supported: SVWN5, BLYP, PBE, B3LYP, "
                             "B3LYP5, PBE0, CAM-B3LYP, wB97X, wB97X-D)")
        return table[norm]

    def exact_exchange_fraction(self) -> float:
        """xc.rs:116-125 (handled by the J/K builder, not by the quadrature)."""
        return {0: 0.0, 1: 0.0, 2: 0.0, 3: 0.20, 4: 0.20, 5: 0.25, 6: 0.19, 7: 0.157706, 8: 0.222036}[int(self)]

    def is_range_separated(self) -> bool:
        return int(self) >= 6

    def range_separated_params(self):
        """(alpha, beta, omega) of the range-separated hybrids (xc.rs:99-113), else None."""
        return {6: (0.19, 0.46, 0.33), 7: (0.157706, 0.842294, 0.30), 8: (0.222036, 0.777964, 0.20)}.get(int(self))

    def is_gga(self) -> bool:
        return self != XcFunctional.SVWN5

    def canonical_name(self) -> str:
        return ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0", "cam-b3lyp", "wb97x", "wb97x-d"][int(self)]
