"""Regenerate the compact basis-set data files in ``calchem_gb300/data/basis/``.

CalChem embeds its Gaussian basis sets as MolSSI-BSE-derived JSON
(``crates/calchem-basis/data/{sto-3g,6-31g,6-31gd,6-31gdp}.json``, loaded by
``crates/calchem-basis/src/lib.rs:10-13, 323-327``).  The XC quadrature only
needs the light elements, so this script keeps H..Ar (Z = 1..18) and writes
one compact JSON per basis with the same content per element:
``{"name": ..., "elements": {"C": [["s", [exps...], [coefs...]], ...]}}``.
Shell order inside an element is preserved because it fixes the AO order.

Usage (needs the CalChem checkout, so it is run on the development machine
only; the generated files are committed):

    python calchem_gb300/data/extract_basis.py /path/to/CalChem
"""

import json
import os
import sys

LIGHT = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
         "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]
FILES = {"sto-3g": "sto-3g.json", "6-31g": "6-31g.json",
         "6-31g(d)": "6-31gd.json", "6-31g(d,p)": "6-31gdp.json"}


def main(ref_root: str) -> None:
    src_dir = os.path.join(ref_root, "crates", "calchem-basis", "data")
    out_dir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis")
    os.makedirs(out_dir, exist_ok=True)
    for name, fname in FILES.items():
        with open(os.path.join(src_dir, fname)) as f:
            raw = json.load(f)
        elements = {}
        for sym in LIGHT:
            if sym not in raw["elements"]:
                continue
            elements[sym] = [[sh["shell_type"], sh["exponents"], sh["coefficients"]]
                             for sh in raw["elements"][sym]]
        out = {"name": name, "source": raw.get("source", ""), "elements": elements}
        with open(os.path.join(out_dir, fname), "w") as f:
            json.dump(out, f, separators=(",", ":"))
            f.write("\n")
        print(f"{name}: {len(elements)} elements -> {fname}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python calchem_gb300/data/extract_basis.py /path/to/CalChem")
    main(sys.argv[1])
