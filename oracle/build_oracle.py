"""Compiles the oracle (calchem_oracle.cpp) into oracle/_build/liboracle.so with g++.

The flags keep IEEE FP64 semantics close to CalChem's Rust: -O2, no -ffast-math,
and -ffp-contract=off so no multiply-add is fused.  OpenMP provides the worker
threads that stand in for rayon.  CalChem itself (Rust, crates not vendored)
cannot be compiled here, so there is no oracle/_ref build.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "calchem_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           SRC, "-o", LIB]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
