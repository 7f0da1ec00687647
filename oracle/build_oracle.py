"""Compiles the oracle into oracle/_build/liboracle.so with g++.

calchem_oracle.cpp (the checker) keeps IEEE FP64 semantics close to CalChem's Rust: -O2, no
-ffast-math, and -ffp-contract=off so no multiply-add is fused.  cpu_gemm.cpp (the register-blocked
product the timed CPU baseline uses for its two contractions, as CalChem's faer GEMM does) is
compiled with -O3 and fused multiply-adds allowed, no -ffast-math and no machine-specific flags, so
it vectorises on both x86-64 and AArch64.  OpenMP provides the worker threads that stand in for
rayon.  CalChem itself (Rust, crates not vendored) cannot be compiled here, so there is no
oracle/_ref build.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "calchem_oracle.cpp")
GEMM = os.path.join(HERE, "cpu_gemm.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(GEMM), os.path.getmtime(__file__))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    o_main = os.path.join(OUT_DIR, "calchem_oracle.o")
    o_gemm = os.path.join(OUT_DIR, "cpu_gemm.o")
    _run(["g++", "-c", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", SRC, "-o", o_main])
    _run(["g++", "-c", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=fast", GEMM, "-o", o_gemm])
    _run(["g++", "-shared", "-fopenmp", o_main, o_gemm, "-o", LIB])
    return LIB


if __name__ == "__main__":
    print(build(force=True))
