"""Builds libcalchem_xc.so (sm_103a) in-tree, with nvcc and g++ directly (no cmake).

Translation units are compiled in parallel; the grid builder is compiled with
``-fmad=false`` and the host preparation code with ``-ffp-contract=off`` so that
their floating-point results round like CalChem's Rust (no fused multiply-add).
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libcalchem_xc.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CUDA_UNITS = {
    "capi.cu": [],
    "vxc_fp64.cu": [],
    "vxc_mixed.cu": [],
    "grid_build.cu": ["-fmad=false"],
    "noalloc.cu": [],
    "mlp.cu": [],
    "fxc.cu": [],
    "xc_grad.cu": [],
    "xc_grad_mixed.cu": [],
}
CXX_UNITS = {"host_prep.cpp": [], "integrals.cpp": []}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build calchem_gb300")
    return cand


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "calchem_xc.h"))
    jobs = []
    objs = []
    for name, extra in CUDA_UNITS.items():
        src = os.path.join(CSRC, name)
        obj = os.path.join(LIBDIR, name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-I", INCLUDE] + ARCH + extra)
    for name, extra in CXX_UNITS.items():
        src = os.path.join(CSRC, name)
        obj = os.path.join(LIBDIR, name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-c", src, "-o", obj, "-O2", "-std=c++17", "-fPIC", "-fopenmp",
                         "-ffp-contract=off", "-I", INCLUDE] + extra)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
