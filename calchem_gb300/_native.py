"""ctypes binding of libcalchem_xc.so (the C ABI in include/calchem_xc.h).

The library is built in-tree by ``calchem_gb300.build.build()``.  There is no
Python or CPU fallback for anything the library does: if it is missing, every
entry point raises.
"""

import ctypes
import os

import numpy as np

from . import build as _build

# numpy mirrors of the #[repr(C)] structs (crates/calchem-cuda/src/lib.rs:46-84)
AO_SHELL = np.dtype([("center", "<f8", (3,)), ("r2_cutoff", "<f8"), ("ao_offset", "<i4"), ("n_funcs", "<i4"),
                     ("prim_start", "<i4"), ("n_prims", "<i4"), ("comp_start", "<i4"), ("atom_index", "<i4")])
AO_PRIM = np.dtype([("exponent", "<f8"), ("weighted_norm", "<f8")])
AO_COMP = np.dtype([("scale", "<f8"), ("lx", "<i4"), ("ly", "<i4"), ("lz", "<i4"), ("_pad", "<i4")])
GRID_PT = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("batch_id", "<i4"), ("host_atom", "<i4")])
assert AO_SHELL.itemsize == 56 and AO_PRIM.itemsize == 16 and AO_COMP.itemsize == 24 and GRID_PT.itemsize == 32

_P = ctypes.c_void_p
_I = ctypes.c_int
_U64 = ctypes.c_uint64
_SZ = ctypes.c_size_t
_DP = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes), the full exported surface of include/calchem_xc.h
SIGNATURES = {
    "calchem_cuda_is_available": (_I, []),
    "calchem_cuda_vxc_upload_grid": (_I, [_P, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I, _I, _U64, _SZ]),
    "calchem_cuda_vxc_eval_rho": (_I, [_U64, _P, _P, _I, _I]),
    "calchem_cuda_vxc_accum": (_I, [_U64, _P, _P, _I, _I]),
    "calchem_cuda_vxc_grad_force": (_I, [_U64, _P, _P, _I, _P, _P, _I, _I, _I, _SZ]),
    "calchem_cuda_vxc_release": (_I, [_U64]),
    "calchem_xc_prepare_shells": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "calchem_xc_overlap": (_I, [_P, _I, _P, _P, _I, _P]),
    "calchem_xc_grid_build": (_I, [_I, _P, _P, _I, _I, _U64, _P]),
    "calchem_xc_grid_build_atoms": (_I, [_I, _P, _P, _P, _P, _P, _U64, _P]),
    "calchem_xc_grid_fetch": (_I, [_U64, _P, _P, _P]),
    "calchem_xc_grid_release": (_I, [_U64]),
    "calchem_xc_upload_points": (_I, [_P, _I, _P, _I, _P, _I, _P, _I, _I, _U64, _SZ]),
    "calchem_xc_upload_points_ex": (_I, [_P, _I, _P, _I, _P, _I, _P, _I, _I, _I, _U64, _SZ]),
    "calchem_xc_upload_points_spatial": (_I, [_P, _I, _P, _I, _P, _I, _P, _I, _I, _I, _U64, _SZ]),
    "calchem_xc_upload_points_screened": (_I, [_P, _I, _P, _I, _P, _I, _P, _I, _I, _I, _U64, _SZ, ctypes.c_double]),
    "calchem_xc_plan_points": (_I, [_P, _I, _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I]),
    "calchem_xc_set_weights": (_I, [_U64, _P, _I]),
    "calchem_xc_plan_stats": (_I, [_U64, _P, _P, _P, _P]),
    "calchem_xc_evaluate_rks": (_I, [_U64, _I, _I, _P, _P, _P, _P]),
    "calchem_xc_evaluate_rks_points": (_I, [_U64, _I, _I, _P, _P, _P, _P]),
    "calchem_xc_set_tile": (_I, [_U64, _I]),
    "calchem_xc_get_tile": (_I, [_U64]),
    "calchem_xc_set_point_atoms": (_I, [_U64, _P, _I, _I]),
    "calchem_xc_evaluate_rks_atoms": (_I, [_U64, _I, _I, _P, _P, _P, _P, _P]),
    "calchem_xc_evaluate_rks_atoms_device": (_I, [_U64, _I, _I, _P, _P, _P, _P, _P]),
    "calchem_xc_eval_closed_shell": (_I, [_I, _I, _I, _P, _P, _P]),
    "calchem_xc_set_ao_cache": (_I, [_U64, _I, _P]),
    "calchem_xc_fxc_contract_ex": (_I, [_U64, _I, _I, _P, _I, _P]),
    "calchem_xc_evaluate_uks": (_I, [_U64, _I, _I, _P, _P, _P, _P, _P, _P]),
    "calchem_xc_evaluate_rks_device": (_I, [_U64, _I, _I, _P, _P, _P, _P]),
    "calchem_xc_evaluate_uks_device": (_I, [_U64, _I, _I, _P, _P, _P, _P, _P, _P]),
    "calchem_xc_last_launch_count": (_I, [_U64]),
    "calchem_xc_set_profiling": (_I, [_U64, _I]),
    "calchem_xc_last_kernel_ms": (_I, [_U64, _P]),
    "calchem_xc_evaluate_rks_static": (_I, [_P, _I, _P, _I, _P, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _I, _P, _P,
                                           _P, _P]),
    "calchem_xc_fxc_prepare": (_I, [_U64, _I, _P]),
    "calchem_xc_fxc_contract": (_I, [_U64, _I, _P, _I, _P]),
    "calchem_xc_fxc_contract_device": (_I, [_U64, _I, _P, _I, _P, _P]),
    "calchem_xc_fxc_contract_device_ex": (_I, [_U64, _I, _I, _P, _I, _P, _P]),
    "calchem_xc_nuclear_gradient": (_I, [_U64, _I, _I, _I, _P, _P, _P, _P, _I, _P, _P, _P]),
    "calchem_xc_group_create": (_I, [_P, _I, _U64, ctypes.c_size_t]),
    "calchem_xc_group_layout": (_I, [_U64, _P, _P, _P]),
    "calchem_xc_graph_capture": (_I, [_U64, _I, _I, _I, _P, _P, _P, _P, _P]),
    "calchem_xc_graph_launch": (_I, [_U64, _P]),
    "calchem_xc_last_status": (_I, [_U64]),
    "calchem_mlp_shape": (_I, [_P, _P, _P, _P, _P]),
    "calchem_mlp_forward": (_I, [_P, _P, _I, _P, _P]),
    "calchem_mlp_loss_grad": (_I, [_P, _P, _P, _P, _I, ctypes.c_float, _P, _P, _P, _P, _P]),
    "calchem_mlp_adam": (_I, [_P, _P, _P, _P, _I, _I, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                              ctypes.c_float, _P]),
    "calchem_scf_boys": (_I, [_I, ctypes.c_double, _P]),
    "calchem_scf_one_electron": (_I, [_P, _I, _P, _P, _I, _I, _P, _P, _P, _P, _P]),
    "calchem_scf_eri": (_I, [_P, _I, _P, _P, _I, _P]),
    "calchem_xc_version": (ctypes.c_char_p, []),
}

_lib = None


class CalchemXcError(RuntimeError):
    """A nonzero status returned by the C ABI (codes documented in include/calchem_xc.h)."""

    MESSAGES = {
        -1: "bad arguments",
        -2: "unknown grid id, size mismatch or size overflow",
        -3: "no usable CUDA device or over the memory budget",
        -4: "device allocation failure",
        -5: "copy or kernel launch failure",
        -6: "device overflow flag",
        -7: "device-side wait expired",
    }

    def __init__(self, func, code):
        self.code = code
        super().__init__(f"{func} returned {code} ({self.MESSAGES.get(code, 'unknown error')})")


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Loads the library; raises if it is not built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"calchem_gb300 native library missing at {path}; run calchem_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(a):
    """Address of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data


def check(func: str, code: int) -> None:
    if code != 0:
        raise CalchemXcError(func, code)
