"""ctypes wrapper of the oracle (calchem_oracle.cpp) -- test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; never by the product.  Basis data are read from the same JSON data
files the product ships (data, not algorithm); the normalisation arithmetic is
the oracle's own (calchem_oracle.cpp).
"""

import ctypes
import json
import os

import numpy as np

from . import build_oracle

_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

_SIGS = {
    "orc_lebedev": (_I, [_I, _P]),
    "orc_bragg_slater_bohr": (_D, [_I]),
    "orc_radial_shell_count": (_I, [_I, _I]),
    "orc_grid_build": (_P, [_I, _P, _P, _I, _I]),
    "orc_grid_from_points": (_P, [_I, _P, _P]),
    "orc_grid_size": (_I, [_P]),
    "orc_grid_points": (None, [_P, _P, _P, _P]),
    "orc_grid_free": (None, [_P]),
    "orc_becke_weight": (_D, [_I, _P, _P, _I, _P]),
    "orc_basis_create": (_P, [_I, _P, _P, _P, _P, _P, _P]),
    "orc_basis_nao": (_I, [_P]),
    "orc_basis_free": (None, [_P]),
    "orc_basis_shell_data": (None, [_P, _P, _P, _P]),
    "orc_ao_grad": (None, [_P, _I, _P, _P]),
    "orc_ao_hess": (None, [_P, _I, _P, _P]),
    "orc_eval_xc": (None, [_I, _I, _P, _P]),
    "orc_lyp": (None, [_P, _P]),
    "orc_vxc_rks_points": (None, [_P, _P, _P, _I, _I, _P, _P, _P]),
    "orc_vxc_uks_points": (None, [_P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P]),
    "orc_rks_engine_create": (_P, [_P, _P, _D, _I]),
    "orc_rks_engine_is_cached": (_I, [_P]),
    "orc_rks_engine_cache_bytes": (_D, [_P]),
    "orc_rks_engine_n_batches": (_I, [_P]),
    "orc_rks_engine_work": (_D, [_P]),
    "orc_rks_engine_evaluate": (None, [_P, _P, _I, _I, _P, _P, _P, _I, _I, _I]),
    "orc_rks_engine_free": (None, [_P]),
    "orc_overlap": (None, [_P, _P]),
    "orc_max_threads": (_I, []),
    "orc_cam_x_one": (None, [_D, _D, _P]),
    "orc_xc_gradient": (None, [_P, _P, _I, _P, _P, _P, _P, _I, _I, _P]),
    "orc_grid_from_points_raw": (_P, [_I, _P, _P, _P]),
}

XC_CODES = {"svwn5": 0, "blyp": 1, "pbe": 2, "b3lyp": 3, "b3lyp5": 4, "pbe0": 5, "camb3lyp": 6, "cam-b3lyp": 6,
            "wb97x": 7, "wb97xd": 8, "wb97x-d": 8}
LEVELS = {"coarse": 0, "medium": 1, "fine": 2, "ultrafine": 3}
_BASIS_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "calchem_gb300", "data",
                          "basis")
_BASIS_FILES = {"sto-3g": "sto-3g.json", "6-31g": "6-31g.json", "6-31g(d)": "6-31gd.json",
                "6-31g(d,p)": "6-31gdp.json"}
_LNUM = {"s": 0, "p": 1, "d": 2, "f": 3}


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        for k, (r, a) in _SIGS.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def xc_code(func):
    if isinstance(func, str):
        return XC_CODES[func.lower()]
    return int(func)


def lebedev(n):
    out = np.zeros((n, 4))
    got = lib().orc_lebedev(n, _p(out))
    assert got == n
    return out


class Grid:
    def __init__(self, handle):
        self.h = handle

    @classmethod
    def build(cls, z, xyz_bohr, level="fine", radial_min=0):
        z = np.ascontiguousarray(z, dtype=np.int32)
        xyz = np.ascontiguousarray(xyz_bohr, dtype=np.float64)
        lv = LEVELS[level] if isinstance(level, str) else int(level)
        return cls(lib().orc_grid_build(len(z), _p(z), _p(xyz), lv, int(radial_min)))

    @classmethod
    def from_points(cls, xyzw, host=None, raw_w=None):
        xyzw = np.ascontiguousarray(xyzw, dtype=np.float64).reshape(-1, 4)
        host = np.zeros(len(xyzw), np.int32) if host is None else np.ascontiguousarray(host, dtype=np.int32)
        if raw_w is None:
            return cls(lib().orc_grid_from_points(len(xyzw), _p(xyzw), _p(host)))
        raw_w = np.ascontiguousarray(raw_w, dtype=np.float64)
        return cls(lib().orc_grid_from_points_raw(len(xyzw), _p(xyzw), _p(raw_w), _p(host)))

    def __len__(self):
        return lib().orc_grid_size(self.h)

    def points(self):
        n = len(self)
        xyzw = np.zeros((n, 4))
        raw = np.zeros(n)
        host = np.zeros(n, np.int32)
        lib().orc_grid_points(self.h, _p(xyzw), _p(raw), _p(host))
        return xyzw, raw, host

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_grid_free(self.h)
            self.h = None


def basis_shells(name, symbols, xyz_bohr):
    """Raw shells (l, atom, centre, exps, coefs) for a molecule from the shipped JSON data."""
    with open(os.path.join(_BASIS_DIR, _BASIS_FILES[name])) as f:
        data = json.load(f)["elements"]
    out = []
    for ia, (s, c) in enumerate(zip(symbols, np.asarray(xyz_bohr).reshape(-1, 3))):
        for st, ex, cf in data[s]:
            out.append((_LNUM[st], ia, c, ex, cf))
    return out


class Basis:
    def __init__(self, shells):
        ls = np.array([s[0] for s in shells], np.int32)
        at = np.array([s[1] for s in shells], np.int32)
        cen = np.ascontiguousarray(np.array([s[2] for s in shells], np.float64))
        npr = np.array([len(s[3]) for s in shells], np.int32)
        ex = np.ascontiguousarray(np.concatenate([np.asarray(s[3], float) for s in shells]))
        cf = np.ascontiguousarray(np.concatenate([np.asarray(s[4], float) for s in shells]))
        self.h = lib().orc_basis_create(len(shells), _p(ls), _p(at), _p(cen), _p(npr), _p(ex), _p(cf))
        self.n_ao = lib().orc_basis_nao(self.h)
        self.n_shells = len(shells)
        self.n_prims = int(npr.sum())

    @classmethod
    def from_name(cls, name, symbols, xyz_bohr):
        return cls(basis_shells(name, symbols, xyz_bohr))

    def shell_data(self):
        r2 = np.zeros(self.n_shells)
        wn = np.zeros(self.n_prims)
        cs = np.zeros(self.n_ao)
        lib().orc_basis_shell_data(self.h, _p(r2), _p(wn), _p(cs))
        return r2, wn, cs

    def ao_grad(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros((len(xyz), self.n_ao, 4))
        lib().orc_ao_grad(self.h, len(xyz), _p(xyz), _p(out))
        return out

    def ao_hess(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros((len(xyz), self.n_ao, 10))
        lib().orc_ao_hess(self.h, len(xyz), _p(xyz), _p(out))
        return out

    def overlap(self):
        S = np.zeros((self.n_ao, self.n_ao))
        lib().orc_overlap(self.h, _p(S))
        return S

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_basis_free(self.h)
            self.h = None


def eval_xc(func, inputs):
    """inputs (N, 5) = (rho_a, rho_b, g_aa, g_ab, g_bb) -> (N, 6) = (f, v_ra, v_rb, v_gaa, v_gab, v_gbb)."""
    x = np.ascontiguousarray(np.atleast_2d(inputs), np.float64)
    out = np.zeros((len(x), 6))
    lib().orc_eval_xc(xc_code(func), len(x), _p(x), _p(out))
    return out


def xc_gradient(basis, grid, z, xyz_bohr, Pa, Pb, func, parts=3):
    """dExc/dR [n_atoms][3] at fixed spin densities (vxc.rs:1769-1912); parts 1 = AO terms only,
    2 = Becke weight term only, 3 = both."""
    z = np.ascontiguousarray(z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz_bohr, dtype=np.float64)
    out = np.zeros((len(z), 3))
    lib().orc_xc_gradient(basis.h, grid.h, len(z), _p(z), _p(xyz), _p(np.ascontiguousarray(Pa, np.float64)),
                          _p(np.ascontiguousarray(Pb, np.float64)), xc_code(func), int(parts), _p(out))
    return out


def cam_x_one(rho, gamma):
    """CAM-B3LYP attenuated exchange of one spin: (f, v_rho, v_gamma)."""
    out = np.zeros(3)
    lib().orc_cam_x_one(float(rho), float(gamma), _p(out))
    return out


def lyp(inputs):
    x = np.ascontiguousarray(inputs, np.float64)
    out = np.zeros(6)
    lib().orc_lyp(_p(x), _p(out))
    return out


def vxc_rks_points(basis, grid, P, func, threads=0):
    P = np.ascontiguousarray(P, np.float64)
    n = basis.n_ao
    V = np.zeros((n, n))
    e = np.zeros(1)
    ne = np.zeros(1)
    lib().orc_vxc_rks_points(basis.h, grid.h, _p(P), xc_code(func), int(threads), _p(e), _p(ne), _p(V))
    return float(e[0]), float(ne[0]), V


def vxc_uks_points(basis, grid, Pa, Pb, func, threads=0):
    Pa = np.ascontiguousarray(Pa, np.float64)
    Pb = np.ascontiguousarray(Pb, np.float64)
    n = basis.n_ao
    Va = np.zeros((n, n))
    Vb = np.zeros((n, n))
    e = np.zeros(1)
    na = np.zeros(1)
    nb = np.zeros(1)
    lib().orc_vxc_uks_points(basis.h, grid.h, _p(Pa), _p(Pb), xc_code(func), int(threads), _p(e), _p(na), _p(nb),
                             _p(Va), _p(Vb))
    return float(e[0]), float(na[0]), float(nb[0]), Va, Vb


class RksEngine:
    """Restatement of RksVxcEngine's CPU path (cached-AO BLAS-3 when under the cache cap)."""

    def __init__(self, basis, grid, cap_bytes=-1.0, threads=0):
        self.basis = basis
        self.h = lib().orc_rks_engine_create(basis.h, grid.h, float(cap_bytes), int(threads))
        self.cached = bool(lib().orc_rks_engine_is_cached(self.h))
        self.cache_bytes = lib().orc_rks_engine_cache_bytes(self.h)
        self.n_batches = lib().orc_rks_engine_n_batches(self.h)
        self.work = lib().orc_rks_engine_work(self.h)  # sum over CalChem's batches of m_b^2 n_b

    def evaluate(self, P, func, threads=0, batch_range=(-1, -1), blocked=False):
        """blocked: the two contractions by the register-blocked FMA product (cpu_gemm.cpp), as the
        reference runs them through faer; the default plain loops are the checker's."""
        P = np.ascontiguousarray(P, np.float64)
        n = self.basis.n_ao
        V = np.zeros((n, n))
        e = np.zeros(1)
        ne = np.zeros(1)
        lib().orc_rks_engine_evaluate(self.h, _p(P), xc_code(func), int(threads), _p(e), _p(ne), _p(V),
                                      int(batch_range[0]), int(batch_range[1]), int(bool(blocked)))
        return float(e[0]), float(ne[0]), V

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_rks_engine_free(self.h)
            self.h = None


def max_threads():
    return lib().orc_max_threads()
