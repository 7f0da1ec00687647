"""Shared test inputs, restated from CalChem's own vxc tests."""

import math

import numpy as np

from calchem_gb300.molecule import Atom, Molecule

DISTORTED_WATER = [("O", [0.02, -0.04, 0.11]), ("H", [0.81, 0.59, -0.37]), ("H", [-0.74, 0.63, -0.42])]


def distorted_water() -> Molecule:
    """crates/calchem-dft/src/vxc.rs:2345-2362."""
    return Molecule([Atom.from_angstrom(s, p) for s, p in DISTORTED_WATER], 0, 1)


def make_positive_density(n: int, seed_shift: int) -> np.ndarray:
    """P = A A^T + 0.05 I with A[mu,k] = 0.22 sin(0.37 (7 mu + 13 k + 5 s + 3)) (vxc.rs:2364-2385)."""
    a = np.zeros((n, 4))
    for mu in range(n):
        for k in range(4):
            a[mu, k] = 0.22 * math.sin((mu * 7 + k * 13 + seed_shift * 5 + 3) * 0.37)
    return a @ a.T + 0.05 * np.eye(n)


def oracle_basis(O, name, mol):
    return O.Basis.from_name(name, [a.symbol for a in mol.atoms], mol.coords_bohr)


def reference_layout(basis, grid):
    """What CalChem's RksVxcEngine::new_with_gpu uploads (vxc.rs:443-596): 128-point chunks of the
    grid, points with |w| < 1e-24 skipped, bounding sphere, candidate shells with
    |C - centre| <= r_box + r_cut; chunks without points or candidates are dropped."""
    from calchem_gb300 import _native

    sh, _, _ = basis.gpu_arrays()
    centers = np.array([s["center"] for s in sh])
    rcut = np.sqrt(sh["r2_cutoff"])
    xyzw = grid.xyzw
    hosts = getattr(grid, "host_atom", None)
    pts, ws, off, cs = [], [], [0], []
    bid = 0
    for s0 in range(0, len(xyzw), 128):
        chunk = xyzw[s0:s0 + 128]
        keep = np.abs(chunk[:, 3]) >= 1e-24
        if not keep.any():
            continue
        c = chunk[keep]
        mn, mx = c[:, :3].min(axis=0), c[:, :3].max(axis=0)
        cen = 0.5 * (mn + mx)
        rbox = float(np.sqrt(np.sum((mx - cen) ** 2)))
        d2 = np.sum((centers - cen) ** 2, axis=1)
        cand = np.where(d2 <= (rbox + rcut) ** 2)[0]
        if len(cand) == 0:
            continue
        cs.extend(int(i) for i in cand)
        off.append(len(cs))
        for k in np.where(keep)[0]:
            p = chunk[k]
            pts.append((p[0], p[1], p[2], bid, 0 if hosts is None else int(hosts[s0 + k])))
            ws.append(p[3])
        bid += 1
    return (np.array(pts, dtype=_native.GRID_PT), np.array(ws), np.array(off, np.int32), np.array(cs, np.int32))
