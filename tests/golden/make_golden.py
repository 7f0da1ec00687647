"""Writes tests/golden/distorted_water_631gd_coarse.npz from the oracle (the CPU restatement pinned by
the reference's known-answer tests): python tests/golden/make_golden.py

Inputs follow the reference's own Vxc tests (crates/calchem-dft/src/vxc.rs:2345-2385): the distorted
water geometry, 6-31G(d), the Coarse grid, and the sine-generated positive densities.  Stored: the
grid size and the sums of its weights and coordinates; RKS (Exc, Nelec, Vxc) for every functional;
UKS (Exc, N_alpha, N_beta, Va, Vb) for BLYP and PBE0; the six functionals' values and partials at
five (rho_a, rho_b, g_aa, g_ab, g_bb) points."""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from tests.helpers import distorted_water, make_positive_density  # noqa: E402

FUNCS = ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"]
XC_POINTS = np.array([[0.3, 0.3, 0.02, 0.02, 0.02], [0.05, 0.02, 1e-3, 4e-4, 2e-4], [1e-4, 1e-4, 1e-9, 1e-9, 1e-9],
                      [2.0, 0.0, 0.5, 0.0, 0.0], [0.7, 0.4, 0.3, -0.05, 0.1]])


def main():
    mol = distorted_water()
    basis = O.Basis.from_name("6-31g(d)", [a.symbol for a in mol.atoms], mol.coords_bohr)
    grid = O.Grid.build(mol.z, mol.coords_bohr, "coarse")
    xyzw, _, _ = grid.points()
    n = basis.n_ao
    P = make_positive_density(n, 7)
    Pa, Pb = make_positive_density(n, 2), make_positive_density(n, 5)
    out = {"grid_n": np.array(len(xyzw)), "grid_w_sum": np.array(xyzw[:, 3].sum()),
           "grid_xyz_sum": xyzw[:, :3].sum(axis=0), "P": P, "Pa": Pa, "Pb": Pb, "xc_points": XC_POINTS}
    for f in FUNCS:
        e, ne, V = O.vxc_rks_points(basis, grid, P, f, threads=1)
        out[f"rks_{f}_exc"] = np.array(e)
        out[f"rks_{f}_nelec"] = np.array(ne)
        out[f"rks_{f}_V"] = V
        out[f"xc_{f}"] = O.eval_xc(f, XC_POINTS)
    for f in ("blyp", "pbe0"):
        e, na, nb, Va, Vb = O.vxc_uks_points(basis, grid, Pa, Pb, f, threads=1)
        out[f"uks_{f}_exc"] = np.array(e)
        out[f"uks_{f}_nelec"] = np.array([na, nb])
        out[f"uks_{f}_Va"] = Va
        out[f"uks_{f}_Vb"] = Vb
    path = os.path.join(HERE, "distorted_water_631gd_coarse.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
