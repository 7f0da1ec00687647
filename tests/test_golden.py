"""Committed golden fixtures (tests/golden/make_golden.py, made by the oracle): the oracle must keep
reproducing them (CPU), and the GPU forms must match them without the oracle at run time."""

import os

import numpy as np
import pytest

from tests.helpers import distorted_water, oracle_basis

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "distorted_water_631gd_coarse.npz"))
FUNCS = ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"]


def test_oracle_reproduces_golden(oracle):
    mol = distorted_water()
    basis = oracle_basis(oracle, "6-31g(d)", mol)
    grid = oracle.Grid.build(mol.z, mol.coords_bohr, "coarse")
    xyzw, _, _ = grid.points()
    assert len(xyzw) == int(GOLD["grid_n"])
    assert xyzw[:, 3].sum() == pytest.approx(float(GOLD["grid_w_sum"]), rel=1e-14)
    for f in ("svwn5", "b3lyp", "pbe0"):
        e, ne, V = oracle.vxc_rks_points(basis, grid, GOLD["P"], f, threads=1)
        assert e == pytest.approx(float(GOLD[f"rks_{f}_exc"]), rel=1e-13, abs=1e-15)
        assert np.max(np.abs(V - GOLD[f"rks_{f}_V"])) < 1e-13
    for f in FUNCS:
        assert np.allclose(oracle.eval_xc(f, GOLD["xc_points"]), GOLD[f"xc_{f}"], rtol=1e-13, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_matches_golden(native_lib, precision):
    from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine
    assert native_lib.calchem_cuda_is_available() == 1
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build(mol, GridLevel.COARSE)
    assert len(grid) == int(GOLD["grid_n"])
    assert grid.weights.sum() == float(GOLD["grid_w_sum"]) or abs(grid.weights.sum() - float(GOLD["grid_w_sum"])) < 1e-12
    exc_tol, v_tol = (1e-9, 1e-10) if precision == "fp64" else (1e-7, 2e-6)
    eng = RksVxcEngine(basis, grid, precision=precision)
    for f in FUNCS:
        e, V = eng.evaluate(basis, grid, f, GOLD["P"])
        assert abs(e - float(GOLD[f"rks_{f}_exc"])) < exc_tol
        assert abs(eng.last_nelec - float(GOLD[f"rks_{f}_nelec"])) < exc_tol
        assert np.max(np.abs(V - GOLD[f"rks_{f}_V"])) < v_tol
    eng.close()
    ueng = UksVxcEngine(basis, grid, precision=precision)
    for f in ("blyp", "pbe0"):
        e, Va, Vb = ueng.evaluate(basis, grid, f, GOLD["Pa"], GOLD["Pb"])
        assert abs(e - float(GOLD[f"uks_{f}_exc"])) < exc_tol
        assert np.max(np.abs(np.array(ueng.last_nelec) - GOLD[f"uks_{f}_nelec"])) < exc_tol
        assert np.max(np.abs(Va - GOLD[f"uks_{f}_Va"])) < v_tol and np.max(np.abs(Vb - GOLD[f"uks_{f}_Vb"])) < v_tol
    ueng.close()
