"""GPU tests of the range-separated hybrids' semilocal parts (CAM-B3LYP, wB97X, wB97X-D): both forms
against the oracle on the reference's distorted water (vxc.rs:2345-2385), RKS and UKS."""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine
from tests.helpers import distorted_water, make_positive_density, oracle_basis

pytestmark = pytest.mark.gpu

FUNCS = ["camb3lyp", "wb97x", "wb97xd"]
TOL = {"fp64": (1e-9, 1e-10), "mixed": (1e-7, 2e-6)}


@pytest.fixture(scope="module")
def setup(native_lib, oracle):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    return mol, basis, grid, oracle_basis(oracle, "6-31g(d)", mol), oracle.Grid.from_points(grid.xyzw)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("func", FUNCS)
def test_rks_matches_oracle(setup, oracle, func, precision):
    mol, basis, grid, ob, og = setup
    P = make_positive_density(basis.n_ao, 7)
    eng = RksVxcEngine(basis, grid, precision=precision)
    e, V = eng.evaluate(basis, grid, func, P)
    e_ref, n_ref, V_ref = oracle.vxc_rks_points(ob, og, P, func)
    etol, vtol = TOL[precision]
    assert abs(e - e_ref) < etol and abs(eng.last_nelec - n_ref) < etol
    assert np.max(np.abs(V - V_ref)) < vtol
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("func", FUNCS)
def test_uks_matches_oracle(setup, oracle, func, precision):
    mol, basis, grid, ob, og = setup
    Pa, Pb = make_positive_density(basis.n_ao, 2), make_positive_density(basis.n_ao, 5)
    eng = UksVxcEngine(basis, grid, precision=precision)
    e, Va, Vb = eng.evaluate(basis, grid, func, Pa, Pb)
    e_ref, na, nb, Va_ref, Vb_ref = oracle.vxc_uks_points(ob, og, Pa, Pb, func)
    etol, vtol = TOL[precision]
    assert abs(e - e_ref) < etol
    assert np.max(np.abs(Va - Va_ref)) < vtol and np.max(np.abs(Vb - Vb_ref)) < vtol
    eng.close()
