"""GPU tests of the tensor-core (mixed-precision) form.

Tolerances (stated here and in the library documentation):
  |dExc| <= 1e-7 Eh and |dNelec| <= 1e-7 against the FP64 form -- tighter than the 1e-6 Eh per
  molecule the design targets; measured errors are ~1e-9;
  max |dVxc| <= 2e-6 (the V contraction runs a three-piece floating BF16 split, ~3e-7 measured).
"""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, workloads
from tests.helpers import distorted_water, make_positive_density, oracle_basis

pytestmark = pytest.mark.gpu

EXC_TOL = 1e-7
N_TOL = 1e-7
V_TOL = 2e-6


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"])
def test_mixed_rks_matches_oracle_distorted_water(lib, oracle, func):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    P = make_positive_density(basis.n_ao, 7)
    eng = RksVxcEngine(basis, grid, precision="mixed")
    exc, V = eng.evaluate(basis, grid, func, P)
    e_ref, n_ref, V_ref = oracle.vxc_rks_points(oracle_basis(oracle, "6-31g(d)", mol),
                                                oracle.Grid.from_points(grid.xyzw), P, func)
    assert abs(exc - e_ref) < EXC_TOL
    assert abs(eng.last_nelec - n_ref) < N_TOL
    assert np.max(np.abs(V - V_ref)) < V_TOL
    assert np.array_equal(V, V.T)


def test_mixed_rks_octane_fine_against_fp64(lib):
    """The benchmark workload (C8H18, B3LYP, 6-31G(d,p), Fine grid): mixed vs the FP64 form."""
    mol = workloads.octane()
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), 33, 7)
    eng = RksVxcEngine(basis, grid)
    e64, V64 = eng.evaluate(basis, grid, "b3lyp", D, precision="fp64")
    n64 = eng.last_nelec
    em, Vm = eng.evaluate(basis, grid, "b3lyp", D, precision="mixed")
    assert abs(em - e64) < EXC_TOL
    assert abs(eng.last_nelec - n64) < N_TOL
    assert np.max(np.abs(Vm - V64)) < V_TOL
    assert abs(eng.last_nelec - 66.0) < 1e-2  # tr(D S) = 2 n_occ up to quadrature error


@pytest.mark.parametrize("func", ["blyp", "pbe0"])
def test_mixed_uks_matches_oracle(lib, oracle, func):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    Pa = make_positive_density(basis.n_ao, 2)
    Pb = make_positive_density(basis.n_ao, 5)
    eng = UksVxcEngine(basis, grid, precision="mixed")
    exc, Va, Vb = eng.evaluate(basis, grid, func, Pa, Pb)
    e_ref, na, nb, Va_ref, Vb_ref = oracle.vxc_uks_points(oracle_basis(oracle, "6-31g(d)", mol),
                                                          oracle.Grid.from_points(grid.xyzw), Pa, Pb, func)
    assert abs(exc - e_ref) < EXC_TOL
    assert abs(eng.last_nelec[0] - na) < N_TOL and abs(eng.last_nelec[1] - nb) < N_TOL
    assert np.max(np.abs(Va - Va_ref)) < V_TOL and np.max(np.abs(Vb - Vb_ref)) < V_TOL


def test_mixed_closed_shell_uks_equals_rks(lib):
    mol = workloads.water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), 5, 3)
    r = RksVxcEngine(basis, grid, precision="mixed")
    u = UksVxcEngine(basis, grid, precision="mixed")
    er, Vr = r.evaluate(basis, grid, "pbe", D)
    eu, Va, Vb = u.evaluate(basis, grid, "pbe", 0.5 * D, 0.5 * D)
    assert abs(er - eu) < 1e-9
    assert np.max(np.abs(Va - Vr)) < V_TOL and np.max(np.abs(Va - Vb)) < 1e-14  # atomic order only


def test_mixed_is_deterministic_in_exc(lib):
    """Exc and Nelec come from a fixed-order reduction: repeated builds agree bit for bit."""
    mol = workloads.water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), 5, 7)
    eng = RksVxcEngine(basis, grid, precision="mixed")
    e1, _ = eng.evaluate(basis, grid, "b3lyp", D)
    n1 = eng.last_nelec
    e2, _ = eng.evaluate(basis, grid, "b3lyp", D)
    assert e1 == e2 and n1 == eng.last_nelec


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "pbe0"])
def test_fully_polarised_uks(lib, oracle, func):
    """A doublet with no beta density anywhere (zeta = 1 at every point: the polarised PW92 / VWN
    channels, f(zeta) at its end point): both GPU forms against the oracle.  The empty spin's
    potential follows the reference's formulas there, which for PBE correlation reach ~1e6 through
    f'(zeta) at zeta = 1, so the potentials are compared relative to their largest entry."""
    from calchem_gb300.molecule import Atom, Molecule
    mol = Molecule([Atom.from_angstrom("H", [0.0, 0.0, 0.0])], 0, 2)
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.MEDIUM)
    S = basis.overlap()
    c = np.zeros(basis.n_ao)
    c[0], c[1] = 0.6, 0.5
    c /= np.sqrt(c @ S @ c)  # one normalised alpha orbital
    Pa = np.outer(c, c)
    Pb = np.zeros_like(Pa)
    e_ref, na, nb, Va_ref, Vb_ref = oracle.vxc_uks_points(oracle_basis(oracle, "6-31g(d,p)", mol),
                                                          oracle.Grid.from_points(grid.xyzw), Pa, Pb, func)
    assert nb == 0.0 and abs(na - 1.0) < 1e-3
    for prec, etol, vtol in (("fp64", 1e-9, 1e-10), ("mixed", EXC_TOL, V_TOL)):
        eng = UksVxcEngine(basis, grid, precision=prec)
        exc, Va, Vb = eng.evaluate(basis, grid, func, Pa, Pb)
        eng.close()
        assert abs(exc - e_ref) < etol, (prec, exc - e_ref)
        for V, V_ref in ((Va, Va_ref), (Vb, Vb_ref)):
            assert np.max(np.abs(V - V_ref)) < vtol * max(1.0, np.max(np.abs(V_ref))), prec
