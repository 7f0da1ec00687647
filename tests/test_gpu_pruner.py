"""GPU tests of the learned grid pruner: per-atom grids, per-atom quadrature shares, and the pruned
grid against the Fine grid as judge."""

import os

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, pruner, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


def test_all_fine_levels_reproduce_the_fine_grid(lib):
    mol = workloads.water_cluster(3, 4)
    g0 = MolecularGrid.build(mol, GridLevel.FINE)
    g1 = pruner.grid_for_levels(mol, [pruner.FINE] * len(mol.atoms))
    assert len(g0) == len(g1)
    assert np.array_equal(g0.xyzw, g1.xyzw) and np.array_equal(g0.host_atom, g1.host_atom)


def test_level_grids_shrink_and_per_atom_levels_mix(lib):
    mol = workloads.water_cluster(2, 9)
    sizes = [len(pruner.grid_for_levels(mol, [l] * len(mol.atoms))) for l in range(len(pruner.LEVELS))]
    assert sizes[0] < sizes[-1] and sizes == sorted(sizes)
    mixed = [0, pruner.FINE] * (len(mol.atoms) // 2) + [3] * (len(mol.atoms) % 2)
    g = pruner.grid_for_levels(mol, mixed)
    per_atom = np.bincount(g.host_atom, minlength=len(mol.atoms))
    fine = np.bincount(pruner.grid_for_levels(mol, [pruner.FINE] * len(mol.atoms)).host_atom)
    assert np.all(per_atom[np.array(mixed) == pruner.FINE] == fine[np.array(mixed) == pruner.FINE])


def test_atom_shares_sum_to_the_engine_results(lib):
    mol = workloads.water_cluster(2, 3)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 4)
    E, T = pruner.atom_shares(mol, basis, grid, "b3lyp", D)
    eng = RksVxcEngine(basis, grid)
    exc, V = eng.evaluate(basis, grid, "b3lyp", D)
    assert abs(E.sum() - exc) < 1e-10
    assert abs(T.sum() - np.sum(D * V)) < 1e-9
    eng.close()


# FP64: the same sums in another order; tensor-core form: its per-point error summed over an
# atom's points (~2e-10 of an oxygen's share of Exc, ~5 Eh)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 3e-9)])
def test_device_atom_sums_match_the_per_point_shares(lib, precision, tol):
    """calchem_xc_evaluate_rks_atoms (shares only, summed per atom on the device) against the host
    sums of calchem_xc_evaluate_rks_points' per-point shares, on a grid and on a subset of its atoms'
    points (what the judge uploads)."""
    mol = workloads.water_cluster(3, 8)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 5)
    n = len(mol.atoms)
    E_ref, T_ref = pruner.atom_shares(mol, basis, grid, "b3lyp", D)
    eng = pruner.ShareEngine(basis, grid, n)
    for _ in range(2):  # resident: a second evaluation reuses the upload (and the AO cache)
        E, T = eng.shares(D, "b3lyp", precision)
        assert np.max(np.abs(E - E_ref)) < tol and np.max(np.abs(T - T_ref)) < tol
    eng.close()
    atoms = np.array([1, 4, 6])
    keep = np.isin(grid.host_atom, atoms)
    sub = MolecularGrid(grid.xyzw[keep], grid.raw_weight[keep], grid.host_atom[keep], grid.level)
    eng = pruner.ShareEngine(basis, sub, n)
    E, T = eng.shares(D, "b3lyp", precision)
    assert np.max(np.abs(E[atoms] - E_ref[atoms])) < tol and np.max(np.abs(T[atoms] - T_ref[atoms])) < tol
    others = np.setdiff1d(np.arange(n), atoms)
    assert np.all(E[others] == 0) and np.all(T[others] == 0)
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_build_with_shares_matches_the_build_and_the_share_engine(lib, precision):
    """evaluate_with_shares: the same Exc, Nelec and Vxc as evaluate (the tensor-core form: the same up
    to the rounding of grad rho, which plain builds sum by FP32 FMAs and builds with shares with
    compensation), and the same per-atom shares as a shares-only evaluation of the same points; the
    judge reverts the same atoms with them."""
    mol = workloads.water_cluster(4, 6)
    basis = BasisSet.from_name("6-31g(d)", mol)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 9)
    lg = pruner.LearnedGrid(mol, basis, tol=5e-7)
    n = len(mol.atoms)
    eng = RksVxcEngine(basis, lg.grid, precision=precision)
    eng.set_point_atoms(lg.grid.host_atom, n)
    e0, V0 = eng.evaluate(basis, lg.grid, "b3lyp", D)
    n0 = eng.last_nelec
    e1, V1, E, T = eng.evaluate_with_shares(basis, lg.grid, "b3lyp", D)
    assert eng.last_nelec == n0
    if precision == "fp64":
        assert e1 == e0 and np.max(np.abs(V1 - V0)) < 1e-12
    else:
        assert abs(e1 - e0) < 2e-9 and np.max(np.abs(V1 - V0)) < 1e-7
    assert abs(E.sum() - e1) < 1e-10
    share = pruner.ShareEngine(basis, lg.grid, n)
    Es, Ts = share.shares(D, "b3lyp", precision)
    assert np.max(np.abs(E - Es)) < 1e-12 and np.max(np.abs(T - Ts)) < 1e-12
    share.close()
    bad_a, err_a = lg.check(D, "b3lyp", precision=precision)
    lg2 = pruner.LearnedGrid(mol, basis, tol=5e-7)
    bad_b, err_b = lg2.check(D, "b3lyp", precision=precision, pruned_shares=(E, T))
    at = lg2.pruned_atoms()
    assert bad_a == bad_b
    assert np.max(np.abs(err_a[at] - err_b[at])) < 1e-12
    eng.close()
    lg.close()
    lg2.close()


def test_level_errors_shrink_towards_fine(lib):
    mol = workloads.water_cluster(2, 3)
    basis = BasisSet.from_name("6-31g(d)", mol)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 4)
    err = pruner.level_errors(mol, basis, "pbe", D)
    assert np.all(err[:, pruner.FINE] == 0)
    assert np.all(np.isfinite(err))
    assert np.median(err[:, 0]) > np.median(err[:, pruner.FINE - 1])


@pytest.mark.skipif(not os.path.exists(pruner.MODEL_PATH), reason="no trained pruner model")
def test_learned_grid_meets_tolerance_with_fewer_points(lib):
    """Held-out geometry: the network prunes, the Fine-grid judge reverts what exceeds the per-atom
    tolerance, and the pruned grid then meets the per-molecule tolerance with fewer points."""
    mol = workloads.water_cluster(10, 4242)
    basis = BasisSet.from_name("6-31g(d)", mol)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 11)
    tol = 5e-7
    lg = pruner.LearnedGrid(mol, basis, tol=tol)
    bad, err = lg.check(D, "b3lyp")
    fine = lg.fine_grid
    assert len(lg.grid) < len(fine)
    E0, T0 = pruner.atom_shares(mol, basis, fine, "b3lyp", D)
    E1, T1 = pruner.atom_shares(mol, basis, lg.grid, "b3lyp", D)
    # the judge runs in the tensor-core form (per-atom share error ~1e-10 Eh): an atom it kept may sit
    # above the per-atom tolerance in FP64 by at most that much
    assert np.all(np.abs(E1 - E0) <= lg.tol_atom + 2e-9)
    assert abs(E1.sum() - E0.sum()) <= tol
    assert abs(T1.sum() - T0.sum()) <= tol
