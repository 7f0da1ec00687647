"""GPU tests of the XC nuclear gradient (calchem_xc_nuclear_gradient and the drop-in
calchem_cuda_vxc_grad_force) against the oracle's restatement of xc_nuclear_gradient
(vxc.rs:1769-1912, grid.rs:423-584), and the reference's own finite-difference check
(vxc.rs:2498-2548) with GPU energies at displaced geometries."""

import numpy as np
import pytest

from calchem_gb300 import (Atom, BasisSet, GpuVxcGrid, GridLevel, MolecularGrid, Molecule, UksVxcEngine,
                           xc_nuclear_gradient)
from tests.helpers import distorted_water, make_positive_density, oracle_basis, reference_layout

pytestmark = pytest.mark.gpu

TOL = 1e-10  # |GPU - oracle| per component, Eh/Bohr (both FP64; different summation orders)


@pytest.fixture(scope="module")
def setup(native_lib, oracle):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    og = oracle.Grid.from_points(grid.xyzw, grid.host_atom, grid.raw_weight)
    return mol, basis, grid, ob, og


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "pbe0", "camb3lyp", "wb97x"])
def test_closed_shell_gradient_matches_oracle(setup, oracle, func):
    mol, basis, grid, ob, og = setup
    P = make_positive_density(basis.n_ao, 3)
    g = xc_nuclear_gradient(mol, basis, grid, func, 0.5 * P, 0.5 * P)
    ref = oracle.xc_gradient(ob, og, mol.z, mol.coords_bohr, 0.5 * P, 0.5 * P, func)
    assert np.max(np.abs(ref)) > 1e-3
    assert np.max(np.abs(g - ref)) < TOL, np.abs(g - ref).max()
    assert np.max(np.abs(g.sum(axis=0))) < 1e-12


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp", "wb97xd"])
def test_open_shell_gradient_matches_oracle(setup, oracle, func):
    mol, basis, grid, ob, og = setup
    Pa, Pb = make_positive_density(basis.n_ao, 3), make_positive_density(basis.n_ao, 8)
    g = xc_nuclear_gradient(mol, basis, grid, func, Pa, Pb)
    ref = oracle.xc_gradient(ob, og, mol.z, mol.coords_bohr, Pa, Pb, func)
    assert np.max(np.abs(g - ref)) < TOL, np.abs(g - ref).max()
    assert np.max(np.abs(g.sum(axis=0))) < 1e-12


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_gpu_gradient_matches_cpu_kat(setup, oracle, func):
    """vxc.rs:2686-2722: RKS (pa, pa) and UKS (pa seed 3, pb seed 9) GPU gradients within 1e-10 of the
    CPU gradient, with GPU kernels launched and no fallback."""
    from calchem_gb300 import xc_nuclear_gradient_with_gpu
    mol, basis, grid, ob, og = setup
    pa, pb = make_positive_density(basis.n_ao, 3), make_positive_density(basis.n_ao, 9)
    for b in (pa, pb):
        g, k, fb = xc_nuclear_gradient_with_gpu(mol, basis, grid, func, pa, b, True)
        assert k >= 1 and fb == 0
        ref = oracle.xc_gradient(ob, og, mol.z, mol.coords_bohr, pa, b, func)
        assert np.max(np.abs(g - ref)) < 1e-10


def test_gradient_is_deterministic_and_engine_form_agrees(setup):
    mol, basis, grid, _, _ = setup
    Pa, Pb = make_positive_density(basis.n_ao, 1), make_positive_density(basis.n_ao, 4)
    eng = UksVxcEngine(basis, grid)
    g1 = eng.nuclear_gradient(mol, grid, "pbe", Pa, Pb)
    g2 = eng.nuclear_gradient(mol, grid, "pbe", Pa, Pb)
    eng.close()
    assert np.array_equal(g1, g2)
    assert np.array_equal(g1, xc_nuclear_gradient(mol, basis, grid, "pbe", Pa, Pb))


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_gradient_matches_finite_differences_of_gpu_energies(setup, func):
    """vxc.rs:2498-2548: central differences of Exc(R +- h) (h = 1e-5 Bohr) with the grid and basis
    rebuilt at each displaced geometry, every component within 1e-8 of the analytic gradient."""
    mol, basis, grid, _, _ = setup
    n = basis.n_ao
    Pa, Pb = make_positive_density(n, 3), make_positive_density(n, 8)
    ana = xc_nuclear_gradient(mol, basis, grid, func, Pa, Pb)
    xyz = np.array(mol.coords_bohr)
    h = 1e-5
    for a in range(len(xyz)):
        for q in range(3):
            e = []
            for sgn in (1.0, -1.0):
                x = xyz.copy()
                x[a, q] += sgn * h
                m2 = Molecule([Atom.from_bohr(at.symbol, x[i]) for i, at in enumerate(mol.atoms)], mol.charge,
                              mol.multiplicity)
                b2 = BasisSet.from_name("6-31g(d)", m2)
                g2 = MolecularGrid.build_for_basis(m2, b2, GridLevel.COARSE)
                eng = UksVxcEngine(b2, g2)
                e.append(eng.evaluate(b2, g2, func, Pa, Pb)[0])
                eng.close()
            fd = (e[0] - e[1]) / (2 * h)
            assert abs(ana[a, q] - fd) < 1e-8, (a, q, ana[a, q], fd)


@pytest.mark.parametrize("is_rks", [True, False])
def test_dropin_grad_force_matches_oracle_ao_term(setup, oracle, is_rks):
    """The reference's GPU gradient flow (vxc.rs:2030-2333) over the drop-in ABI: eval_rho per spin,
    the functional and the coefficients w v_rho, w u on the host, then calchem_cuda_vxc_grad_force;
    its result is the AO part of the gradient."""
    mol, basis, grid, ob, og = setup
    n = basis.n_ao
    Pa = make_positive_density(n, 3)
    Pb = Pa if is_rks else make_positive_density(n, 8)
    sh, pr, co = basis.gpu_arrays()
    pts, w, off, cs = reference_layout(basis, grid)
    gg = GpuVxcGrid.upload(sh, pr, co, pts, off, cs, n)
    ra_g = gg.eval_rho_grad(Pa)
    rb_g = ra_g if is_rks else gg.eval_rho_grad(Pb)
    ra, rb = np.maximum(ra_g[:, 0], 0), np.maximum(rb_g[:, 0], 0)
    ga, gb = ra_g[:, 1:4], rb_g[:, 1:4]
    inp = np.stack([ra, rb, np.sum(ga * ga, 1), np.sum(ga * gb, 1), np.sum(gb * gb, 1)], axis=1)
    out = oracle.eval_xc("b3lyp", inp)
    live = (ra + rb >= 1e-18)[:, None]
    ua = 2 * out[:, 3:4] * ga + out[:, 4:5] * gb
    ub = 2 * out[:, 5:6] * gb + out[:, 4:5] * ga
    wxc = np.where(live, np.concatenate([out[:, 1:2], ua, out[:, 2:3], ub], axis=1) * w[:, None], 0.0)
    g = gg.eval_grad_force(Pa, Pb, is_rks, wxc, len(mol.z))
    gg.release()
    ref = oracle.xc_gradient(ob, og, mol.z, mol.coords_bohr, Pa, Pb, "b3lyp", parts=1)
    assert np.max(np.abs(g - ref)) < TOL, np.abs(g - ref).max()


def test_gradient_error_codes(setup, native_lib):
    mol, basis, grid, _, _ = setup
    eng = UksVxcEngine(basis, grid)
    bad = grid.host_atom.copy()
    bad[0] = len(mol.z)  # host atom outside [0, n_atoms): rejected before any launch
    z = np.ascontiguousarray(mol.z, dtype=np.int32)
    xyz = np.ascontiguousarray(mol.coords_bohr)
    P = make_positive_density(basis.n_ao, 1)
    out = np.zeros((len(z), 3))
    from calchem_gb300 import _native
    rc = native_lib.calchem_xc_nuclear_gradient(eng.grid_id, 1, 0, len(z), _native.ptr(z), _native.ptr(xyz),
                                                _native.ptr(grid.raw_weight), _native.ptr(bad), len(bad),
                                                _native.ptr(P), None, _native.ptr(out))
    assert rc == -1
    rc = native_lib.calchem_xc_nuclear_gradient(eng.grid_id, 1, 0, len(z), _native.ptr(z), _native.ptr(xyz),
                                                _native.ptr(grid.raw_weight), _native.ptr(grid.host_atom),
                                                len(bad) - 1, _native.ptr(P), None, _native.ptr(out))
    assert rc == -2
    eng.close()


MIXED_TOL = 1e-9  # tensor-core form vs the oracle, Eh/Bohr per component (measured ~7e-11 on water)


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp", "camb3lyp"])
def test_mixed_gradient_matches_oracle(setup, oracle, func):
    mol, basis, grid, ob, og = setup
    P = make_positive_density(basis.n_ao, 3)
    Pa, Pb = make_positive_density(basis.n_ao, 3), make_positive_density(basis.n_ao, 8)
    for pa, pb in ((0.5 * P, 0.5 * P), (Pa, Pb)):
        g = xc_nuclear_gradient(mol, basis, grid, func, pa, pb, precision="mixed")
        ref = oracle.xc_gradient(ob, og, mol.z, mol.coords_bohr, pa, pb, func)
        assert np.max(np.abs(g - ref)) < MIXED_TOL, np.abs(g - ref).max()
        assert np.max(np.abs(g.sum(axis=0))) < 1e-12


def test_mixed_gradient_octane_matches_fp64():
    """C8H18 B3LYP on the Medium grid: the tensor-core gradient within 5e-9 Eh/Bohr of the FP64 one
    (measured 5.4e-10 on the Fine grid), deterministic on repeat."""
    from calchem_gb300 import BasisSet as BS, RksVxcEngine, workloads
    mol = workloads.octane()
    basis = BS.from_name("6-31g(d,p)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.MEDIUM)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    eng = RksVxcEngine(basis, grid)
    g64 = eng.nuclear_gradient(mol, grid, "b3lyp", 0.5 * D)
    gm = eng.nuclear_gradient(mol, grid, "b3lyp", 0.5 * D, precision="mixed")
    gm2 = eng.nuclear_gradient(mol, grid, "b3lyp", 0.5 * D, precision="mixed")
    eng.close()
    assert np.max(np.abs(gm - g64)) < 5e-9, np.abs(gm - g64).max()
    assert np.array_equal(gm, gm2)


def test_mixed_gradient_long_contractions_and_many_atoms():
    """(H2O)61, 183 atoms, 1159 AOs, Coarse grid: batches of more than 1024 AOs (CalChem's batching of
    consecutive points; compact batches stay near 500) take the running-sum path of the tensor-core
    contractions, and 183 atoms exceed the shared-memory pair tables of the weight derivative (the
    per-warp scratch path).  Tensor-core vs FP64 gradient within 5e-9."""
    from calchem_gb300 import BasisSet as BS, RksVxcEngine, workloads
    mol = workloads.water_cluster(61, 61)
    basis = BS.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    eng = RksVxcEngine(basis, grid, batching="reference")
    assert eng.plan_stats()[3] > 1024
    g64 = eng.nuclear_gradient(mol, grid, "pbe", 0.5 * D)
    gm = eng.nuclear_gradient(mol, grid, "pbe", 0.5 * D, precision="mixed")
    eng.close()
    assert np.max(np.abs(gm - g64)) < 5e-9, np.abs(gm - g64).max()
    assert np.max(np.abs(gm.sum(axis=0))) < 1e-11
