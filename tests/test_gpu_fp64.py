"""GPU parity of the plain FP64 form against the oracle (tolerances from the drop-in contract:
|dExc| <= 1e-9 Eh, max |dVxc| <= 1e-10, |dNelec| <= 1e-9)."""

import numpy as np
import pytest

from calchem_gb300 import (BasisSet, GpuVxcGrid, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, workloads)
from calchem_gb300 import _native
from tests.helpers import distorted_water, make_positive_density, oracle_basis, reference_layout

pytestmark = pytest.mark.gpu

EXC_TOL = 1e-9
V_TOL = 1e-10
N_TOL = 1e-9


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


def test_gpu_grid_matches_oracle_point_for_point(lib, oracle):
    for mol, level in [(workloads.water(), GridLevel.FINE), (distorted_water(), GridLevel.COARSE),
                       (workloads.octane(), GridLevel.FINE)]:
        g = MolecularGrid.build(mol, level)
        og = oracle.Grid.build(mol.z, mol.coords_bohr, int(level))
        xyzw, raw, host = og.points()
        assert len(g) == len(xyzw)
        assert np.array_equal(g.host_atom, host)
        # no fused multiply-add on either side: identical arithmetic, identical bits
        assert np.max(np.abs(g.xyzw - xyzw)) == 0.0
        assert np.max(np.abs(g.raw_weight - raw)) == 0.0


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"])
def test_rks_fp64_matches_oracle_distorted_water(lib, oracle, func):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    P = make_positive_density(basis.n_ao, 7)
    eng = RksVxcEngine.new_with_gpu(basis, grid, True)
    exc, V = eng.evaluate(basis, grid, func, P)
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    og = oracle.Grid.from_points(grid.xyzw)
    e_ref, n_ref, V_ref = oracle.vxc_rks_points(ob, og, P, func)
    assert abs(exc - e_ref) < EXC_TOL
    assert abs(eng.last_nelec - n_ref) < N_TOL
    assert np.max(np.abs(V - V_ref)) < V_TOL
    assert np.max(np.abs(V - V.T)) == 0.0
    k, fb = eng.telemetry()
    assert k >= 1 and fb == 0


@pytest.mark.parametrize("func", ["svwn5", "b3lyp"])
def test_rks_fp64_water_fine_seeded(lib, oracle, func):
    mol = workloads.water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), 5, 7)
    eng = RksVxcEngine.new_with_gpu(basis, grid, True)
    exc, V = eng.evaluate(basis, grid, func, D)
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    og = oracle.Grid.from_points(grid.xyzw)
    oe = oracle.RksEngine(ob, og)
    e_ref, n_ref, V_ref = oe.evaluate(D, func)
    assert abs(exc - e_ref) < EXC_TOL
    assert abs(eng.last_nelec - n_ref) < N_TOL
    assert np.max(np.abs(V - V_ref)) < V_TOL
    assert abs(eng.last_nelec - 10.0) < 1e-4  # tr(DS) = 2 n_occ up to quadrature error


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "pbe0"])
def test_uks_fp64_matches_oracle(lib, oracle, func):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    Pa = make_positive_density(basis.n_ao, 2)
    Pb = make_positive_density(basis.n_ao, 5)
    eng = UksVxcEngine.new_with_gpu(basis, grid, True)
    exc, Va, Vb = eng.evaluate(basis, grid, func, Pa, Pb)
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    og = oracle.Grid.from_points(grid.xyzw)
    e_ref, na, nb, Va_ref, Vb_ref = oracle.vxc_uks_points(ob, og, Pa, Pb, func)
    assert abs(exc - e_ref) < EXC_TOL
    assert abs(eng.last_nelec[0] - na) < N_TOL and abs(eng.last_nelec[1] - nb) < N_TOL
    assert np.max(np.abs(Va - Va_ref)) < V_TOL
    assert np.max(np.abs(Vb - Vb_ref)) < V_TOL


def test_closed_shell_uks_equals_rks(lib):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    P = make_positive_density(basis.n_ao, 1)
    r = RksVxcEngine(basis, grid)
    u = UksVxcEngine(basis, grid)
    for func in ["svwn5", "pbe", "b3lyp"]:
        er, Vr = r.evaluate(basis, grid, func, P)
        eu, Va, Vb = u.evaluate(basis, grid, func, 0.5 * P, 0.5 * P)
        assert abs(er - eu) < 1e-13
        assert np.max(np.abs(Va - Vr)) < 1e-13 and np.max(np.abs(Vb - Vr)) < 1e-13


def _reference_engine_gpu_branch(basis, grid, func, P, oracle):
    """CalChem's RksVxcEngine GPU branch (vxc.rs:728-799) driven through the drop-in C ABI:
    upload the reference layout, eval_rho, functional on the host (oracle), accum, mirror."""
    sh, pr, co = basis.gpu_arrays()
    pts, w, off, cs = reference_layout(basis, grid)
    g = GpuVxcGrid.upload(sh, pr, co, pts, off, cs, basis.n_ao)
    rg = g.eval_rho_grad(P)
    rho = rg[:, 0]
    grad = rg[:, 1:4]
    live = rho >= 1e-18
    gss = 0.25 * np.sum(grad * grad, axis=1)
    inp = np.stack([0.5 * rho, 0.5 * rho, gss, gss, gss], axis=1)
    out = oracle.eval_xc(func, inp)
    exc = float(np.sum(np.where(live, w * out[:, 0], 0.0)))
    wv = np.zeros((len(w), 4))
    wv[:, 0] = np.where(live, 0.5 * w * out[:, 1], 0.0)
    us = np.where(live, w * (out[:, 3] + 0.5 * out[:, 4]), 0.0)
    wv[:, 1:4] = us[:, None] * grad
    Vl = g.accumulate_vxc(wv)
    g.release()
    assert np.all(np.triu(Vl, 1) == 0.0)
    V = np.tril(Vl) + np.tril(Vl, -1).T
    return exc, V


def test_dropin_four_call_flow_matches_oracle(lib, oracle):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    P = make_positive_density(basis.n_ao, 7)
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    og = oracle.Grid.from_points(grid.xyzw)
    for func in ["svwn5", "pbe", "b3lyp"]:
        exc, V = _reference_engine_gpu_branch(basis, grid, func, P, oracle)
        e_ref, _, V_ref = oracle.vxc_rks_points(ob, og, P, func)
        assert abs(exc - e_ref) < 1e-12 * max(1.0, abs(e_ref)) + 1e-12
        assert np.max(np.abs(V - V_ref)) < 1e-11


def test_error_codes(lib):
    mol = workloads.water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build(mol, GridLevel.COARSE)
    n = basis.n_ao
    P = np.eye(n)
    out = np.zeros((len(grid), 4))
    # unknown id
    assert lib.calchem_cuda_vxc_eval_rho(987654321, _native.ptr(P), _native.ptr(out), len(grid), n) == -2
    # null pointers
    assert lib.calchem_cuda_vxc_eval_rho(1, None, None, len(grid), n) == -1
    eng = RksVxcEngine(basis, grid)
    V = np.zeros((n, n))
    e = np.zeros(1)
    ne = np.zeros(1)
    # unknown functional code
    assert lib.calchem_xc_evaluate_rks(eng.grid_id, 99, 0, _native.ptr(P), _native.ptr(e), _native.ptr(ne),
                                       _native.ptr(V)) == -1
    # size mismatch on the reference entry points
    assert lib.calchem_cuda_vxc_eval_rho(eng.grid_id, _native.ptr(P), _native.ptr(out), len(grid) + 1, n) == -2
    # release is idempotent
    eng.close()
    assert lib.calchem_cuda_vxc_release(eng.grid_id) == 0


def test_zero_weight_grid_gives_exact_zeros(lib):
    mol = distorted_water()
    basis = BasisSet.from_name("sto-3g", mol)
    n = basis.n_ao
    sh, pr, co = basis.gpu_arrays()
    # One point at the origin with zero weight: the batch is dropped, nothing to upload (vxc.rs:2744-2783).
    xyzw = np.array([[0.0, 0.0, 0.0, 0.0]])
    gid = 424242
    rc = lib.calchem_xc_upload_points(_native.ptr(sh), len(sh), _native.ptr(pr), len(pr), _native.ptr(co), len(co),
                                      _native.ptr(xyzw), 1, n, gid, 1 << 30)
    assert rc == -1
    # A grid with a live point but a zero-density matrix gives exactly zero Exc and V.
    xyzw = np.array([[0.1, 0.2, 0.3, 0.5]])
    from calchem_gb300.grid import MolecularGrid as MG

    g = MG(xyzw, np.array([0.5]), np.array([0]), GridLevel.COARSE)
    eng = RksVxcEngine(basis, g)
    e0, V0 = eng.evaluate(basis, g, "b3lyp", np.zeros((n, n)))
    assert e0 == 0.0 and np.all(V0 == 0.0)
