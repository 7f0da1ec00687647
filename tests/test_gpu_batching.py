"""Spatially compact batches (calchem_xc_upload_points_spatial) against CalChem's batching of
consecutive points (vxc.rs:443-493): the same per-point contributions, so the same Exc, Nelec and
Vxc up to summation order, with far fewer AOs per batch.
"""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, workloads
from calchem_gb300 import _native
from calchem_gb300.vxc import _PRECISION, _xc_code

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def octane():
    mol = workloads.octane()
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.MEDIUM)
    D = workloads.seeded_density_rks(basis.overlap(), 33, 7)
    return mol, basis, grid, D


def _points(eng, n_pts, func, D, prec):
    lib = _native.load()
    out = np.zeros(2 * n_pts)
    exc, ne = np.zeros(1), np.zeros(1)
    P = np.ascontiguousarray(D)
    _native.check("calchem_xc_evaluate_rks_points", lib.calchem_xc_evaluate_rks_points(
        eng.grid_id, _xc_code(func), _PRECISION[prec], _native.ptr(P), _native.ptr(exc), _native.ptr(ne),
        _native.ptr(out)))
    return exc[0], out.reshape(-1, 2)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_spatial_batches_match_reference_batches(octane, prec):
    mol, basis, grid, D = octane
    ref = RksVxcEngine(basis, grid, precision=prec, batching="reference")
    sp = RksVxcEngine(basis, grid, precision=prec, batching="spatial")
    st_ref, st_sp = ref.plan_stats(), sp.plan_stats()
    assert st_sp[1] < 0.75 * st_ref[1]  # sum m^2 n: compact batches see far fewer AOs
    e_ref, V_ref = ref.evaluate(basis, grid, "b3lyp", D)
    e_sp, V_sp = sp.evaluate(basis, grid, "b3lyp", D)
    if prec == "fp64":
        assert abs(e_sp - e_ref) < 1e-10
        assert abs(sp.last_nelec - ref.last_nelec) < 1e-10
        assert np.max(np.abs(V_sp - V_ref)) < 1e-12
        # per point, in the caller's order: the same contributions up to rounding
        _, p_ref = _points(ref, len(grid), "b3lyp", D, prec)
        _, p_sp = _points(sp, len(grid), "b3lyp", D, prec)
        assert np.max(np.abs(p_sp - p_ref)) < 1e-13
    else:
        assert abs(e_sp - e_ref) < 1e-7
        assert np.max(np.abs(V_sp - V_ref)) < 2e-6
    ref.close()
    sp.close()


def test_spatial_batches_uks_and_repeatable(octane):
    mol, basis, grid, D = octane
    ref = UksVxcEngine(basis, grid, batching="reference")
    sp = UksVxcEngine(basis, grid)
    Pa, Pb = 0.55 * D, 0.45 * D
    e_ref, Va_ref, Vb_ref = ref.evaluate(basis, grid, "pbe0", Pa, Pb)
    e_sp, Va_sp, Vb_sp = sp.evaluate(basis, grid, "pbe0", Pa, Pb)
    assert abs(e_sp - e_ref) < 1e-10
    assert max(np.max(np.abs(Va_sp - Va_ref)), np.max(np.abs(Vb_sp - Vb_ref))) < 1e-12
    sp2 = UksVxcEngine(basis, grid)
    e2, Va2, Vb2 = sp2.evaluate(basis, grid, "pbe0", Pa, Pb)
    # the plan is deterministic: Exc (reduced in batch order) repeats exactly; V, accumulated with
    # FP64 atomics, to rounding
    assert e2 == e_sp
    assert max(np.max(np.abs(Va2 - Va_sp)), np.max(np.abs(Vb2 - Vb_sp))) < 1e-14
    for e in (ref, sp, sp2):
        e.close()


def test_mixed_long_contractions_reference_batching():
    """(H2O)61, 1159 AOs, Coarse grid, CalChem's batching: batches of more than 1024 AOs take the
    running-sum path of the tensor-core GEMM1 (K beyond 16 blocks of 64); mixed vs FP64."""
    mol = workloads.water_cluster(61, 61)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    eng = RksVxcEngine(basis, grid, batching="reference")
    assert eng.plan_stats()[3] > 1024
    e64, V64 = eng.evaluate(basis, grid, "b3lyp", D, precision="fp64")
    em, Vm = eng.evaluate(basis, grid, "b3lyp", D, precision="mixed")
    eng.close()
    assert abs(em - e64) < 1e-7
    assert np.max(np.abs(Vm - V64)) < 2e-6


@pytest.mark.parametrize("shape", ["one_point", "coincident", "colinear"])
def test_spatial_batches_degenerate_grids(shape):
    """Degenerate point sets (one point; 1000 coincident points; 1000 points on a line) plan and
    evaluate under compact batches as under CalChem's chunks."""
    from calchem_gb300.grid import MolecularGrid as MG
    from tests.helpers import distorted_water, make_positive_density
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    rng = np.random.default_rng(11)
    if shape == "one_point":
        xyz = np.array([[0.1, 0.2, 0.3]])
    elif shape == "coincident":
        xyz = np.tile([[0.3, -0.2, 0.5]], (1000, 1))
    else:
        xyz = np.stack([np.linspace(-3.0, 3.0, 1000), np.zeros(1000), np.zeros(1000)], axis=1)
    w = rng.uniform(0.01, 0.1, len(xyz))
    xyzw = np.concatenate([xyz, w[:, None]], axis=1)
    g = MG(xyzw, w.copy(), np.zeros(len(xyz), np.int32), GridLevel.COARSE)
    P = make_positive_density(basis.n_ao, 5)
    for prec in ("fp64", "mixed"):
        ref = RksVxcEngine(basis, g, precision=prec, batching="reference")
        sp = RksVxcEngine(basis, g, precision=prec, batching="spatial")
        e_ref, V_ref = ref.evaluate(basis, g, "pbe", P)
        e_sp, V_sp = sp.evaluate(basis, g, "pbe", P)
        ref.close()
        sp.close()
        tol_e, tol_v = (1e-11, 1e-12) if prec == "fp64" else (1e-7, 2e-6)
        assert abs(e_sp - e_ref) < tol_e * max(1.0, abs(e_ref))
        assert np.max(np.abs(V_sp - V_ref)) < tol_v


@pytest.mark.gpu
def test_value_screen_floor_changes_little_and_cuts_work(native_lib):
    """The compact plan's value screen: the exact floor (1e-17, the default) leaves out only shells
    the reference zeroes itself; the tensor-core engines' floor (1e-12) leaves out contributions below
    it, which moves Exc by far less than the mixed form's own error and cuts sum m^2 n; floors outside
    [1e-17, 1e-6] are rejected."""
    from calchem_gb300.vxc import MIXED_AO_FLOOR
    from calchem_gb300 import _native
    mol = workloads.water_cluster(8, 5)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    ref = RksVxcEngine(basis, grid, batching="reference")
    e_ref, V_ref = ref.evaluate(basis, grid, "b3lyp", D)
    ref.close()
    out = {}
    for floor in (None, MIXED_AO_FLOOR):
        for prec in ("fp64", "mixed"):
            eng = RksVxcEngine(basis, grid, precision=prec, ao_floor=floor)
            e, V = eng.evaluate(basis, grid, "b3lyp", D)
            out[(floor, prec)] = (e, V, eng.plan_stats()[1])
            eng.close()
    e0, V0, w0 = out[(None, "fp64")]
    assert abs(e0 - e_ref) < 1e-10 and np.max(np.abs(V0 - V_ref)) < 1e-12  # the exact screen
    e1, V1, w1 = out[(MIXED_AO_FLOOR, "fp64")]
    assert w1 < 0.9 * w0
    assert abs(e1 - e0) < 1e-9 and np.max(np.abs(V1 - V0)) < 1e-9
    em0, Vm0, _ = out[(None, "mixed")]
    em1, Vm1, _ = out[(MIXED_AO_FLOOR, "mixed")]
    # the mixed form sums grad rho in FP32 FMAs, whose roundings follow the set of AOs summed: V
    # moves by ~2e-8 between the floors, against its ~1e-6 agreement with FP64
    assert abs(em1 - em0) < 1e-9 and np.max(np.abs(Vm1 - Vm0)) < 1e-7
    assert RksVxcEngine(basis, grid, precision="mixed").ao_floor == MIXED_AO_FLOOR
    for bad in (1e-18, 1e-5):
        with pytest.raises(_native.CalchemXcError):
            RksVxcEngine(basis, grid, ao_floor=bad)