"""CPU tests of the batch plan (calchem_xc_plan_points, the host step of both uploads).

batching "reference" must reproduce CalChem's upload layout exactly (RksVxcEngine::new_with_gpu,
crates/calchem-dft/src/vxc.rs:443-596, restated in tests/helpers.reference_layout): the same
128-point chunks, kept points, candidate shells and batch ids.  batching "spatial" reorders the kept
points into compact batches; it must give every point at least the shells that reach it (the
kernels' exact-zero test r^2 > r2_cutoff), keep only shells that reach a point of the batch, and be
a deterministic function of its inputs.
"""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, _native, plan_points, workloads
from calchem_gb300._native import CalchemXcError
from tests.helpers import distorted_water, reference_layout


class _Points:
    def __init__(self, xyzw):
        self.xyzw = xyzw


@pytest.fixture(scope="module", params=["water", "octane"])
def case(request, oracle):
    if request.param == "water":
        mol, bn = distorted_water(), "6-31g(d)"
    else:
        mol, bn = workloads.octane(), "6-31g(d,p)"
    basis = BasisSet.from_name(bn, mol)
    xyzw, _, _ = oracle.Grid.build([a.z for a in mol.atoms], mol.coords_bohr, "fine").points()
    return request.param, basis, xyzw


def _reach(basis, xyz):
    """reach[k, s]: shell s is nonzero at point k (|r - C_s|^2 <= r2_cutoff_s)."""
    sh, _, _ = basis.gpu_arrays()
    d2 = ((xyz[:, None, :] - sh["center"][None, :, :]) ** 2).sum(-1)
    return d2 <= sh["r2_cutoff"][None, :]


def _m2n(basis, plan):
    sh, _, _ = basis.gpu_arrays()
    off, cand = plan["cand_offsets"], plan["cand_shells"]
    m = np.array([sh["n_funcs"][cand[off[b]:off[b + 1]]].sum() for b in range(len(off) - 1)], dtype=np.float64)
    n = np.bincount(plan["batch_of"], minlength=len(m))
    return float((m * m * n).sum()), int(m.max())


def test_reference_batching_is_calchems_layout(case):
    _, basis, xyzw = case
    plan = plan_points(basis, xyzw, batching="reference")
    pts, w, off, cs = reference_layout(basis, _Points(xyzw))
    assert np.array_equal(plan["cand_offsets"], off)
    assert np.array_equal(plan["cand_shells"], cs)
    assert np.array_equal(plan["batch_of"], pts["batch_id"])
    assert np.array_equal(xyzw[plan["order"], 3], w)
    assert np.array_equal(xyzw[plan["order"], 0], pts["x"])
    assert (plan["sum_m2n"], plan["max_m"]) == _m2n(basis, plan)


@pytest.mark.parametrize("batch_pts", [128, 64])
def test_spatial_batches_cover_every_reaching_shell(case, batch_pts):
    name, basis, xyzw = case
    ref = plan_points(basis, xyzw, batch_pts, batching="reference")
    sp = plan_points(basis, xyzw, batch_pts, batching="spatial")
    order, bof, off, cand = sp["order"], sp["batch_of"], sp["cand_offsets"], sp["cand_shells"]
    nb = len(off) - 1
    # a permutation of kept points, batches contiguous and at most batch_pts points
    assert len(np.unique(order)) == len(order)
    assert np.all(np.diff(bof) >= 0) and bof[0] == 0 and bof[-1] == nb - 1
    assert np.bincount(bof).max() <= batch_pts
    assert np.all(np.abs(xyzw[order, 3]) >= 1e-24)
    # points CalChem keeps and the spatial plan drops are reached by no shell
    dropped = np.setdiff1d(ref["order"], order)
    if len(dropped):
        assert not _reach(basis, xyzw[dropped, :3]).any()
    assert len(np.setdiff1d(order, ref["order"])) == 0
    # every shell that reaches a point is among its batch's candidates, and every candidate reaches
    # some point of its batch (within the 1e-6 relative margin of the planner's test)
    sh, _, _ = basis.gpu_arrays()
    member = np.zeros((nb, len(sh)), bool)
    for b in range(nb):
        member[b, cand[off[b]:off[b + 1]]] = True
    step = 20000
    hit = np.zeros((nb, len(sh)), bool)
    for k0 in range(0, len(order), step):
        xyz = xyzw[order[k0:k0 + step], :3]
        r = _reach(basis, xyz)
        assert not (r & ~member[bof[k0:k0 + step]]).any()
        d2 = ((xyz[:, None, :] - sh["center"][None, :, :]) ** 2).sum(-1)
        near = d2 <= sh["r2_cutoff"][None, :] * (1.0 + 1e-6)
        np.logical_or.at(hit, bof[k0:k0 + step], near)
    assert not (member & ~hit).any()
    assert (sp["sum_m2n"], sp["max_m"]) == _m2n(basis, sp)
    if name == "octane":
        assert sp["sum_m2n"] < 0.6 * ref["sum_m2n"]


def test_spatial_plan_is_deterministic(case):
    _, basis, xyzw = case
    a = plan_points(basis, xyzw)
    b = plan_points(basis, xyzw)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_ragged_and_degenerate_point_sets():
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    rng = np.random.default_rng(5)
    # 1000 points, a third with zero weight, 300 on one spot, 7 far outside every shell
    xyz = rng.normal(scale=2.0, size=(1000, 3))
    xyz[100:400] = xyz[100]
    xyz[-7:] = 1e3
    w = rng.uniform(0.1, 1.0, 1000)
    w[::3] = 0.0
    xyzw = np.ascontiguousarray(np.column_stack([xyz, w]))
    live = np.where(w != 0.0)[0]
    reached = live[_reach(basis, xyz[live]).any(axis=1)]
    assert 0 < len(reached) < len(live)
    for batching in ("reference", "spatial"):
        p = plan_points(basis, xyzw, 128, batching)
        # no zero-weight point, every point that an AO reaches, batches of at most 128 points
        assert len(np.setdiff1d(p["order"], live)) == 0
        assert len(np.setdiff1d(reached, p["order"])) == 0
        assert np.bincount(p["batch_of"]).max() <= 128
    sp = plan_points(basis, xyzw, 128, "spatial")
    assert all(np.array_equal(sp[k], plan_points(basis, xyzw, 128, "spatial")[k]) for k in sp)
    # every weight zero: no batch and no point in either plan (the uploads then refuse the grid)
    xyzw[:, 3] = 0.0
    for batching in ("reference", "spatial"):
        p = plan_points(basis, xyzw, 128, batching)
        assert len(p["order"]) == 0 and list(p["cand_offsets"]) == [0] and p["max_m"] == 0


def test_argument_checks(native_lib):
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    sh, _, _ = basis.gpu_arrays()
    xyzw = np.ascontiguousarray(np.column_stack([np.zeros((4, 3)), np.ones(4)]))
    f = native_lib.calchem_xc_plan_points
    p = _native.ptr
    nb = np.zeros(1, np.int32)
    assert f(p(sh), len(sh), p(xyzw), 4, 8, 1, p(nb), None, None, None, None, None, None, None, None, 0) == -1
    assert f(p(sh), len(sh), p(xyzw), 4, 256, 1, p(nb), None, None, None, None, None, None, None, None, 0) == -1
    assert f(p(sh), len(sh), p(xyzw), 0, 128, 1, p(nb), None, None, None, None, None, None, None, None, 0) == -1
    assert f(None, len(sh), p(xyzw), 4, 128, 1, p(nb), None, None, None, None, None, None, None, None, 0) == -1
    cand = np.zeros(1, np.int32)
    assert f(p(sh), len(sh), p(xyzw), 4, 128, 0, p(nb), None, None, None, None, None, None, None, p(cand), 1) == -2
    assert f(p(sh), len(sh), p(xyzw), 4, 128, 0, p(nb), None, None, None, None, None, None, None, None, 0) == 0
    assert nb[0] == 1
    with pytest.raises(ValueError):
        plan_points(basis, xyzw, batching="chunks")
    with pytest.raises(CalchemXcError):
        plan_points(basis, xyzw, batch_pts=8)
