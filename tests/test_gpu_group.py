"""GPU tests of multi-molecule groups (one persistent launch over many molecules) and of CUDA-graph
replay.

A group member is batched exactly as a single engine batches it and its batch partials are summed in
the same fixed order, so per-member Exc and Nelec must equal the single-engine values bit for bit;
Vxc is accumulated with atomics in a different order, so it is compared to 1e-12.
"""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, VxcGroup, workloads
from tests.helpers import distorted_water, make_positive_density

pytestmark = pytest.mark.gpu

V_TOL = 1e-12


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


def _members():
    mols = [workloads.water(), distorted_water(), workloads.water_cluster(3, 11), workloads.water_cluster(2, 5)]
    out = []
    for i, mol in enumerate(mols):
        basis = BasisSet.from_name("6-31g(d)", mol)
        grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE if i % 2 else GridLevel.FINE)
        D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 100 + i)
        out.append((mol, basis, grid, D))
    return out


@pytest.fixture(scope="module")
def members(lib):
    return _members()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("func", ["pbe", "b3lyp"])
def test_group_rks_equals_single_engines(members, precision, func):
    grp = VxcGroup([(b, g) for _, b, g, _ in members], precision=precision)
    assert grp.n_mols == len(members)
    exc, ne, Vs = grp.evaluate_rks(func, [D for *_, D in members])
    for i, (_, basis, grid, D) in enumerate(members):
        eng = RksVxcEngine(basis, grid, precision=precision)
        e1, V1 = eng.evaluate(basis, grid, func, D)
        assert exc[i] == e1
        assert ne[i] == eng.last_nelec
        assert np.max(np.abs(Vs[i] - V1)) < V_TOL
        assert np.array_equal(Vs[i], Vs[i].T)
        eng.close()
    grp.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_group_uks_equals_single_engines(members, precision):
    grp = VxcGroup([(b, g) for _, b, g, _ in members], precision=precision)
    pas = [make_positive_density(b.n_ao, 3 + i) for i, (_, b, _, _) in enumerate(members)]
    pbs = [make_positive_density(b.n_ao, 30 + i) for i, (_, b, _, _) in enumerate(members)]
    exc, ne, Vas, Vbs = grp.evaluate_uks("pbe0", pas, pbs)
    for i, (_, basis, grid, _) in enumerate(members):
        eng = UksVxcEngine(basis, grid, precision=precision)
        e1, Va, Vb = eng.evaluate(basis, grid, "pbe0", pas[i], pbs[i])
        assert exc[i] == e1
        assert tuple(ne[i]) == eng.last_nelec
        assert np.max(np.abs(Vas[i] - Va)) < V_TOL and np.max(np.abs(Vbs[i] - Vb)) < V_TOL
        eng.close()
    grp.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_direct_evaluation(members, precision):
    torch = pytest.importorskip("torch")
    grp = VxcGroup([(b, g) for _, b, g, _ in members], precision=precision)
    exc, ne, Vs = grp.evaluate_rks("pbe", [D for *_, D in members])
    dev = torch.device("cuda:0")
    d_P = torch.from_numpy(grp.pack([D for *_, D in members])).to(dev)
    d_V = torch.zeros(grp.packed_size, dtype=torch.float64, device=dev)
    d_res = torch.zeros(3 * grp.n_mols, dtype=torch.float64, device=dev)
    grp.capture_rks("pbe", d_P.data_ptr(), d_res.data_ptr(), d_V.data_ptr())
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):
        d_V.fill_(7.0)
        d_res.fill_(7.0)
        grp.replay(stream.cuda_stream)
        torch.cuda.synchronize(dev)
        assert grp.status() == 0
        res = d_res.cpu().numpy()
        V = grp.unpack(d_V.cpu().numpy())
        for i in range(grp.n_mols):
            assert res[2 * i] == exc[i] and res[2 * i + 1] == ne[i]
            assert np.max(np.abs(V[i] - Vs[i])) < V_TOL
    grp.close()


def test_group_rejects_bad_members(lib):
    import ctypes
    from calchem_gb300 import _native
    ids = (ctypes.c_uint64 * 2)(12345678, 87654321)
    assert lib.calchem_xc_group_create(ids, 2, 999999, 1 << 40) == -2  # unknown members
    assert lib.calchem_xc_group_create(None, 2, 999999, 1 << 40) == -1
    assert _native.load().calchem_xc_graph_launch(424242, None) == -2
