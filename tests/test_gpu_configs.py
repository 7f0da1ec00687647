"""Full-size workload checks on the GPU: the UKS flake (C54H18, PBE0) and the learned-pruned grid on
the 61-water cluster, each against the FP64 form on the Fine grid with the per-molecule tolerance
|dExc| <= 1e-6 Eh (the accuracy target of the mixed, pruned build).  Timings are printed (pytest -s)
for the record; the assertions are on accuracy and on the pruned grid being smaller."""

import time

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, VxcGroup, pruner, workloads

pytestmark = pytest.mark.gpu

EXC_TOL = 1e-6


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


def test_c54h18_uks_pbe0_mixed_against_fp64(lib):
    mol, basis, func, (Pa, Pb) = workloads.build_workload("c54h18_pbe0_uks", 7)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    eng = UksVxcEngine(basis, grid)
    e64, Va64, Vb64 = eng.evaluate(basis, grid, func, Pa, Pb, precision="fp64")
    n64 = eng.last_nelec
    t0 = time.perf_counter()
    em, Vam, Vbm = eng.evaluate(basis, grid, func, Pa, Pb, precision="mixed")
    t = time.perf_counter() - t0
    print(f"\nC54H18 UKS PBE0: {len(grid)} points, mixed build {t * 1e3:.1f} ms (host call), dExc {em - e64:.2e}")
    assert abs(em - e64) < EXC_TOL
    assert abs(eng.last_nelec[0] - n64[0]) < 1e-6 and abs(eng.last_nelec[1] - n64[1]) < 1e-6
    assert np.max(np.abs(Vam - Va64)) < 2e-6 and np.max(np.abs(Vbm - Vb64)) < 2e-6
    na, nb = mol.n_alpha_beta()
    assert abs(n64[0] - na) < 1e-2 and abs(n64[1] - nb) < 1e-2
    eng.close()


def test_water61_learned_grid_mixed_against_fp64_fine(lib):
    """183 atoms, 1159 AOs, B3LYP/6-31G(d): MLP-pruned grid, Fine-grid judge, mixed precision,
    against FP64 on the full Fine grid."""
    mol = workloads.water_cluster(61, 61)
    basis = BasisSet.from_name("6-31g(d)", mol)
    assert basis.n_ao == 1159
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    fine = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    lg = pruner.LearnedGrid(mol, basis, tol=5e-7)
    picked = lg.levels.copy()
    reverted, _ = lg.check(D, "b3lyp")
    ref = RksVxcEngine(basis, fine)
    e_ref, V_ref = ref.evaluate(basis, fine, "b3lyp", D, precision="fp64")
    eng = RksVxcEngine(basis, lg.grid, precision="mixed")
    eng.evaluate(basis, lg.grid, "b3lyp", D)
    t0 = time.perf_counter()
    e, V = eng.evaluate(basis, lg.grid, "b3lyp", D)
    t = time.perf_counter() - t0
    print(f"\n(H2O)61: Fine {len(fine)} points, learned {len(lg.grid)} ({len(lg.grid) / len(fine):.3f}), "
          f"levels {np.bincount(picked, minlength=len(pruner.LEVELS)).tolist()}, reverted {len(reverted)}, "
          f"mixed pruned build {t * 1e3:.1f} ms (host call), dExc {e - e_ref:.2e}, max|dV| {np.abs(V - V_ref).max():.2e}")
    assert len(lg.grid) < len(fine)
    assert abs(e - e_ref) < EXC_TOL
    ref.close()
    eng.close()


def test_water_clusters_64_group_graph_mixed_against_fp64(lib):
    """The 64-cluster batched workload at full size (PBE / 6-31G(d), Fine grid): one group, one
    persistent launch per build, the autotuned tile, a CUDA-graph replay; every molecule within
    |dExc| <= 1e-6 Eh of the FP64 form, and the replay equal to the host call."""
    torch = pytest.importorskip("torch")
    sizes = workloads.cluster_batch_sizes()
    members, dens = [], []
    for i, k in enumerate(sizes):
        mol = workloads.water_cluster(k, 1000 + i)
        basis = BasisSet.from_name("6-31g(d)", mol)
        grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
        members.append((basis, grid))
        dens.append(workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7 + i))
    fp64 = VxcGroup(members, precision="fp64")
    e64, n64, V64 = fp64.evaluate_rks("pbe", dens)
    fp64.close()
    grp = VxcGroup(members, precision="mixed")
    t0 = time.perf_counter()
    em, nm, Vm = grp.evaluate_rks("pbe", dens)  # tunes the tile on the first evaluation
    t = time.perf_counter() - t0
    assert grp.tile in (64, 128)
    print(f"\n64 clusters ({sum(sizes)} waters, {sum(len(g) for _, g in members)} points): tile {grp.tile}, "
          f"first mixed call {t * 1e3:.0f} ms, max |dExc| {np.max(np.abs(em - e64)):.2e}")
    assert np.max(np.abs(em - e64)) <= EXC_TOL
    assert np.max(np.abs(nm - n64)) < 1e-6
    assert max(float(np.max(np.abs(a - b))) for a, b in zip(Vm, V64)) < 2e-6
    # one graph replay of the whole build on device buffers
    dev = torch.device("cuda")
    dP = torch.from_numpy(grp.pack(dens)).to(dev)
    dV = torch.zeros(grp.packed_size, dtype=torch.float64, device=dev)
    dres = torch.zeros(3 * grp.n_mols + 1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    grp.capture_rks("pbe", dP.data_ptr(), dres.data_ptr(), dV.data_ptr())
    grp.replay(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert grp.status() == 0
    res = dres.cpu().numpy()
    assert np.array_equal(res[0:2 * grp.n_mols:2], em)
    Vg = grp.unpack(dV.cpu().numpy())
    assert max(float(np.max(np.abs(a - b))) for a, b in zip(Vg, Vm)) < 1e-12
    grp.close()