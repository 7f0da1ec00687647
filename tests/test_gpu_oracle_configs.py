"""The FP64 drop-in against the oracle on the benchmark configurations.

The drop-in contract holds the plain FP64 form to the reference's FP64 path within 1e-9 Eh on Exc
and 1e-10 on every Vxc element (the reference's own GPU-vs-CPU bound is tighter still,
crates/calchem-dft/src/vxc.rs:2624-2641).  The oracle restates that path on the CPU, so these tests
compare the two on the same points:

* octane C8H18, B3LYP / 6-31G(d,p), Fine grid: every point (the oracle's cached-AO path);
* C54H18 UKS PBE0 / 6-31G(d) and (H2O)61 B3LYP / 6-31G(d): a seeded sample of 200 of CalChem's
  128-point chunks of the Fine grid, the GPU form on exactly those points against the oracle on the
  same points (the full grids take the CPU minutes);
* the 64 water clusters (PBE / 6-31G(d), Fine grid): four seeded clusters of eight waters or fewer,
  evaluated as one multi-molecule group, each member against the oracle on its own grid.

Nelec is compared wherever Exc is, and on the full grids its closeness to the electron count
(tr(D S) = 2 n_occ for the seeded densities) is checked as well.
"""

import numpy as np
import pytest

from calchem_gb300 import (BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, VxcGroup, workloads)
from calchem_gb300.vxc import plan_points
from tests.helpers import oracle_basis

pytestmark = pytest.mark.gpu

EXC_TOL = 1e-9
V_TOL = 1e-10
N_TOL = 1e-9
SAMPLE_BATCHES = 200


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


def sampled_subgrid(basis, grid, n_batches, seed):
    """The points of n_batches seeded chunks of CalChem's batching (vxc.rs:443-493) of the grid, as a
    grid of their own (same coordinates, weights and host atoms)."""
    plan = plan_points(basis, grid.xyzw, 128, "reference")
    nb = len(plan["cand_offsets"]) - 1
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = np.sort(rng.choice(nb, size=min(n_batches, nb), replace=False))
    sel = plan["order"][np.isin(plan["batch_of"], pick)]
    sub = MolecularGrid(grid.xyzw[sel], grid.raw_weight[sel], grid.host_atom[sel], grid.level)
    return sub, len(pick)


def test_octane_b3lyp_fine_fp64_matches_oracle_on_every_point(lib, oracle):
    mol, basis, func, (D,) = workloads.build_workload("octane_b3lyp", 7)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    ob = oracle_basis(oracle, "6-31g(d,p)", mol)
    oe = oracle.RksEngine(ob, oracle.Grid.from_points(grid.xyzw))
    e_ref, n_ref, V_ref = oe.evaluate(D, func)
    for batching in ("reference", "spatial"):
        eng = RksVxcEngine(basis, grid, batching=batching)
        exc, V = eng.evaluate(basis, grid, func, D)
        assert abs(exc - e_ref) < EXC_TOL, batching
        assert abs(eng.last_nelec - n_ref) < N_TOL, batching
        assert np.max(np.abs(V - V_ref)) < V_TOL, batching
        eng.close()
    assert abs(n_ref - mol.nelectron()) < 5e-3


def test_c54h18_uks_pbe0_fp64_matches_oracle_on_sampled_chunks(lib, oracle):
    mol, basis, func, (Pa, Pb) = workloads.build_workload("c54h18_pbe0_uks", 7)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    sub, nb = sampled_subgrid(basis, grid, SAMPLE_BATCHES, 31)
    assert nb == SAMPLE_BATCHES
    eng = UksVxcEngine(basis, sub)
    exc, Va, Vb = eng.evaluate(basis, sub, func, Pa, Pb)
    na, nb_ = eng.last_nelec
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    e_ref, na_ref, nb_ref, Va_ref, Vb_ref = oracle.vxc_uks_points(ob, oracle.Grid.from_points(sub.xyzw), Pa, Pb, func)
    assert abs(exc - e_ref) < EXC_TOL
    assert abs(na - na_ref) < N_TOL and abs(nb_ - nb_ref) < N_TOL
    assert np.max(np.abs(Va - Va_ref)) < V_TOL
    assert np.max(np.abs(Vb - Vb_ref)) < V_TOL
    eng.close()
    # the full grid: the electron counts of the seeded spin densities (n_alpha 172, n_beta 170)
    full = UksVxcEngine(basis, grid)
    full.evaluate(basis, grid, func, Pa, Pb)
    n_alpha, n_beta = mol.n_alpha_beta()
    assert abs(full.last_nelec[0] - n_alpha) < 5e-3 and abs(full.last_nelec[1] - n_beta) < 5e-3
    full.close()


def test_water61_b3lyp_fp64_matches_oracle_on_sampled_chunks(lib, oracle):
    mol = workloads.water_cluster(61, 61)
    basis = BasisSet.from_name("6-31g(d)", mol)
    assert basis.n_ao == 1159
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    sub, nb = sampled_subgrid(basis, grid, SAMPLE_BATCHES, 61)
    assert nb == SAMPLE_BATCHES
    ob = oracle_basis(oracle, "6-31g(d)", mol)
    oe = oracle.RksEngine(ob, oracle.Grid.from_points(sub.xyzw))
    e_ref, n_ref, V_ref = oe.evaluate(D, "b3lyp")
    for batching in ("reference", "spatial"):
        eng = RksVxcEngine(basis, sub, batching=batching)
        exc, V = eng.evaluate(basis, sub, "b3lyp", D)
        assert abs(exc - e_ref) < EXC_TOL, batching
        assert abs(eng.last_nelec - n_ref) < N_TOL, batching
        assert np.max(np.abs(V - V_ref)) < V_TOL, batching
        eng.close()
    full = RksVxcEngine(basis, grid)
    full.evaluate(basis, grid, "b3lyp", D)
    assert abs(full.last_nelec - mol.nelectron()) < 5e-3
    full.close()


def test_water_clusters_group_fp64_matches_oracle(lib, oracle):
    """Four seeded clusters (of those with at most eight waters) of the 64-cluster workload, as one
    group launch; each member against the oracle's cached-AO path on its Fine grid."""
    sizes = workloads.cluster_batch_sizes()
    small = [i for i, k in enumerate(sizes) if k <= 8]
    rng = np.random.Generator(np.random.PCG64(2))
    pick = sorted(rng.choice(small, size=4, replace=False).tolist())
    members, dens, mols = [], [], []
    for i in pick:
        mol = workloads.water_cluster(sizes[i], 1000 + i)
        basis = BasisSet.from_name("6-31g(d)", mol)
        grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
        members.append((basis, grid))
        dens.append(workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7 + i))
        mols.append(mol)
    grp = VxcGroup(members, precision="fp64")
    exc, ne, Vs = grp.evaluate_rks("pbe", dens)
    for k, (mol, (basis, grid), D) in enumerate(zip(mols, members, dens)):
        ob = oracle_basis(oracle, "6-31g(d)", mol)
        oe = oracle.RksEngine(ob, oracle.Grid.from_points(grid.xyzw), cap_bytes=8e9)
        e_ref, n_ref, V_ref = oe.evaluate(D, "pbe")
        assert abs(exc[k] - e_ref) < EXC_TOL, pick[k]
        assert abs(ne[k] - n_ref) < N_TOL, pick[k]
        assert np.max(np.abs(Vs[k] - V_ref)) < V_TOL, pick[k]
        assert abs(n_ref - mol.nelectron()) < 5e-3
    grp.close()
