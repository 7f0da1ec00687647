"""Autotuner: selection and cache logic on the CPU (a fake timer), and the tuned engine on the GPU."""

import json

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, autotune, workloads


class _Grid:
    def __init__(self, n):
        self.xyzw = np.zeros((n, 4))


def test_tune_picks_fastest_and_breaks_ties_to_larger_batches():
    res = autotune.tune(None, None, "pbe", measure=lambda bp, t: {128: 5.0, 96: 4.0, 64: 4.0}[bp])
    assert res["batch_pts"] == 96 and res["tile_n"] == 64
    assert res["ms"] == {"128/64": 5.0, "96/64": 4.0, "64/64": 4.0}


def test_tune_searches_tiles_for_the_tensor_core_form():
    ms = {(128, 64): 5.0, (128, 128): 3.0, (96, 64): 4.0, (96, 128): 3.0, (64, 64): 6.0, (64, 128): 3.5}
    res = autotune.tune(None, None, "pbe", "mixed", measure=lambda bp, t: ms[(bp, t)])
    assert (res["batch_pts"], res["tile_n"]) == (128, 128)  # tie at 3.0 goes to the larger batch
    assert len(res["ms"]) == 6
    # a tie between tiles goes to the narrow one (two CTAs per SM)
    res = autotune.tune(None, None, "pbe", "mixed", candidates=(128,), measure=lambda bp, t: 1.0)
    assert res["tile_n"] == 64


def test_tile_choice_is_cached(tmp_path, monkeypatch):
    monkeypatch.setenv("CALCHEM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    calls = []

    def measure():
        calls.append(1)
        return {64: 2.0, 128: 1.5}

    assert autotune.choose_tile("k", measure) == 128
    assert autotune.choose_tile("k", measure) == 128
    assert len(calls) == 1
    assert autotune.choose_tile("k2", lambda: {64: 1.0, 128: 1.0}) == 64
    data = json.loads((tmp_path / "tune.json").read_text())
    assert data["k|tile"]["tile_n"] == 128 and data["k2|tile"]["tile_n"] == 64


def test_choice_is_cached_per_signature(tmp_path, monkeypatch):
    monkeypatch.setenv("CALCHEM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    basis = BasisSet.from_name("6-31g(d)", workloads.water())
    calls = []

    def measure(bp, tile):
        calls.append((bp, tile))
        return {128: 3.0, 96: 2.0, 64: 2.5}[bp] + (0.1 if tile == 64 else 0.0)

    assert autotune.choose_plan(basis, _Grid(1000), "pbe", "mixed", measure=measure) == {"batch_pts": 96,
                                                                                          "tile_n": 128}
    assert sorted(calls) == [(64, 64), (64, 128), (96, 64), (96, 128), (128, 64), (128, 128)]
    assert autotune.choose_batch_pts(basis, _Grid(1000), "pbe", "mixed", measure=measure) == 96
    assert len(calls) == 6  # second call served from the cache
    data = json.loads((tmp_path / "tune.json").read_text())
    (key,) = data
    assert "6-31G(d)" in key or "6-31g(d)" in key.lower()
    # another functional is another workload
    autotune.choose_batch_pts(basis, _Grid(1000), "b3lyp", "mixed", measure=measure)
    assert len(calls) == 12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_size_changes_speed_not_results(native_lib, tmp_path, monkeypatch, precision):
    monkeypatch.setenv("CALCHEM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    mol = workloads.water_cluster(4, 3)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    ref = None
    for bp in autotune.CANDIDATES:
        eng = RksVxcEngine(basis, grid, precision=precision, batch_pts=bp)
        e, V = eng.evaluate(basis, grid, "pbe", D)
        if ref is None:
            ref = (e, eng.last_nelec, V)
        else:
            tol = 1e-10 if precision == "fp64" else 1e-7
            assert abs(e - ref[0]) < tol and abs(eng.last_nelec - ref[1]) < tol
            assert np.max(np.abs(V - ref[2])) < (1e-12 if precision == "fp64" else 2e-6)
        eng.close()
    tuned = RksVxcEngine(basis, grid, precision=precision, batch_pts="auto", func="pbe")
    assert tuned.batch_pts in autotune.CANDIDATES
    e, V = tuned.evaluate(basis, grid, "pbe", D)
    assert abs(e - ref[0]) < 1e-7
    tuned.close()


@pytest.mark.gpu
def test_tile_changes_speed_not_results(native_lib, tmp_path, monkeypatch):
    """Both GEMM1 tiles accumulate the same products in the same order: Exc and Nelec are equal bit
    for bit, Vxc up to the order of its atomics; batches of more than 128 AOs included, closed and
    open shell, a single grid and a group."""
    from calchem_gb300 import UksVxcEngine, VxcGroup
    monkeypatch.setenv("CALCHEM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    mol = workloads.water_cluster(8, 5)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    D = workloads.seeded_density_rks(basis.overlap(), mol.nelectron() // 2, 7)
    res = {}
    for tile in autotune.TILES:
        eng = RksVxcEngine(basis, grid, precision="mixed", tile=tile, ao_floor=None)  # keeps batches > 128 AOs
        assert eng.plan_stats()[3] > 128
        for _ in range(2):  # the second evaluation reads the AO cache
            e, V = eng.evaluate(basis, grid, "b3lyp", D)
        res[tile] = (e, eng.last_nelec, V)
        assert native_lib.calchem_xc_get_tile(eng.grid_id) == tile
        eng.close()
    assert res[64][0] == res[128][0] and res[64][1] == res[128][1]
    assert np.max(np.abs(res[64][2] - res[128][2])) < 1e-12
    Pa, Pb = workloads.seeded_density_uks(basis.overlap(), 41, 39, 3, 4)
    out = {}
    for tile in autotune.TILES:
        eng = UksVxcEngine(basis, grid, precision="mixed", tile=tile, ao_floor=None)
        out[tile] = eng.evaluate(basis, grid, "pbe0", Pa, Pb)
        eng.close()
    assert out[64][0] == out[128][0]
    assert max(np.max(np.abs(a - b)) for a, b in zip(out[64][1:], out[128][1:])) < 1e-12
    # the default engine tunes the tile on its first tensor-core evaluation and keeps the result
    auto = RksVxcEngine(basis, grid, precision="mixed", ao_floor=None)
    assert auto.tile is None
    e, V = auto.evaluate(basis, grid, "b3lyp", D)
    assert auto.tile in autotune.TILES and e == res[64][0]
    auto.close()
    grp = {}
    for tile in autotune.TILES:
        g = VxcGroup([(basis, grid), (basis, grid)], precision="mixed", tile=tile, ao_floor=None)
        grp[tile] = g.evaluate_rks("b3lyp", [D, D])
        g.close()
    assert np.array_equal(grp[64][0], grp[128][0]) and grp[64][0][0] == res[64][0]
    with pytest.raises(Exception):
        RksVxcEngine(basis, grid, precision="mixed", tile=96)