"""Autotuner: selection and cache logic on the CPU (a fake timer), and the tuned engine on the GPU."""

import json

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, autotune, workloads


class _Grid:
    def __init__(self, n):
        self.xyzw = np.zeros((n, 4))


def test_tune_picks_fastest_and_breaks_ties_to_larger_batches():
    res = autotune.tune(None, None, "pbe", measure=lambda bp: {128: 5.0, 96: 4.0, 64: 4.0}[bp])
    assert res["batch_pts"] == 96
    assert res["ms"] == {"128": 5.0, "96": 4.0, "64": 4.0}


def test_choice_is_cached_per_signature(tmp_path, monkeypatch):
    monkeypatch.setenv("CALCHEM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    basis = BasisSet.from_name("6-31g(d)", workloads.water())
    calls = []

    def measure(bp):
        calls.append(bp)
        return {128: 3.0, 96: 2.0, 64: 2.5}[bp]

    assert autotune.choose_batch_pts(basis, _Grid(1000), "pbe", "mixed", measure=measure) == 96
    assert sorted(calls) == [64, 96, 128]
    assert autotune.choose_batch_pts(basis, _Grid(1000), "pbe", "mixed", measure=measure) == 96
    assert len(calls) == 3  # second call served from the cache
    data = json.loads((tmp_path / "tune.json").read_text())
    (key,) = data
    assert "6-31G(d)" in key or "6-31g(d)" in key.lower()
    # another functional is another workload
    autotune.choose_batch_pts(basis, _Grid(1000), "b3lyp", "mixed", measure=measure)
    assert len(calls) == 6


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
