"""The tensor-core form's AO cache (calchem_xc_set_ao_cache): per-batch AO planes, packed operand
and row exponents kept across evaluations, as CalChem's RksVxcEngine keeps its per-batch AO cache
across SCF iterations (crates/calchem-dft/src/vxc.rs:386-394, 600-716).  The cached evaluations
must equal the uncached ones: Exc and Nelec bit for bit (fixed-order reductions), Vxc to the
rounding of its FP64 atomics.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, UksVxcEngine, VxcGroup, workloads

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def octane():
    mol = workloads.octane()
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.MEDIUM)
    D = workloads.seeded_density_rks(basis.overlap(), 33, 7)
    return mol, basis, grid, D


def test_cached_evaluations_equal_uncached(octane):
    mol, basis, grid, D = octane
    eng = RksVxcEngine(basis, grid, precision="mixed")
    assert eng.ao_cache_bytes() == 0
    e1, V1 = eng.evaluate(basis, grid, "b3lyp", D)  # fills the cache
    n1 = eng.last_nelec
    nb, _, _, _ = eng.plan_stats()
    assert eng.ao_cache_bytes() > 0
    e2, V2 = eng.evaluate(basis, grid, "b3lyp", D)  # reads it
    n2 = eng.last_nelec
    e3, V3 = eng.evaluate(basis, grid, "pbe", 0.9 * D)  # another functional and density, same AOs
    eng.set_ao_cache(False)
    assert eng.ao_cache_bytes() == 0
    e2n, V2n = eng.evaluate(basis, grid, "b3lyp", D)
    e3n, V3n = eng.evaluate(basis, grid, "pbe", 0.9 * D)
    eng.close()
    assert e1 == e2 == e2n and n1 == n2
    assert e3 == e3n
    assert np.max(np.abs(V2 - V1)) < 1e-13 and np.max(np.abs(V2 - V2n)) < 1e-13
    assert np.max(np.abs(V3 - V3n)) < 1e-13


def test_cache_serves_both_spins_and_fp64_is_unaffected(octane):
    mol, basis, grid, D = octane
    Pa, Pb = 0.55 * D, 0.45 * D
    eng = UksVxcEngine(basis, grid, precision="mixed")
    r1 = eng.evaluate(basis, grid, "pbe0", Pa, Pb)
    r2 = eng.evaluate(basis, grid, "pbe0", Pa, Pb)
    f64 = eng.evaluate(basis, grid, "pbe0", Pa, Pb, precision="fp64")
    eng.set_ao_cache(False)
    r3 = eng.evaluate(basis, grid, "pbe0", Pa, Pb)
    eng.close()
    assert r1[0] == r2[0] == r3[0]
    for k in (1, 2):
        assert np.max(np.abs(r2[k] - r3[k])) < 1e-13
    assert abs(r2[0] - f64[0]) < 1e-7


def test_group_cache(octane):
    mol, basis, grid, D = octane
    w = workloads.water_cluster(3, 5)
    bw = BasisSet.from_name("6-31g(d)", w)
    gw = MolecularGrid.build_for_basis(w, bw, GridLevel.COARSE)
    Dw = workloads.seeded_density_rks(bw.overlap(), w.nelectron() // 2, 3)
    grp = VxcGroup([(basis, grid), (bw, gw)], precision="mixed")
    a = grp.evaluate_rks("b3lyp", [D, Dw])
    assert grp.ao_cache_bytes() > 0
    b = grp.evaluate_rks("b3lyp", [D, Dw])
    grp.set_ao_cache(False)
    c = grp.evaluate_rks("b3lyp", [D, Dw])
    grp.close()
    assert np.array_equal(a[0], b[0]) and np.array_equal(b[0], c[0])
    for vb, vc in zip(b[2], c[2]):
        assert np.max(np.abs(vb - vc)) < 1e-13


def test_cache_cap_from_environment():
    """CALCHEM_MAX_AO_GRID_BYTES below the cache's size leaves it off (checked in a child process,
    since the cap is read when a grid's cache is first decided)."""
    code = (
        "import numpy as np\n"
        "from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, workloads\n"
        "mol = workloads.water_cluster(2, 1)\n"
        "b = BasisSet.from_name('6-31g(d)', mol)\n"
        "g = MolecularGrid.build_for_basis(mol, b, GridLevel.COARSE)\n"
        "D = workloads.seeded_density_rks(b.overlap(), mol.nelectron() // 2, 1)\n"
        "e = RksVxcEngine(b, g, precision='mixed')\n"
        "x = e.evaluate(b, g, 'pbe', D)[0]\n"
        "print(e.ao_cache_bytes(), repr(x))\n")
    env = dict(os.environ, CALCHEM_MAX_AO_GRID_BYTES="4096")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    nbytes, _ = out.stdout.split()[-2:]
    assert int(nbytes) == 0


def test_per_point_shares_with_cache(octane):
    """calchem_xc_evaluate_rks_points (per-point w f and w v.rho, in the caller's order) reads the
    same cache: the cached call repeats the filling call bit for bit, and both equal the call with
    the cache off."""
    from calchem_gb300 import _native
    from calchem_gb300.vxc import _xc_code
    mol, basis, grid, D = octane
    eng = RksVxcEngine(basis, grid, precision="mixed")
    lib = _native.load()

    def points():
        out = np.zeros(2 * len(grid))
        exc, ne = np.zeros(1), np.zeros(1)
        _native.check("calchem_xc_evaluate_rks_points", lib.calchem_xc_evaluate_rks_points(
            eng.grid_id, _xc_code("b3lyp"), 1, _native.ptr(np.ascontiguousarray(D)), _native.ptr(exc),
            _native.ptr(ne), _native.ptr(out)))
        return exc[0], out

    e1, p1 = points()
    assert eng.ao_cache_bytes() > 0
    e2, p2 = points()
    eng.set_ao_cache(False)
    e3, p3 = points()
    eng.close()
    assert e1 == e2 == e3
    assert np.array_equal(p1, p2) and np.array_equal(p2, p3)
    assert abs(p1[0::2].sum() - e1) < 1e-9


def test_partial_cache_equals_full_and_none(octane):
    """With the cap below the cache's size, the batches whose blocks fit (in batch order) are cached
    and the others evaluate their AOs in the CTA's slab: Exc and Nelec equal the full cache's and the
    uncached form's bit for bit, the second (reading) evaluation included; Vxc to its atomics'
    rounding."""
    mol, basis, grid, D = octane
    full = RksVxcEngine(basis, grid, precision="mixed")
    e_full, V_full = full.evaluate(basis, grid, "b3lyp", D)
    n_full = full.last_nelec
    nbytes = full.ao_cache_bytes()
    full.close()
    assert nbytes > 0
    old = os.environ.get("CALCHEM_MAX_AO_GRID_BYTES")
    os.environ["CALCHEM_MAX_AO_GRID_BYTES"] = str(nbytes // 3)
    try:
        part = RksVxcEngine(basis, grid, precision="mixed")
        e1, V1 = part.evaluate(basis, grid, "b3lyp", D)  # fills the cached batches' blocks
        pbytes = part.ao_cache_bytes()
        e2, V2 = part.evaluate(basis, grid, "b3lyp", D)  # reads them, evaluates the rest
        n2 = part.last_nelec
        part.close()
    finally:
        if old is None:
            del os.environ["CALCHEM_MAX_AO_GRID_BYTES"]
        else:
            os.environ["CALCHEM_MAX_AO_GRID_BYTES"] = old
    assert 0 < pbytes <= nbytes // 3
    none = RksVxcEngine(basis, grid, precision="mixed")
    none.set_ao_cache(False)
    e3, V3 = none.evaluate(basis, grid, "b3lyp", D)
    none.close()
    assert e1 == e2 == e_full == e3 and n2 == n_full
    assert max(np.max(np.abs(V1 - V_full)), np.max(np.abs(V2 - V_full)), np.max(np.abs(V3 - V_full))) < 1e-13
