"""The evaluation entry point that allocates no device memory (calchem_xc_evaluate_rks_static).

It serves callers that cannot call cudaMalloc -- a framework that owns every device buffer through
its own pool, or a serving loop that must not take cudaMalloc's device-wide synchronisation in the
middle of an SCF iteration.  The caller owns all inputs and outputs (here allocated with torch, as
such a framework would); the library takes its working memory from a fixed static device array.
This file is collected last so that a run stopping at its first failure has run everything else.
"""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, MolecularGrid, RksVxcEngine, workloads
from calchem_gb300 import _native
from tests.helpers import distorted_water, make_positive_density, reference_layout

pytestmark = pytest.mark.gpu

EXC_TOL = 1e-9   # the FP64 form's tolerances (tests/test_gpu_fp64.py)
N_TOL = 1e-9
V_TOL = 1e-10


def _device(torch, arr):
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()


def _static_call(lib, torch, basis, grid, D, func_code, dV, dres):
    sh, pr, co = basis.gpu_arrays()
    pts, w, off, cs = reference_layout(basis, grid)
    nf = sh["n_funcs"]
    max_m = int(max(nf[cs[off[b]:off[b + 1]]].sum() for b in range(len(off) - 1)))
    bufs = [_device(torch, x) for x in (sh, pr, co, pts, w, off, cs, D)]
    torch.cuda.synchronize()
    rc = lib.calchem_xc_evaluate_rks_static(
        bufs[0].data_ptr(), len(sh), bufs[1].data_ptr(), len(pr), bufs[2].data_ptr(), len(co), bufs[3].data_ptr(),
        bufs[4].data_ptr(), len(pts), bufs[5].data_ptr(), bufs[6].data_ptr(), len(off) - 1, len(cs), basis.n_ao,
        max_m, func_code, bufs[7].data_ptr(), dres.data_ptr(), dV.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return rc, max_m, bufs


@pytest.mark.parametrize("case", ["distorted_water_coarse", "water_fine"])
def test_static_entry_matches_allocating_entry_twice(native_lib, case):
    torch = pytest.importorskip("torch")
    lib = native_lib
    assert lib.calchem_cuda_is_available() == 1
    if case == "distorted_water_coarse":
        mol = distorted_water()
        basis = BasisSet.from_name("6-31g(d)", mol)
        grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
        D = make_positive_density(basis.n_ao, 7)
    else:
        mol = workloads.water()
        basis = BasisSet.from_name("6-31g(d)", mol)
        grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
        D = workloads.seeded_density_rks(basis.overlap(), 5, 7)
    eng = RksVxcEngine(basis, grid)  # the existing (allocating) entry point
    e_ref, V_ref = eng.evaluate(basis, grid, "b3lyp", D)
    n_ref = eng.last_nelec
    n = basis.n_ao
    dV = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
    dres = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row: the static buffer keeps the previous call's contents
        rc, _, _ = _static_call(lib, torch, basis, grid, D, 3, dV, dres)
        assert rc == 0, f"call {call}: rc={rc}"
        torch.cuda.synchronize()
        V = dV.cpu().numpy()
        exc, nelec = dres.cpu().numpy()
        assert abs(exc - e_ref) < EXC_TOL
        assert abs(nelec - n_ref) < N_TOL
        assert np.max(np.abs(V - V_ref)) < V_TOL
        dV.fill_(float("nan"))


def _raw_call(lib, torch, arrays, n_batches, n_ao, max_m, dres, dV):
    """One call of the static entry point on the given host arrays (copied to the device first)."""
    sh, pr, co, pts, w, off, cs, D = arrays
    bufs = [_device(torch, x) for x in (sh, pr, co, pts, w, off, cs, D)]
    torch.cuda.synchronize()
    return lib.calchem_xc_evaluate_rks_static(
        bufs[0].data_ptr(), len(sh), bufs[1].data_ptr(), len(pr), bufs[2].data_ptr(), len(co), bufs[3].data_ptr(),
        bufs[4].data_ptr(), len(pts), bufs[5].data_ptr(), bufs[6].data_ptr(), n_batches, len(cs), n_ao, max_m, 3,
        bufs[7].data_ptr(), dres.data_ptr(), dV.data_ptr(), torch.cuda.current_stream().cuda_stream)


def test_static_entry_rejects_inconsistent_layouts(native_lib):
    """Each layout error the device-side checks catch returns -2 (the allocating upload rejects the
    same inputs on the host), and a valid call right after each rejected one still matches the
    allocating entry point."""
    torch = pytest.importorskip("torch")
    lib = native_lib
    mol = distorted_water()
    basis = BasisSet.from_name("sto-3g", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    D = make_positive_density(basis.n_ao, 3)
    eng = RksVxcEngine(basis, grid)
    e_ref, V_ref = eng.evaluate(basis, grid, "b3lyp", D)
    eng.close()
    sh, pr, co = basis.gpu_arrays()
    pts, w, off, cs = reference_layout(basis, grid)
    nb = len(off) - 1
    nf = sh["n_funcs"]
    max_m = int(max(nf[cs[off[b]:off[b + 1]]].sum() for b in range(nb)))
    assert nb >= 3 and np.all(np.bincount(pts["batch_id"])[:2] > 64)
    n = basis.n_ao
    dV = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    dres = torch.zeros(2, dtype=torch.float64, device="cuda")

    def bad(kind):
        p, c, o, mm = pts.copy(), cs.copy(), off.copy(), max_m
        if kind == "batch_over_128_points":  # the first two batches' points under one id
            p["batch_id"][p["batch_id"] == 1] = 0
        elif kind == "unsorted_batch_ids":  # two points of different batches swap ids
            i0, i1 = int(np.argmax(p["batch_id"] == 0)), int(np.argmax(p["batch_id"] == 1))
            p["batch_id"][i0], p["batch_id"][i1] = 1, 0
        elif kind == "batch_id_out_of_range":
            p["batch_id"][-1] = nb
        elif kind == "negative_batch_id":
            p["batch_id"][0] = -1
        elif kind == "shell_index_out_of_range":
            c[0] = len(sh)
        elif kind == "decreasing_candidate_offsets":
            o[1], o[2] = o[2], o[1]
        elif kind == "batch_over_max_ao":
            mm = max_m - 1
        return (sh, pr, co, p, w, o, c, D), mm

    kinds = ["batch_over_128_points", "unsorted_batch_ids", "batch_id_out_of_range", "negative_batch_id",
             "shell_index_out_of_range", "decreasing_candidate_offsets", "batch_over_max_ao"]
    for kind in kinds:
        arrays, mm = bad(kind)
        assert _raw_call(lib, torch, arrays, nb, n, mm, dres, dV) == -2, kind
        dV.fill_(float("nan"))
        assert _raw_call(lib, torch, (sh, pr, co, pts, w, off, cs, D), nb, n, max_m, dres, dV) == 0, kind
        torch.cuda.synchronize()
        exc, _ = dres.cpu().numpy()
        assert abs(exc - e_ref) < EXC_TOL, kind
        assert np.max(np.abs(dV.cpu().numpy() - V_ref)) < V_TOL, kind


def test_static_entry_matches_oracle(native_lib, oracle):
    """The allocation-free form against the CPU restatement of CalChem's per-point path on the
    reference's distorted-water case."""
    torch = pytest.importorskip("torch")
    lib = native_lib
    mol = distorted_water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.COARSE)
    D = make_positive_density(basis.n_ao, 11)
    n = basis.n_ao
    dV = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    dres = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc, _, _ = _static_call(lib, torch, basis, grid, D, 3, dV, dres)
    assert rc == 0
    torch.cuda.synchronize()
    exc, nelec = dres.cpu().numpy()
    ob = oracle.Basis.from_name("6-31g(d)", [a.symbol for a in mol.atoms], mol.coords_bohr)
    e_or, n_or, V_or = oracle.vxc_rks_points(ob, oracle.Grid.from_points(grid.xyzw), D, "b3lyp")
    assert abs(exc - e_or) < EXC_TOL
    assert abs(nelec - n_or) < N_TOL
    assert np.max(np.abs(dV.cpu().numpy() - V_or)) < V_TOL


def test_static_entry_rejects_oversized_requests(native_lib):
    torch = pytest.importorskip("torch")
    lib = native_lib
    mol = distorted_water()
    basis = BasisSet.from_name("sto-3g", mol)
    grid = MolecularGrid.build(mol, GridLevel.COARSE)
    sh, pr, co = basis.gpu_arrays()
    pts, w, off, cs = reference_layout(basis, grid)
    bufs = [_device(torch, x) for x in (sh, pr, co, pts, w, off, cs, np.eye(basis.n_ao))]
    dV = torch.zeros((basis.n_ao, basis.n_ao), dtype=torch.float64, device="cuda")
    dres = torch.zeros(2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    # one CTA's working set for 40000 AOs per batch exceeds the 96 MiB buffer: rejected before any launch
    rc = lib.calchem_xc_evaluate_rks_static(
        bufs[0].data_ptr(), len(sh), bufs[1].data_ptr(), len(pr), bufs[2].data_ptr(), len(co), bufs[3].data_ptr(),
        bufs[4].data_ptr(), len(pts), bufs[5].data_ptr(), bufs[6].data_ptr(), len(off) - 1, len(cs), basis.n_ao,
        40000, 3, bufs[7].data_ptr(), dres.data_ptr(), dV.data_ptr(), 0)
    assert rc == -3
    assert lib.calchem_xc_evaluate_rks_static(None, 0, None, 0, None, 0, None, None, 0, None, None, 0, 0, 0, 0, 3,
                                              None, None, None, None) == -1
