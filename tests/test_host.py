"""CPU tests of the product's host side and C ABI (no GPU calls beyond availability checks)."""

import os
import re

import numpy as np
import pytest

from calchem_gb300 import BasisSet, GridLevel, XcFunctional, workloads
from calchem_gb300 import _native
from calchem_gb300.basis import canonical_name
from tests.helpers import oracle_basis

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "calchem_xc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(calchem_\w+)\s*\(", src)))


def test_library_exports_every_header_symbol(native_lib):
    names = header_functions()
    assert len(names) >= 19
    for name in names:
        assert hasattr(native_lib, name), name
    assert set(names) == set(_native.SIGNATURES), "ctypes signature table out of sync with the header"


def test_struct_layouts_match_reference_repr_c():
    # crates/calchem-cuda/src/lib.rs:46-84 (#[repr(C)]): 56 / 16 / 24 / 32 bytes
    assert _native.AO_SHELL.itemsize == 56
    assert _native.AO_SHELL.fields["ao_offset"][1] == 32
    assert _native.AO_PRIM.itemsize == 16
    assert _native.AO_COMP.itemsize == 24
    assert _native.GRID_PT.itemsize == 32
    assert _native.GRID_PT.fields["batch_id"][1] == 24


def test_no_device_means_error_codes_not_fallback(native_lib):
    if native_lib.calchem_cuda_is_available() == 1:
        pytest.skip("a GPU is present")
    P = np.eye(4)
    out = np.zeros((8, 4))
    assert native_lib.calchem_cuda_vxc_eval_rho(1, _native.ptr(P), _native.ptr(out), 8, 4) == -3
    assert native_lib.calchem_cuda_vxc_eval_rho(1, None, None, 8, 4) == -1
    assert native_lib.calchem_cuda_vxc_release(0) == 0
    z = np.array([8], np.int32)
    xyz = np.zeros(3)
    n = np.zeros(1, np.int32)
    assert native_lib.calchem_xc_grid_build(1, _native.ptr(z), _native.ptr(xyz), 2, 0, 5, _native.ptr(n)) == -3
    assert native_lib.calchem_xc_grid_build(1, _native.ptr(z), _native.ptr(xyz), 9, 0, 5, _native.ptr(n)) == -1
    # the XC gradient entry points: argument checks first, then "no device"
    g = np.zeros((1, 3))
    raw = np.ones(8)
    host = np.zeros(8, np.int32)
    assert native_lib.calchem_xc_nuclear_gradient(1, 3, 0, 1, _native.ptr(z), _native.ptr(xyz), _native.ptr(raw),
                                                  _native.ptr(host), 8, _native.ptr(P), None, _native.ptr(g)) == -3
    assert native_lib.calchem_xc_nuclear_gradient(1, 3, 2, 1, _native.ptr(z), _native.ptr(xyz), _native.ptr(raw),
                                                  _native.ptr(host), 8, _native.ptr(P), None, _native.ptr(g)) == -1
    assert native_lib.calchem_xc_nuclear_gradient(1, 99, 0, 1, _native.ptr(z), _native.ptr(xyz), _native.ptr(raw),
                                                  _native.ptr(host), 8, _native.ptr(P), None, _native.ptr(g)) == -1
    wxc = np.zeros((8, 8))
    assert native_lib.calchem_cuda_vxc_grad_force(1, _native.ptr(P), None, 1, _native.ptr(wxc), _native.ptr(g), 8, 4,
                                                  1, 0) == -3
    assert native_lib.calchem_cuda_vxc_grad_force(1, _native.ptr(P), None, 0, _native.ptr(wxc), _native.ptr(g), 8, 4,
                                                  1, 0) == -1
    # the device point functional: argument checks, then "no device"
    x = np.ones(4)
    f3 = np.empty(12)
    assert native_lib.calchem_xc_eval_closed_shell(3, 1, 4, _native.ptr(x), _native.ptr(x), _native.ptr(f3)) == -3
    assert native_lib.calchem_xc_eval_closed_shell(9, 0, 4, _native.ptr(x), _native.ptr(x), _native.ptr(f3)) == -1
    assert native_lib.calchem_xc_eval_closed_shell(3, 2, 4, _native.ptr(x), _native.ptr(x), _native.ptr(f3)) == -1
    assert native_lib.calchem_xc_eval_closed_shell(3, 0, 0, _native.ptr(x), _native.ptr(x), _native.ptr(f3)) == -1


def test_spatial_upload_argument_checks(native_lib):
    """calchem_xc_upload_points_spatial checks its arguments and plans before touching a device: a
    grid whose only point has zero weight leaves nothing to upload (-1, as the reference drops the
    chunk, vxc.rs:2744-2783), and batch sizes outside 16..128 are rejected."""
    from tests.helpers import distorted_water
    basis = BasisSet.from_name("sto-3g", distorted_water())
    sh, pr, co = basis.gpu_arrays()
    args = (_native.ptr(sh), len(sh), _native.ptr(pr), len(pr), _native.ptr(co), len(co))
    zero = np.array([[0.0, 0.0, 0.0, 0.0]])
    assert native_lib.calchem_xc_upload_points_spatial(*args, _native.ptr(zero), 1, basis.n_ao, 128, 7, 1 << 30) == -1
    one = np.array([[0.1, 0.2, 0.3, 0.5]])
    assert native_lib.calchem_xc_upload_points_spatial(*args, _native.ptr(one), 1, basis.n_ao, 8, 7, 1 << 30) == -1
    assert native_lib.calchem_xc_upload_points_spatial(*args, _native.ptr(one), 1, basis.n_ao, 256, 7, 1 << 30) == -1
    assert native_lib.calchem_xc_upload_points_spatial(*args, _native.ptr(one), 1, basis.n_ao, 128, 0, 1 << 30) == -1


def test_gradient_has_no_cpu_path():
    from calchem_gb300 import xc_nuclear_gradient_with_gpu
    from tests.helpers import distorted_water
    mol = distorted_water()
    with pytest.raises(NotImplementedError):
        xc_nuclear_gradient_with_gpu(mol, None, None, "pbe", np.eye(2), np.eye(2), use_gpu=False)


def test_version_string(native_lib):
    assert b"sm_103a" in native_lib.calchem_xc_version()


@pytest.mark.parametrize("bname", ["sto-3g", "6-31g", "6-31g(d)", "6-31g(d,p)"])
def test_prepared_shells_match_oracle_normalisation(oracle, bname):
    mol = workloads.octane()
    basis = BasisSet.from_name(bname, mol)
    sh, pr, co = basis.gpu_arrays()
    ob = oracle_basis(oracle, bname, mol)
    r2, wn, cs = ob.shell_data()
    assert ob.n_ao == basis.n_ao
    np.testing.assert_allclose(sh["r2_cutoff"], r2, rtol=0, atol=0)
    np.testing.assert_allclose(pr["weighted_norm"], wn, rtol=1e-15, atol=0)
    np.testing.assert_allclose(co["scale"], cs, rtol=1e-15, atol=0)
    assert list(sh["ao_offset"]) == sorted(sh["ao_offset"])


def test_overlap_matches_oracle(oracle):
    mol = workloads.octane()
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    S = basis.overlap()
    S_ref = oracle_basis(oracle, "6-31g(d,p)", mol).overlap()
    assert np.max(np.abs(S - S_ref)) < 1e-14
    assert np.max(np.abs(np.diag(S) - 1.0)) < 1e-12


def test_workload_ao_counts():
    assert BasisSet.from_name("6-31g(d)", workloads.water()).n_ao == 19
    assert BasisSet.from_name("6-31g(d,p)", workloads.octane()).n_ao == 210
    assert BasisSet.from_name("6-31g(d)", workloads.circumcoronene()).n_ao == 846
    assert BasisSet.from_name("6-31g(d)", workloads.water_cluster(61, 61)).n_ao == 1159


def _dist(a, b):
    return float(np.linalg.norm(a - b))


def test_octane_geometry():
    mol = workloads.octane()
    xyz = mol.coords_bohr / 1.8897261245650618
    sym = [a.symbol for a in mol.atoms]
    assert sym.count("C") == 8 and sym.count("H") == 18
    C = xyz[:8]
    for i in range(7):
        assert abs(_dist(C[i], C[i + 1]) - 1.54) < 1e-12
    for i in range(1, 7):
        a, b = C[i - 1] - C[i], C[i + 1] - C[i]
        ang = np.degrees(np.arccos(np.dot(a, b) / np.linalg.norm(a) / np.linalg.norm(b)))
        assert abs(ang - 109.4712206) < 1e-6
    for h in xyz[8:]:
        d = np.min(np.linalg.norm(C - h, axis=1))
        assert abs(d - 1.09) < 1e-9
    # every H-C-X angle tetrahedral
    for h in xyz[8:]:
        ci = int(np.argmin(np.linalg.norm(C - h, axis=1)))
        for other in list(C) + list(xyz[8:]):
            if _dist(other, C[ci]) < 1.6 and _dist(other, C[ci]) > 0.1 and _dist(other, h) > 0.1:
                a, b = h - C[ci], other - C[ci]
                ang = np.degrees(np.arccos(np.dot(a, b) / np.linalg.norm(a) / np.linalg.norm(b)))
                assert abs(ang - 109.4712206) < 1e-4


def test_circumcoronene_geometry():
    mol = workloads.circumcoronene()
    sym = [a.symbol for a in mol.atoms]
    assert sym.count("C") == 54 and sym.count("H") == 18
    mol.multiplicity = 3
    assert mol.n_alpha_beta() == (172, 170)
    xyz = mol.coords_bohr / 1.8897261245650618
    assert np.max(np.abs(xyz[:, 2])) == 0.0
    C, H = xyz[:54], xyz[54:]
    for h in H:
        assert abs(np.min(np.linalg.norm(C - h, axis=1)) - 1.09) < 1e-9
    dmin = min(_dist(C[i], C[j]) for i in range(54) for j in range(i + 1, 54))
    assert abs(dmin - 1.42) < 1e-9


def test_water_cluster_packing_is_seeded_and_valid():
    a = workloads.water_cluster(20, 5)
    b = workloads.water_cluster(20, 5)
    assert np.array_equal(a.coords_bohr, b.coords_bohr)
    xyz = a.coords_bohr / 1.8897261245650618
    O = xyz[0::3]
    for i in range(len(O)):
        for j in range(i + 1, len(O)):
            assert _dist(O[i], O[j]) >= 2.6
    for k in range(20):  # rigid monomers
        o, h1, h2 = xyz[3 * k:3 * k + 3]
        assert abs(_dist(o, h1) - np.hypot(0.757, 0.586)) < 1e-12
        assert abs(_dist(o, h2) - np.hypot(0.757, 0.586)) < 1e-12
    sizes = workloads.cluster_batch_sizes()
    assert len(sizes) == 64 and min(sizes) >= 1 and max(sizes) <= 32


def test_seeded_density_properties():
    mol = workloads.water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    S = basis.overlap()
    D = workloads.seeded_density_rks(S, 5, 7)
    assert np.max(np.abs(D - D.T)) < 1e-15
    assert abs(np.trace(D @ S) - 10.0) < 1e-10
    assert np.max(np.abs(D @ S @ D - 2.0 * D)) < 1e-10  # idempotent: (D/2) S (D/2) = D/2
    D2 = workloads.seeded_density_rks(S, 5, 7)
    assert np.array_equal(D, D2)


def test_name_parsing():
    assert XcFunctional.from_name("B3-LYP") == XcFunctional.B3LYP
    assert XcFunctional.from_name("PBE1PBE") == XcFunctional.PBE0
    assert XcFunctional.from_name("lda") == XcFunctional.SVWN5
    with pytest.raises(ValueError):
        XcFunctional.from_name("m06")
    assert GridLevel.from_name("FINE") == GridLevel.FINE
    assert GridLevel.from_name("whatever") == GridLevel.MEDIUM
    assert canonical_name("6-31G**") == "6-31g(d,p)"
    assert canonical_name("6-31g*") == "6-31g(d)"
