"""GPU tests of the batched TD-DFT kernel contraction (FxcKernel), following the reference's own
checks (crates/calchem-dft/src/fxc.rs:663-750, 862-990): singlet / triplet dV[M] must equal the
4-point central finite difference of the UKS Vxc along (P/2 + eps M, P/2 +- eps M), for every
functional, and be symmetric; a batch must equal its members contracted one by one."""

import numpy as np
import pytest

from calchem_gb300 import BasisSet, FxcKernel, GridLevel, MolecularGrid, UksVxcEngine
from calchem_gb300.molecule import Atom, Molecule

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    mol = Molecule([Atom.from_angstrom("O", [0.0, 0.0, 0.1173]), Atom.from_angstrom("H", [0.0, 0.7572, -0.4692]),
                    Atom.from_angstrom("H", [0.0, -0.7572, -0.4692])], 0, 1)
    basis = BasisSet.from_name("6-31g(d)", mol)
    grid = MolecularGrid.build(mol, GridLevel.COARSE)
    n = basis.n_ao
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    P0 = np.where(i == j, 0.25 + 0.01 * i, 0.015 * np.sin(np.minimum(i, j) * 7 + np.maximum(i, j) * 3))
    M = 0.02 * np.cos(np.minimum(i, j) * 5 + np.maximum(i, j) * 11 + 1)
    return mol, basis, grid, P0, M


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"])
def test_fxc_matches_uks_vxc_finite_differences(setup, func):
    mol, basis, grid, P0, M = setup
    ker = FxcKernel(basis, grid, func, P0)
    uks = UksVxcEngine(basis, grid)
    eps = 1e-5
    for triplet, sign_b in ((False, 1.0), (True, -1.0)):
        dv = ker.contract(M, triplet)
        assert np.max(np.abs(dv - dv.T)) < 1e-13
        va = {}
        for k in (-2, -1, 1, 2):
            _, va[k], _ = uks.evaluate(basis, grid, func, 0.5 * P0 + k * eps * M, 0.5 * P0 + k * sign_b * eps * M)
        fd = (va[-2] - 8 * va[-1] + 8 * va[1] - va[2]) / (12 * eps)
        assert np.max(np.abs(dv - fd)) < 1e-8, (func, triplet, np.max(np.abs(dv - fd)))
    ker.close()
    uks.close()


def test_batch_equals_single_contractions_and_zero_trials(setup):
    mol, basis, grid, P0, M = setup
    ker = FxcKernel(basis, grid, "b3lyp", P0)
    rng = np.random.default_rng(3)
    mats = [M, 0.5 * (lambda a: a + a.T)(rng.normal(size=M.shape)) * 0.01, np.zeros_like(M)]
    for triplet in (False, True):
        batch = ker.contract_batch(mats, triplet)
        for m, dv in zip(mats, batch):
            assert np.max(np.abs(dv - ker.contract(m, triplet))) < 1e-13
        assert np.all(batch[2] == 0.0)
    assert ker.contract_batch([], False) == []
    ker.close()


@pytest.mark.parametrize("func", ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"])
def test_tensor_core_contraction_matches_fp64(setup, func):
    """calchem_xc_fxc_contract_ex with CALCHEM_XC_MIXED (the closed-shell tensor-core pipeline per trial
    matrix, the AO cache shared by the trials) against the FP64 contraction: within 1e-6 of the
    largest dV entry, symmetric, exact zeros for a zero trial matrix."""
    mol, basis, grid, P0, M = setup
    ker = FxcKernel(basis, grid, func, P0)
    rng = np.random.default_rng(5)
    mats = [M, 0.5 * (lambda a: a + a.T)(rng.normal(size=M.shape)) * 0.01, np.zeros_like(M)]
    for triplet in (False, True):
        ref = ker.contract_batch(mats, triplet, precision="fp64")
        got = ker.contract_batch(mats, triplet, precision="mixed")
        for r, d in zip(ref[:2], got[:2]):
            scale = np.max(np.abs(r))
            assert scale > 0
            assert np.max(np.abs(d - r)) < 1e-6 * scale, (func, triplet, np.max(np.abs(d - r)) / scale)
            assert np.array_equal(d, d.T)
        assert np.all(got[2] == 0.0)
    ker.close()


def test_tensor_core_contraction_octane():
    """C8H18 B3LYP/6-31G(d,p), Medium grid, five trial matrices: the tensor-core contraction against FP64."""
    from calchem_gb300 import workloads
    mol = workloads.octane()
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.MEDIUM)
    D = workloads.seeded_density_rks(basis.overlap(), 33, 7)
    ker = FxcKernel(basis, grid, "b3lyp", D, precision="mixed")
    rng = np.random.default_rng(9)
    mats = [0.01 * (lambda a: a + a.T)(rng.normal(size=D.shape)) for _ in range(5)]
    got = ker.contract_batch(mats)
    ref = ker.contract_batch(mats, precision="fp64")
    ker.close()
    for r, d in zip(ref, got):
        assert np.max(np.abs(d - r)) < 1e-6 * np.max(np.abs(r))


def test_device_pointer_contraction_with_precision(setup):
    """calchem_xc_fxc_contract_device_ex (device buffers, caller's stream) equals the host-buffer call
    in both precisions."""
    torch = pytest.importorskip("torch")
    from calchem_gb300 import _native
    mol, basis, grid, P0, M = setup
    ker = FxcKernel(basis, grid, "pbe0", P0)
    lib = _native.load()
    dev = torch.device("cuda:0")
    mats = np.ascontiguousarray(np.stack([M, 0.5 * M.T + 0.5 * M]))
    d_m = torch.from_numpy(mats).to(dev)
    d_v = torch.zeros_like(d_m)
    stream = torch.cuda.current_stream(dev)
    for prec in ("fp64", "mixed"):
        host = ker.contract_batch(list(mats), precision=prec)
        d_v.fill_(7.0)
        assert lib.calchem_xc_fxc_contract_device_ex(ker.grid_id, 0, 0 if prec == "fp64" else 1, d_m.data_ptr(), 2,
                                                     d_v.data_ptr(), stream.cuda_stream) == 0
        torch.cuda.synchronize(dev)
        out = d_v.cpu().numpy()
        for a, b in zip(host, out):
            assert np.max(np.abs(a - b)) < 1e-13 * max(1.0, np.max(np.abs(a)))
    assert lib.calchem_xc_fxc_contract_device_ex(ker.grid_id, 0, 5, d_m.data_ptr(), 2, d_v.data_ptr(), None) == -1
    ker.close()
