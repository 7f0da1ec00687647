"""SCF with the GPU XC quadrature: the reference's water benchmark (crates/calchem-scf/tests/
kohn_sham_dft.rs:39-78), closed-shell UKS = RKS, and the converged energy of the mixed-precision,
learned-pruned build against the FP64 Fine-grid build (within 1e-6 Eh)."""

import math

import pytest

from calchem_gb300 import BasisSet, GridLevel, scf, workloads
from calchem_gb300.molecule import Atom, Molecule

pytestmark = pytest.mark.gpu


def water_standard():
    r, half = 0.9572, math.radians(104.52 / 2)
    hy, hz = r * math.sin(half), -r * math.cos(half)
    return Molecule([Atom.from_angstrom("O", [0, 0, 0]), Atom.from_angstrom("H", [0, hy, hz]),
                     Atom.from_angstrom("H", [0, -hy, hz])], 0, 1)


@pytest.fixture(scope="module")
def lib(native_lib):
    assert native_lib.calchem_cuda_is_available() == 1, "no sm_103a device"
    return native_lib


def test_water_b3lyp_631gd_benchmark(lib):
    mol = water_standard()
    basis = BasisSet.from_name("6-31g(d)", mol)
    fine = scf.rks(mol, basis, "b3lyp", GridLevel.FINE)
    med = scf.rks(mol, basis, "b3lyp", GridLevel.MEDIUM)
    assert fine.converged and med.converged
    print(f"\nH2O B3LYP/6-31G(d): Fine {fine.total_energy_hartree:.8f} in {fine.iterations} iterations, "
          f"Medium {med.total_energy_hartree:.8f}")
    assert abs(med.total_energy_hartree - fine.total_energy_hartree) < 5e-5
    assert abs(fine.total_energy_hartree - (-76.40895)) < 1.5e-3


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_closed_shell_uks_matches_rks(lib, func):
    mol = water_standard()
    basis = BasisSet.from_name("6-31g(d)", mol)
    r = scf.rks(mol, basis, func, GridLevel.MEDIUM)
    u = scf.uks(mol, basis, func, GridLevel.MEDIUM)
    assert r.converged and u.converged
    assert abs(r.total_energy_hartree - u.total_energy_hartree) < 1e-9
    assert abs(u.s_squared) < 1e-10


def test_mixed_learned_scf_energy_matches_fp64_fine(lib):
    """The accuracy criterion for the fast path: converged SCF energy of the mixed-precision build on the
    learned-pruned grid (judge every 5 iterations) within 1e-6 Eh of the FP64 Fine-grid SCF."""
    mol = workloads.water_cluster(2, 17)
    basis = BasisSet.from_name("6-31g(d)", mol)
    ref = scf.rks(mol, basis, "b3lyp", GridLevel.FINE, precision="fp64")
    fast = scf.rks(mol, basis, "b3lyp", precision="mixed", learned=True, tol=5e-7)
    assert ref.converged and fast.converged
    print(f"\n(H2O)2 B3LYP: FP64 Fine {ref.total_energy_hartree:.10f} ({ref.grid_points} points), mixed learned "
          f"{fast.total_energy_hartree:.10f} ({fast.grid_points} points, reverted {len(fast.reverted_atoms)}), "
          f"dE {fast.total_energy_hartree - ref.total_energy_hartree:.2e}")
    assert fast.grid_points < ref.grid_points
    assert abs(fast.total_energy_hartree - ref.total_energy_hartree) < 1e-6


def test_octane_mixed_learned_scf_energy_matches_fp64_fine(lib, oracle):
    """The fast path's accuracy criterion on the C8H18 benchmark molecule (B3LYP / 6-31G(d,p), 210 AOs,
    33 doubly occupied orbitals): the converged SCF energy with the tensor-core build on the learned
    grid (judge every 5 iterations) within 1e-6 Eh of the FP64 Fine-grid SCF; and the FP64 Fine
    SCF's first-iteration Exc (core-Hamiltonian guess density) against the oracle's CalChem
    restatement on the same grid."""
    mol = workloads.octane()
    basis = BasisSet.from_name("6-31g(d,p)", mol)
    ints = scf.integrals(mol, basis)
    ref = scf.rks(mol, basis, "b3lyp", GridLevel.FINE, precision="fp64", ints=ints, e_tol=1e-9, g_tol=1e-6)
    fast = scf.rks(mol, basis, "b3lyp", precision="mixed", learned=True, tol=5e-7, ints=ints, e_tol=1e-9,
                   g_tol=1e-6)
    assert ref.converged and fast.converged
    print(f"\nC8H18 B3LYP/6-31G(d,p): FP64 Fine {ref.total_energy_hartree:.10f} ({ref.grid_points} points, "
          f"{ref.iterations} iterations), mixed learned {fast.total_energy_hartree:.10f} ({fast.grid_points} "
          f"points, {fast.iterations} iterations, reverted {len(fast.reverted_atoms)}), "
          f"dE {fast.total_energy_hartree - ref.total_energy_hartree:.2e}")
    assert fast.grid_points < ref.grid_points
    assert abs(fast.total_energy_hartree - ref.total_energy_hartree) < 1e-6
    from calchem_gb300 import MolecularGrid
    grid = MolecularGrid.build_for_basis(mol, basis, GridLevel.FINE)
    ob = oracle.Basis.from_name("6-31g(d,p)", [a.symbol for a in mol.atoms], mol.coords_bohr)
    e_or, _, _ = oracle.RksEngine(ob, oracle.Grid.from_points(grid.xyzw)).evaluate(ref.first_density, "b3lyp")
    assert abs(ref.first_exc - e_or) < 1e-9