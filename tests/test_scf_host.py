"""SCF harness on the CPU: the integral code against closed forms and the quadrature's overlap, and a
Hartree-Fock energy against its textbook value (no GPU needed)."""

import math

import numpy as np
import pytest

from calchem_gb300 import BasisSet, scf, workloads
from calchem_gb300.molecule import Atom, Molecule


def test_boys_function_against_quadrature(native_lib):
    scipy = pytest.importorskip("scipy.integrate")
    for t in (0.0, 1e-6, 0.3, 2.5, 12.0, 34.9, 35.1, 80.0):
        F = np.zeros(18)
        assert native_lib.calchem_scf_boys(17, t, F.ctypes.data) == 0
        for n in (0, 1, 4, 9, 17):
            ref, _ = scipy.quad(lambda s: s ** (2 * n) * math.exp(-t * s * s), 0.0, 1.0, epsabs=1e-15, epsrel=1e-13)
            assert abs(F[n] - ref) < 1e-13 * max(1.0, ref) + 1e-16


def _single_s(alpha):
    mol = Molecule([Atom("H", [0.0, 0.0, 0.0])], 0, 2)
    from calchem_gb300.basis import Shell
    sh = Shell(0, np.zeros(3), 0, [alpha], [1.0], 0)
    return mol, BasisSet("s", [sh])


def test_one_electron_and_eri_closed_forms(native_lib):
    alpha = 0.7
    mol, basis = _single_s(alpha)
    S, T, V = scf.core_matrices(basis, mol)
    assert abs(S[0, 0] - 1.0) < 1e-13
    assert abs(T[0, 0] - 1.5 * alpha) < 1e-13
    assert abs(V[0, 0] + 2.0 * math.sqrt(2.0 * alpha / math.pi)) < 1e-13
    eri = scf.eri_tensor(basis)
    assert abs(eri[0, 0, 0, 0] - 2.0 * math.sqrt(alpha / math.pi)) < 1e-13


def test_overlap_equals_quadrature_layout_overlap_and_eri_symmetry(native_lib):
    mol = workloads.water()
    basis = BasisSet.from_name("6-31g(d)", mol)
    S, T, V = scf.core_matrices(basis, mol)
    assert np.max(np.abs(S - basis.overlap())) < 1e-12
    assert np.allclose(T, T.T) and np.allclose(V, V.T)
    assert np.all(np.linalg.eigvalsh(T) > 0)
    eri = scf.eri_tensor(BasisSet.from_name("sto-3g", mol))
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        assert np.max(np.abs(eri - eri.transpose(perm))) < 1e-14


def test_h2_rhf_sto3g_textbook_energy(native_lib):
    """H2 at R = 1.4 Bohr, RHF/STO-3G: -1.1167 Eh (Szabo & Ostlund, Modern Quantum Chemistry, 3.5)."""
    mol = Molecule([Atom("H", [0.0, 0.0, 0.0]), Atom("H", [0.0, 0.0, 1.4])], 0, 1)
    res = scf.rhf(mol, BasisSet.from_name("sto-3g", mol))
    assert res.converged
    assert abs(res.total_energy_hartree - (-1.1167)) < 1e-4
    ur = scf.uks(mol, BasisSet.from_name("sto-3g", mol), None)
    assert abs(ur.total_energy_hartree - res.total_energy_hartree) < 1e-10
