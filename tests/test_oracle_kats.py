"""The reference's own known-answer tests for the XC quadrature, re-run against the oracle.

These pin the oracle (the CPU restatement used to check the GPU) to CalChem's
tests: every bound below is the bound in the cited reference test.
"""

import math

import numpy as np
import pytest

from tests.helpers import distorted_water, make_positive_density, oracle_basis

FUNCS = ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0", "camb3lyp", "wb97x", "wb97xd"]


def _dfact(n):
    acc = 1.0
    while n > 1:
        acc *= n
        n -= 2
    return acc


def _sphere_monomial(p, q, r):
    if p % 2 or q % 2 or r % 2:
        return 0.0
    return 4.0 * math.pi * _dfact(p - 1) * _dfact(q - 1) * _dfact(r - 1) / _dfact(p + q + r + 1)


@pytest.mark.parametrize("n,order", [(26, 7), (50, 11), (110, 17), (194, 23), (302, 29), (590, 41)])
def test_lebedev_monomial_exactness(oracle, n, order):
    """lebedev.rs:278-326: unit vectors, positive weights, monomials exact to 1e-12 up to the order."""
    L = oracle.lebedev(n)
    u, w = L[:, :3], L[:, 3]
    assert np.max(np.abs(np.sum(u * u, axis=1) - 1.0)) < 1e-14
    assert np.all(w > 0)
    x, y, z = u.T
    for p in range(order + 1):
        for q in range(order + 1 - p):
            for r in range(order + 1 - p - q):
                num = float(np.sum(w * x ** p * y ** q * z ** r))
                assert abs(num - _sphere_monomial(p, q, r)) < 1e-12, (n, p, q, r)


def test_lebedev_exp_benchmark(oracle):
    """int_{S^2} exp(x) = 4 pi sinh(1) on the 302-point rule to 1e-13 (lebedev.rs:316-325)."""
    L = oracle.lebedev(302)
    assert abs(np.sum(L[:, 3] * np.exp(L[:, 0])) - 4 * math.pi * math.sinh(1.0)) < 1e-13


def test_single_center_gaussian_integral(oracle):
    """grid.rs:837-857: one C atom, Medium grid, int exp(-a r^2) = (pi/a)^(3/2) to rel 1e-6."""
    g = oracle.Grid.build([6], [[0.0, 0.0, 0.0]], "medium")
    xyzw, _, _ = g.points()
    r2 = np.sum(xyzw[:, :3] ** 2, axis=1)
    for a in (0.15, 1.0, 8.5):
        exact = (math.pi / a) ** 1.5
        assert abs(np.sum(xyzw[:, 3] * np.exp(-a * r2)) - exact) / exact < 1e-6


def test_multicenter_becke_gaussian_sum(oracle):
    """grid.rs:860-888: distorted water, Medium grid, three unit Gaussians integrate to 3 pi^(3/2)."""
    from calchem_gb300.molecule import Atom, Molecule

    mol = Molecule([Atom.from_angstrom("O", [0.02, -0.04, 0.12]), Atom.from_angstrom("H", [0.08, 0.78, -0.45]),
                    Atom.from_angstrom("H", [-0.05, -0.74, -0.49])])
    g = oracle.Grid.build(mol.z, mol.coords_bohr, "medium")
    xyzw, _, _ = g.points()
    val = np.zeros(len(xyzw))
    for c in mol.coords_bohr:
        val += np.exp(-np.sum((xyzw[:, :3] - c) ** 2, axis=1))
    exact = 3.0 * math.pi ** 1.5
    assert abs(np.sum(xyzw[:, 3] * val) - exact) / exact < 2e-5


def test_fine_grid_point_counts(oracle):
    """Fine grid: 99 radial shells for every Z <= 18 (grid.rs:745-752), pruned to 16,182 raw points."""
    for z in (1, 6, 8):
        n = 0
        rbs = oracle.lib().orc_bragg_slater_bohr(z)
        for i in range(1, 100):
            r = rbs * i * i / (100 - i) ** 2
            ratio = r / max(rbs, 0.3)
            n += 50 if ratio < 0.18 else 110 if ratio < 0.5 else 194 if ratio < 0.95 else 302 if ratio < 5 else 194
        assert n == 16182
    g = oracle.Grid.build([6], [[0.0, 0.0, 0.0]], "fine")
    assert len(g) == 16182  # a single atom keeps every point (Becke weight 1)


@pytest.mark.parametrize("alpha", [1e-4, 1e-6])
def test_diffuse_gaussian_density_conserves_one_electron(oracle, alpha):
    """calchem-dft/tests/redteam_diffuse.rs:5-24 with the diffuse radial extension (grid.rs:650-663)."""
    extra = min(math.ceil(180.0 * (1e-4 / alpha) ** 0.25), 4096)
    g = oracle.Grid.build([1], [[0.0, 0.0, 0.0]], "fine", extra)
    xyzw, _, _ = g.points()
    norm = (2.0 * alpha / math.pi) ** 1.5
    q = np.sum(xyzw[:, 3] * norm * np.exp(-2.0 * alpha * np.sum(xyzw[:, :3] ** 2, axis=1)))
    assert abs(q - 1.0) < 1e-6


def test_ao_gradient_and_hessian_vs_finite_differences(oracle):
    """ao_grid.rs:307-379: 6-31G(d,p) O-H plus an f shell; grad vs FD < 1e-9, Hessian vs FD < 1e-8."""
    from calchem_gb300.molecule import Atom, Molecule

    mol = Molecule([Atom.from_angstrom("O", [0.1, -0.2, 0.05]), Atom.from_angstrom("H", [0.8, 0.5, -0.3])])
    shells = oracle.basis_shells("6-31g(d,p)", ["O", "H"], mol.coords_bohr)
    shells.append((3, 0, mol.coords_bohr[0], [0.85], [1.0]))
    b = oracle.Basis(shells)
    r0 = np.array([0.43, -0.61, 0.29])
    ana = b.ao_hess(r0)[0]
    h = 1e-6
    for q in range(3):
        rp, rm = r0.copy(), r0.copy()
        rp[q] += h
        rm[q] -= h
        gp, gm = b.ao_grad(rp)[0], b.ao_grad(rm)[0]
        fd_grad = (gp[:, 0] - gm[:, 0]) / (2 * h)
        assert np.max(np.abs(ana[:, 1 + q] - fd_grad)) < 1e-9
        hrow = {0: [4, 5, 6], 1: [5, 7, 8], 2: [6, 8, 9]}[q]
        for p in range(3):
            fd_h = (gp[:, 1 + p] - gm[:, 1 + p]) / (2 * h)
            assert np.max(np.abs(ana[:, hrow[p]] - fd_h)) < 1e-8


XC_POINTS = [
    (0.37, 0.19, 0.41, 0.12, 0.23),              # open shell
    (0.25, 0.25, 0.18, 0.18, 0.18),              # closed shell
    (14.2, 13.8, 120.0, 110.0, 105.0),           # core
    (1.2e-4, 0.7e-4, 3.5e-7, 1.1e-7, 2.0e-7),   # tail
    (0.42, 0.0, 0.31, 0.0, 0.0),                 # fully polarised
]


@pytest.mark.parametrize("func", FUNCS)
@pytest.mark.parametrize("pt", XC_POINTS)
def test_xc_partials_vs_finite_differences(oracle, func, pt):
    """xc.rs:1142-1238: 4-point central differences, |ana - fd| < 1e-9."""
    ra, rb, gaa, gab, gbb = pt
    ana = oracle.eval_xc(func, np.array([pt]))[0]
    hr = 1e-6 * max(ra + rb, 1e-2)
    hg = 1e-6 * (gaa + gbb + 1.0)

    def f(x):
        return oracle.eval_xc(func, np.array([x]))[0, 0]

    def fd4(idx, h):
        def sh(d):
            x = list(pt)
            x[idx] += d
            return f(x)
        return (-sh(2 * h) + 8 * sh(h) - 8 * sh(-h) + sh(-2 * h)) / (12 * h)

    if ra > 5 * hr:
        assert abs(ana[1] - fd4(0, hr)) < 1e-9
    if rb > 5 * hr:
        assert abs(ana[2] - fd4(1, hr)) < 1e-9
    if gaa > 5 * hg:
        assert abs(ana[3] - fd4(2, hg)) < 1e-9
    if gaa > 5 * hg and gbb > 5 * hg:
        assert abs(ana[4] - fd4(3, hg)) < 1e-9
    if gbb > 5 * hg:
        assert abs(ana[5] - fd4(4, hg)) < 1e-9


def test_lyp_one_electron_correlation_vanishes(oracle):
    """xc.rs:1240-1247."""
    out = oracle.lyp(np.array([0.53, 0.0, 0.77, 0.0, 0.0]))
    assert abs(out[0]) < 1e-16 and abs(out[1]) < 1e-16 and abs(out[3]) < 1e-16


@pytest.fixture(scope="module")
def water_coarse(oracle):
    mol = distorted_water()
    b = oracle_basis(oracle, "6-31g(d)", mol)
    g = oracle.Grid.build(mol.z, mol.coords_bohr, "coarse")
    return mol, b, g


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_rks_vxc_is_density_derivative_and_symmetric(oracle, water_coarse, func):
    """vxc.rs:2387-2436: V = dExc/dP by central differences (eps 1e-6) to 1e-9; V symmetric to 1e-14."""
    _, b, g = water_coarse
    n = b.n_ao
    P = make_positive_density(n, 1)
    eps = 1e-6
    _, _, V = oracle.vxc_rks_points(b, g, P, func)
    for mu, nu in [(0, 0), (0, 3), (2, 7), (5, 11), (8, 14), (12, 12)]:
        assert abs(V[mu, nu] - V[nu, mu]) < 1e-14
        Pp, Pm = P.copy(), P.copy()
        Pp[mu, nu] += eps
        Pm[mu, nu] -= eps
        if mu != nu:
            Pp[nu, mu] += eps
            Pm[nu, mu] -= eps
        ep = oracle.vxc_rks_points(b, g, Pp, func)[0]
        em = oracle.vxc_rks_points(b, g, Pm, func)[0]
        fd = (ep - em) / ((2.0 if mu == nu else 4.0) * eps)
        assert abs(V[mu, nu] - fd) < 1e-9


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_closed_shell_uks_matches_rks(oracle, water_coarse, func):
    """vxc.rs:2438-2449: UKS(P/2, P/2) == RKS(P) to 1e-13."""
    _, b, g = water_coarse
    P = make_positive_density(b.n_ao, 1)
    er, _, Vr = oracle.vxc_rks_points(b, g, P, func)
    eu, _, _, Va, Vb = oracle.vxc_uks_points(b, g, 0.5 * P, 0.5 * P, func)
    assert abs(er - eu) < 1e-13
    assert np.max(np.abs(Va - Vr)) < 1e-13 and np.max(np.abs(Vb - Vr)) < 1e-13


@pytest.mark.parametrize("func", ["blyp", "b3lyp", "pbe0"])
def test_uks_vxc_is_spin_density_derivative(oracle, water_coarse, func):
    """vxc.rs:2451-2495: open-shell V_sigma = dExc/dP_sigma to 1e-9."""
    _, b, g = water_coarse
    n = b.n_ao
    Pa, Pb = make_positive_density(n, 2), make_positive_density(n, 5)
    eps = 1e-6
    _, _, _, Va, Vb = oracle.vxc_uks_points(b, g, Pa, Pb, func)
    for mu, nu in [(1, 1), (1, 6), (4, 10), (9, 15)]:
        den = 2 * eps if mu == nu else 4 * eps

        def shifted(M, s):
            M = M.copy()
            M[mu, nu] += s
            if mu != nu:
                M[nu, mu] += s
            return M
        fda = (oracle.vxc_uks_points(b, g, shifted(Pa, eps), Pb, func)[0] -
               oracle.vxc_uks_points(b, g, shifted(Pa, -eps), Pb, func)[0]) / den
        fdb = (oracle.vxc_uks_points(b, g, Pa, shifted(Pb, eps), func)[0] -
               oracle.vxc_uks_points(b, g, Pa, shifted(Pb, -eps), func)[0]) / den
        assert abs(Va[mu, nu] - fda) < 1e-9
        assert abs(Vb[mu, nu] - fdb) < 1e-9


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_cached_gemm_path_matches_per_point_path(oracle, water_coarse, func):
    """vxc.rs:2628-2645: the BLAS-3 engine agrees with evaluate_vxc_rks to 1e-12 in Exc and V."""
    _, b, g = water_coarse
    P = make_positive_density(b.n_ao, 7)
    e1, n1, V1 = oracle.vxc_rks_points(b, g, P, func)
    eng = oracle.RksEngine(b, g)
    assert eng.cached
    e2, n2, V2 = eng.evaluate(P, func)
    assert abs(e1 - e2) < 1e-12 and abs(n1 - n2) < 1e-12
    assert np.max(np.abs(V1 - V2)) < 1e-12


def test_zero_weight_grid_gives_zeros(oracle):
    """vxc.rs:2744-2783: a single zero-weight point gives exactly zero Exc and V."""
    mol = distorted_water()
    b = oracle_basis(oracle, "sto-3g", mol)
    g = oracle.Grid.from_points(np.array([[0.0, 0.0, 0.0, 0.0]]))
    P = make_positive_density(b.n_ao, 1)
    e, ne, V = oracle.vxc_rks_points(b, g, P, "b3lyp")
    assert e == 0.0 and ne == 0.0 and np.all(V == 0.0)
    e, na, nb, Va, Vb = oracle.vxc_uks_points(b, g, P, P, "b3lyp")
    assert e == 0.0 and np.all(Va == 0.0) and np.all(Vb == 0.0)


def test_overlap_is_normalised_and_seeded_density_traces(oracle):
    """Contracted AOs are normalised (normalization.rs:52-58); tr(D S) = 2 n_occ for seeded D."""
    from calchem_gb300 import workloads

    mol = workloads.water()
    b = oracle_basis(oracle, "6-31g(d)", mol)
    S = b.overlap()
    assert np.max(np.abs(np.diag(S) - 1.0)) < 1e-12
    assert np.max(np.abs(S - S.T)) < 1e-14
    D = workloads.seeded_density_rks(S, 5, 7)
    assert abs(np.trace(D @ S) - 10.0) < 1e-10


def test_cam_exchange_matches_70_digit_ityh_reference(oracle):
    """xc.rs:1110-1140: CAM-B3LYP attenuated exchange of one spin against independent high-precision
    values (rho_s, gamma_ss) -> (f, v_rho, v_gamma)."""
    for rho, gam, e, vr, vg in [(0.05, 0.001, -0.010533928866947627, -0.2932000891552038, -0.10900565576558356),
                                (0.2, 0.1, -0.07507503986684043, -0.4990012926064571, -0.01800971179470531),
                                (0.001, 0.3, -0.003471498357842851, -0.5447077074153023, -0.005110453550847137)]:
        got = oracle.cam_x_one(rho, gam)
        assert abs(got[0] - e) < 1e-12
        assert abs(got[1] - vr) < 1e-10
        assert abs(got[2] - vg) < 1e-10


@pytest.mark.parametrize("func", ["svwn5", "pbe", "b3lyp"])
def test_xc_gradient_matches_finite_differences_with_moving_grid(oracle, func):
    """vxc.rs:2498-2548: the analytic XC nuclear gradient (AO and Becke-weight terms) equals the
    central difference of Exc(R +- h) with the grid and basis moving with the atoms (h = 1e-5 Bohr,
    |ana - fd| < 1e-8), and sums to zero over the atoms (translational invariance, < 1e-12)."""
    from tests.helpers import distorted_water, make_positive_density
    mol = distorted_water()
    sym = [a.symbol for a in mol.atoms]
    xyz = np.array(mol.coords_bohr)
    basis = oracle.Basis.from_name("6-31g(d)", sym, xyz)
    n = basis.n_ao
    Pa, Pb = make_positive_density(n, 3), make_positive_density(n, 8)
    grid = oracle.Grid.build(mol.z, xyz, "coarse")
    ana = oracle.xc_gradient(basis, grid, mol.z, xyz, Pa, Pb, func)
    assert np.max(np.abs(ana.sum(axis=0))) < 1e-12
    h = 1e-5
    for a in range(len(sym)):
        for q in range(3):
            e = []
            for sgn in (1.0, -1.0):
                x = xyz.copy()
                x[a, q] += sgn * h
                b = oracle.Basis.from_name("6-31g(d)", sym, x)
                g = oracle.Grid.build(mol.z, x, "coarse")
                e.append(oracle.vxc_uks_points(b, g, Pa, Pb, func)[0])
            fd = (e[0] - e[1]) / (2 * h)
            assert abs(ana[a, q] - fd) < 1e-8, (a, q, ana[a, q], fd)


def test_xc_gradient_parts_add_up(oracle):
    """The AO term (parts=1) and the Becke weight term (parts=2) sum to the full gradient."""
    from tests.helpers import distorted_water, make_positive_density
    mol = distorted_water()
    xyz = np.array(mol.coords_bohr)
    basis = oracle.Basis.from_name("6-31g(d)", [a.symbol for a in mol.atoms], xyz)
    grid = oracle.Grid.build(mol.z, xyz, "coarse")
    Pa, Pb = make_positive_density(basis.n_ao, 3), make_positive_density(basis.n_ao, 8)
    full = oracle.xc_gradient(basis, grid, mol.z, xyz, Pa, Pb, "pbe")
    ao = oracle.xc_gradient(basis, grid, mol.z, xyz, Pa, Pb, "pbe", parts=1)
    wt = oracle.xc_gradient(basis, grid, mol.z, xyz, Pa, Pb, "pbe", parts=2)
    assert np.max(np.abs(ao + wt - full)) < 1e-13
    assert np.max(np.abs(wt)) > 1e-4 and np.max(np.abs(ao)) > 1e-3
