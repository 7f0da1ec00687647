"""Synthetic workloads: the benchmark molecules and seeded densities.

No public benchmark suite is involved: the inputs are geometries built from
stated rules and densities seeded from numpy's PCG64.

* water: O (0, 0, 0), H (+-0.757, 0.586, 0) Angstrom.
* n-octane C8H18: all-trans zigzag, C-C 1.54, C-H 1.09 Angstrom, tetrahedral angles.
* water clusters of k molecules: rigid monomers (the water above), uniformly random
  orientations, oxygens placed uniformly in a cube of side (29.9 k)^(1/3) Angstrom
  (1 g/cm^3) by rejection until every O-O distance is >= 2.6 Angstrom.
* circumcoronene-type flake C54H18: 19 hexagons (one centre, two rings), C-C 1.42,
  edge C-H 1.09 Angstrom along the outward bisector, planar.

Seeded densities: G ~ N(0, 1) (n_ao x n_occ, PCG64(seed)), C = G (G^T S G)^(-1/2)
so that C^T S C = I, and D = 2 C C^T (closed shell) or D_sigma = C_sigma C_sigma^T.
"""

import math

import numpy as np

from .basis import BasisSet
from .molecule import Atom, Molecule

WATER_GEOMETRY = (("O", (0.0, 0.0, 0.0)), ("H", (0.757, 0.586, 0.0)), ("H", (-0.757, 0.586, 0.0)))


def water() -> Molecule:
    return Molecule([Atom.from_angstrom(s, p) for s, p in WATER_GEOMETRY], 0, 1)


def _unit(v):
    return v / np.linalg.norm(v)


def _rotate(v, axis, angle):
    k = _unit(axis)
    return v * math.cos(angle) + np.cross(k, v) * math.sin(angle) + k * np.dot(k, v) * (1 - math.cos(angle))


def alkane(n_carbon: int = 8) -> Molecule:
    """All-trans CnH2n+2 in the xy plane."""
    cc, ch = 1.54, 1.09
    half = math.radians(109.4712206) / 2.0
    dx, dy = cc * math.sin(half), cc * math.cos(half)
    carbons = [np.array([i * dx, (i % 2) * dy, 0.0]) for i in range(n_carbon)]
    atoms = [("C", c) for c in carbons]
    normal = np.array([0.0, 0.0, 1.0])
    hs = []
    for i, c in enumerate(carbons):
        nbr = [carbons[j] for j in (i - 1, i + 1) if 0 <= j < n_carbon]
        if len(nbr) == 2:
            b = _unit(nbr[0] - c) + _unit(nbr[1] - c)
            s = math.sqrt(max(0.0, 1.0 - np.dot(b, b) / 4.0))
            for sg in (1.0, -1.0):
                hs.append(c + ch * (-b / 2.0 + sg * s * normal))
        else:
            # terminal CH3: one H where the zigzag would continue, two rotated by +-120 degrees
            virt = np.array([(i + (1 if i > 0 else -1)) * dx, ((i + 1) % 2) * dy, 0.0])
            axis = _unit(nbr[0] - c)
            h0 = _unit(virt - c)
            for ang in (0.0, 2 * math.pi / 3, 4 * math.pi / 3):
                hs.append(c + ch * _rotate(h0, axis, ang))
    atoms += [("H", h) for h in hs]
    return Molecule([Atom.from_angstrom(s, p) for s, p in atoms], 0, 1)


def octane() -> Molecule:
    return alkane(8)


def _random_rotation(rng):
    u1, u2, u3 = rng.random(3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(k: int, seed: int, min_oo: float = 2.6, max_tries: int = 200000) -> Molecule:
    rng = np.random.Generator(np.random.PCG64(seed))
    side = (29.9 * k) ** (1.0 / 3.0)
    mono = np.array([p for _, p in WATER_GEOMETRY])
    oxy = []
    atoms = []
    tries = 0
    while len(oxy) < k:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"could not place {k} waters with O-O >= {min_oo} A")
        o = rng.random(3) * side
        if oxy and np.min(np.linalg.norm(np.array(oxy) - o, axis=1)) < min_oo:
            continue
        rot = _random_rotation(rng)
        oxy.append(o)
        for (sym, _), p in zip(WATER_GEOMETRY, mono):
            atoms.append(Atom.from_angstrom(sym, o + rot @ p))
    return Molecule(atoms, 0, 1)


def cluster_batch_sizes(n_clusters: int = 64, seed: int = 2024, kmax: int = 32):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [int(v) for v in rng.integers(1, kmax + 1, size=n_clusters)]


def circumcoronene() -> Molecule:
    d, ch = 1.42, 1.09
    a1 = np.array([math.sqrt(3) * d, 0.0])
    a2 = np.array([math.sqrt(3) / 2 * d, 1.5 * d])
    centres = []
    for i in range(-2, 3):
        for j in range(-2, 3):
            k = -i - j
            if max(abs(i), abs(j), abs(k)) <= 2:
                centres.append(i * a1 + j * a2)
    verts = []
    for c in centres:
        for t in range(6):
            ang = math.radians(30 + 60 * t)
            v = c + d * np.array([math.cos(ang), math.sin(ang)])
            if not any(np.linalg.norm(v - u) < 1e-6 for u in verts):
                verts.append(v)
    verts = np.array(verts)
    atoms = [("C", (v[0], v[1], 0.0)) for v in verts]
    for i, v in enumerate(verts):
        dist = np.linalg.norm(verts - v, axis=1)
        nb = np.where((dist > 1e-6) & (dist < d * 1.05))[0]
        if len(nb) == 2:
            out = -(_unit(verts[nb[0]] - v) + _unit(verts[nb[1]] - v))
            h = v + ch * _unit(out)
            atoms.append(("H", (h[0], h[1], 0.0)))
    return Molecule([Atom.from_angstrom(s, p) for s, p in atoms], 0, 1)


def orthonormal_orbitals(S: np.ndarray, n_occ: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    G = rng.standard_normal((S.shape[0], n_occ))
    M = G.T @ S @ G
    w, U = np.linalg.eigh(M)
    return G @ (U @ np.diag(1.0 / np.sqrt(w)) @ U.T)


def seeded_density_rks(S: np.ndarray, n_occ: int, seed: int) -> np.ndarray:
    C = orthonormal_orbitals(S, n_occ, seed)
    D = 2.0 * C @ C.T
    return 0.5 * (D + D.T)


def seeded_density_uks(S: np.ndarray, n_alpha: int, n_beta: int, seed_a: int, seed_b: int):
    Ca = orthonormal_orbitals(S, n_alpha, seed_a)
    Cb = orthonormal_orbitals(S, n_beta, seed_b)
    Pa = Ca @ Ca.T
    Pb = Cb @ Cb.T
    return 0.5 * (Pa + Pa.T), 0.5 * (Pb + Pb.T)


# Named workloads: (molecule builder, basis, functional, spin)
CONFIGS = {
    "water_svwn5": (water, "6-31g(d)", "svwn5", "rks"),
    "octane_b3lyp": (octane, "6-31g(d,p)", "b3lyp", "rks"),
    "c54h18_pbe0_uks": (circumcoronene, "6-31g(d)", "pbe0", "uks"),
}


def build_workload(name: str, seed: int = 7):
    """Returns (mol, basis, functional name, densities) for a named workload."""
    mk, bname, func, spin = CONFIGS[name]
    mol = mk()
    if name == "c54h18_pbe0_uks":
        mol.multiplicity = 3
    basis = BasisSet.from_name(bname, mol)
    S = basis.overlap()
    if spin == "rks":
        dens = (seeded_density_rks(S, mol.nelectron() // 2, seed),)
    else:
        na, nb = mol.n_alpha_beta()
        dens = seeded_density_uks(S, na, nb, seed, seed + 1)
    return mol, basis, func, dens
