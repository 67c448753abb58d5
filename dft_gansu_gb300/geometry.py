"""Seeded synthetic geometries of the benchmark molecules (angstrom in, bohr out).

The reference measures on no public suite; these generators stand in for the
named inputs with the stated shapes:
  water            O (0,0,0), H (+-0.7572, 0.5865, 0)
  n-alkane CnH2n+2 zig-zag chain, C-C 1.54, C-H 1.09, tetrahedral angles,
                   N(0, sigma) jitter (decane: n=10, sigma 0.02)
  C60              truncated icosahedron with 1.40 (6-6) / 1.45 (5-6) bonds,
                   N(0, 0.01) jitter
  water clusters   (H2O)n, O-H 0.96, H-O-H 104.5 deg, O-O >= 2.7
All randomness comes from numpy.random.default_rng(seed).
"""
from __future__ import annotations

import math

import numpy as np

ANGSTROM_TO_BOHR = 1.8897259886
TETRA = math.radians(109.4712206)
Z = {"H": 1, "C": 6, "N": 7, "O": 8}


def _to_atoms(symbols, xyz_ang):
    xyz = np.asarray(xyz_ang, dtype=float) * ANGSTROM_TO_BOHR
    return [(Z[s], float(x), float(y), float(z)) for s, (x, y, z) in zip(symbols, xyz)]


def water():
    """Water of the STO-3G configuration (bohr)."""
    return _to_atoms(["O", "H", "H"], [[0.0, 0.0, 0.0], [0.7572, 0.5865, 0.0], [-0.7572, 0.5865, 0.0]])


def _unit(v):
    return v / np.linalg.norm(v)


def alkane(n_carbon: int = 10, jitter: float = 0.02, seed: int = 0, cc: float = 1.54, ch: float = 1.09):
    """Zig-zag n-alkane C_n H_{2n+2} with tetrahedral angles (bohr)."""
    if n_carbon == 1:  # methane: four H on the tetrahedron vertices
        t = ch / math.sqrt(3.0)
        coords = np.array([[0.0, 0.0, 0.0], [t, t, t], [t, -t, -t], [-t, t, -t], [-t, -t, t]])
        if jitter:
            coords = coords + np.random.default_rng(seed).normal(0.0, jitter, coords.shape)
        return _to_atoms(["C", "H", "H", "H", "H"], coords)
    half = TETRA / 2.0
    carbons = np.array([[i * cc * math.sin(half), (i % 2) * cc * math.cos(half), 0.0] for i in range(n_carbon)])
    symbols, coords = [], []
    for c in carbons:
        symbols.append("C")
        coords.append(c)
    ez = np.array([0.0, 0.0, 1.0])
    for i, c in enumerate(carbons):
        nbr = []
        if i > 0:
            nbr.append(_unit(carbons[i - 1] - c))
        if i + 1 < n_carbon:
            nbr.append(_unit(carbons[i + 1] - c))
        if len(nbr) == 1:  # terminal: continue the zig-zag in plane with one H
            j = -1 if i == 0 else n_carbon
            ghost = np.array([j * cc * math.sin(half), (j % 2) * cc * math.cos(half), 0.0])
            h_in = _unit(ghost - c)
            symbols.append("H")
            coords.append(c + ch * h_in)
            nbr.append(h_in)
        b = -_unit(nbr[0] + nbr[1])
        for sgn in (1.0, -1.0):
            symbols.append("H")
            coords.append(c + ch * (b * math.cos(half) + sgn * ez * math.sin(half)))
    coords = np.array(coords)
    if jitter:
        coords = coords + np.random.default_rng(seed).normal(0.0, jitter, coords.shape)
    return _to_atoms(symbols, coords)


def c60(jitter: float = 0.01, seed: int = 0, bond66: float = 1.40, bond56: float = 1.45):
    """C60 truncated icosahedron: cut each icosahedron edge (length a) at x from
    both ends; pentagon edges = x (5-6 bonds), remaining edge middles = a - 2x."""
    phi = (1 + 5 ** 0.5) / 2
    ico = []
    for s1 in (1, -1):
        for s2 in (1, -1):
            ico += [(0, s1, s2 * phi), (s1, s2 * phi, 0), (s2 * phi, 0, s1)]
    ico = np.array(ico, dtype=float)
    a = bond66 + 2 * bond56
    ico *= a / 2.0  # icosahedron edge 2 -> a
    verts = []
    for i in range(12):
        for j in range(12):
            if i != j and abs(np.linalg.norm(ico[i] - ico[j]) - a) < 1e-6:
                verts.append(ico[i] + bond56 / a * (ico[j] - ico[i]))
    coords = np.array(verts)
    assert coords.shape == (60, 3)
    if jitter:
        coords = coords + np.random.default_rng(seed).normal(0.0, jitter, coords.shape)
    return _to_atoms(["C"] * 60, coords)


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(n: int, rng, oh: float = 0.96, hoh: float = 104.5, min_oo: float = 2.7):
    """(H2O)_n with random O positions (O-O >= min_oo) and orientations (bohr)."""
    half = math.radians(hoh) / 2
    mono = np.array([[0.0, 0.0, 0.0], [oh * math.sin(half), oh * math.cos(half), 0.0],
                     [-oh * math.sin(half), oh * math.cos(half), 0.0]])
    box = max(min_oo, (n * 30.0) ** (1.0 / 3.0))  # ~30 A^3 per molecule
    placed_o, symbols, coords = [], [], []
    tries = 0
    while len(placed_o) < n:
        tries += 1
        if tries > 100000:
            box *= 1.1
            tries = 0
        o = rng.uniform(0.0, box, 3)
        if any(np.linalg.norm(o - p) < min_oo for p in placed_o):
            continue
        w = mono @ _random_rotation(rng).T + o
        # intermolecular contacts no shorter than an H-bond: O...H >= 1.7 A, H...H >= 2.0 A
        if coords:
            old = np.asarray(coords)
            old_h = np.array([i % 3 != 0 for i in range(len(old))])
            too_close = False
            for j, r in enumerate(w):
                d = np.linalg.norm(old - r, axis=1)
                if d.min() < 1.7 or (j > 0 and d[old_h].min() < 2.0):
                    too_close = True
                    break
            if too_close:
                continue
        placed_o.append(o)
        for s, r in zip(["O", "H", "H"], w):
            symbols.append(s)
            coords.append(r)
    return _to_atoms(symbols, coords)


def water_cluster_set(count: int = 256, nmax: int = 16, seed: int = 0):
    """`count` clusters with n ~ U{1..nmax}."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(1, nmax + 1, size=count)
    return [water_cluster(int(k), rng) for k in sizes]


def write_xyz(path, atoms, comment="generated"):
    inv = {v: k for k, v in Z.items()}
    with open(path, "w") as f:
        f.write(f"{len(atoms)}\n{comment}\n")
        for zz, x, y, w in atoms:
            f.write(f"{inv[zz]} {x / ANGSTROM_TO_BOHR:.10f} {y / ANGSTROM_TO_BOHR:.10f} {w / ANGSTROM_TO_BOHR:.10f}\n")
