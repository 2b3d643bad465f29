"""Seeded synthetic molecules used by the benchmark and the tests.

Geometry strings use the reference's ``;``-separated atom-line format
(slowquant/molecule/moleculeclass.py:55-76) in Angstrom unless stated.

* ``water_monomer`` -- O at the origin, O-H 0.96 A, H-O-H 104.5 deg.
* ``water_cluster(n, box, seed)`` -- n rigid monomers at uniform random
  positions in a cube of edge ``box`` A with uniformly random orientations
  (random unit quaternion); a placement is rejected while any O-O distance is
  below 2.7 A.  Seeds are recorded by the caller.
* ``hydrogen_chain(n, seed)`` -- linear H_n with bond lengths uniform in
  [0.7, 1.1] A.
* ``octane()`` -- all-anti n-octane C8H18 (C-C 1.53 A, C-H 1.09 A,
  tetrahedral angles).
"""

from __future__ import annotations

import numpy as np

OH = 0.96
HOH_DEG = 104.5


def _water_local() -> np.ndarray:
    half = np.deg2rad(HOH_DEG) / 2.0
    return np.array([
        [0.0, 0.0, 0.0],
        [OH * np.sin(half), OH * np.cos(half), 0.0],
        [-OH * np.sin(half), OH * np.cos(half), 0.0],
    ])


def _fmt(symbols, xyz) -> str:
    return ";".join(f"{s} {x:.12f} {y:.12f} {z:.12f}" for s, (x, y, z) in zip(symbols, xyz))


def water_monomer() -> str:
    return _fmt(["O", "H", "H"], _water_local())


def _quat_to_matrix(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def water_cluster(n: int, box: float, seed: int, min_oo: float = 2.7, max_tries: int = 100000) -> str:
    """Seeded (H2O)_n cluster in a cube of edge ``box`` Angstrom."""
    rng = np.random.default_rng(seed)
    local = _water_local()
    oxygens: list[np.ndarray] = []
    symbols: list[str] = []
    coords: list[np.ndarray] = []
    tries = 0
    while len(oxygens) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"could not place {n} waters in a {box} A cube")
        pos = rng.uniform(0.0, box, 3)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        if any(np.linalg.norm(pos - o) < min_oo for o in oxygens):
            continue
        rot = _quat_to_matrix(q)
        oxygens.append(pos)
        for s, r in zip(["O", "H", "H"], local):
            symbols.append(s)
            coords.append(pos + rot @ r)
    return _fmt(symbols, np.array(coords))


def hydrogen_chain(n: int, seed: int, lo: float = 0.7, hi: float = 1.1) -> str:
    rng = np.random.default_rng(seed)
    bonds = rng.uniform(lo, hi, n - 1)
    x = np.concatenate([[0.0], np.cumsum(bonds)])
    return _fmt(["H"] * n, np.stack([x, np.zeros(n), np.zeros(n)], axis=1))


def octane(cc: float = 1.53, ch: float = 1.09) -> str:
    """All-anti n-octane: zig-zag carbon backbone in the xy plane."""
    tet = np.arccos(-1.0 / 3.0)
    half = tet / 2.0
    dx, dy = cc * np.sin(half), cc * np.cos(half)
    carbons = np.array([[i * dx, (i % 2) * dy, 0.0] for i in range(8)])
    symbols = ["C"] * 8
    coords = [c for c in carbons]
    for i, c in enumerate(carbons):
        # bisector pointing away from the backbone neighbours
        nb = [carbons[j] for j in (i - 1, i + 1) if 0 <= j < 8]
        away = sum((c - m) / np.linalg.norm(c - m) for m in nb)
        away /= np.linalg.norm(away)
        if len(nb) == 2:
            # two H in the plane perpendicular to the backbone plane
            for sgn in (1.0, -1.0):
                d = np.cos(half) * away + sgn * np.sin(half) * np.array([0.0, 0.0, 1.0])
                coords.append(c + ch * d / np.linalg.norm(d))
                symbols.append("H")
        else:
            # terminal CH3: one H anti to the C-C bond in the plane, two out of plane
            bond = (c - nb[0]) / np.linalg.norm(c - nb[0])
            perp = np.cross(bond, np.array([0.0, 0.0, 1.0]))
            perp /= np.linalg.norm(perp)
            if np.dot(perp, np.array([0.0, 1.0, 0.0]) * (1 if i == 0 else -1)) > 0:
                perp = -perp
            ca, sa = np.cos(np.pi - tet), np.sin(np.pi - tet)
            d0 = ca * bond + sa * perp
            coords.append(c + ch * d0)
            symbols.append("H")
            for ang in (2 * np.pi / 3, -2 * np.pi / 3):
                # rotate d0 about the bond axis
                k = bond
                v = d0
                vr = v * np.cos(ang) + np.cross(k, v) * np.sin(ang) + k * np.dot(k, v) * (1 - np.cos(ang))
                coords.append(c + ch * vr)
                symbols.append("H")
    return _fmt(symbols, np.array(coords))
