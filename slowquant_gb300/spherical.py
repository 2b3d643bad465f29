"""Real solid-harmonic (spherical) basis functions on top of the Cartesian shells.

The reference builds Cartesian shells only (slowquant/molecule/basis_reader.py:
50-70: 6 d and 10 f components, each normalised on its own,
moleculeclass.py:269-301).  Published results for cc-pVXZ bases use the
2l+1 real solid harmonics per shell instead (24 functions per water in
cc-pVDZ rather than 25).  This module gives the block-diagonal matrix T
(n_cartesian x n_spherical) whose columns are the normalised solid harmonics
written in this package's normalised Cartesian functions, so that

    S_sph = T^T S T,   D_cart = T D_sph T^T,   J_sph = T^T J(D_cart) T,

and the integral kernels keep working on Cartesian shells.

Column order per shell: m = -l .. l with the polynomials (up to normalisation)
  d: xy, yz, 2z^2 - x^2 - y^2, xz, x^2 - y^2;
  f: 3x^2 y - y^3, xyz, y(4z^2 - x^2 - y^2), z(2z^2 - 3x^2 - 3y^2),
     x(4z^2 - x^2 - y^2), z(x^2 - y^2), x^3 - 3xy^2.
s and p shells are unchanged (identity blocks, p in the order x, y, z).

Normalisation uses the angular integrals of Cartesian monomials over a
common radial factor: <x^a y^b z^c> is proportional to (a-1)!!(b-1)!!(c-1)!!
for even a, b, c and zero otherwise, so each column has unit norm in the
metric of the shell's normalised Cartesian functions.
"""

from __future__ import annotations

import numpy as np

from .molecule import CARTESIAN, factorial2

# Solid-harmonic polynomials as {(a, b, c): coefficient} of x^a y^b z^c.
_SOLID = {
    2: [
        {(1, 1, 0): 1.0},
        {(0, 1, 1): 1.0},
        {(0, 0, 2): 2.0, (2, 0, 0): -1.0, (0, 2, 0): -1.0},
        {(1, 0, 1): 1.0},
        {(2, 0, 0): 1.0, (0, 2, 0): -1.0},
    ],
    3: [
        {(2, 1, 0): 3.0, (0, 3, 0): -1.0},
        {(1, 1, 1): 1.0},
        {(0, 1, 2): 4.0, (2, 1, 0): -1.0, (0, 3, 0): -1.0},
        {(0, 0, 3): 2.0, (2, 0, 1): -3.0, (0, 2, 1): -3.0},
        {(1, 0, 2): 4.0, (3, 0, 0): -1.0, (1, 2, 0): -1.0},
        {(2, 0, 1): 1.0, (0, 2, 1): -1.0},
        {(3, 0, 0): 1.0, (1, 2, 0): -3.0},
    ],
}


def _monomial_overlap(p, q) -> float:
    """Angular factor of <x^{p} | x^{q}> shared by all monomials of one shell (radial part common)."""
    out = 1.0
    for e in np.asarray(p) + np.asarray(q):
        if e % 2:
            return 0.0
        out *= factorial2(e - 1)
    return out


def cart_to_sph(l: int) -> np.ndarray:
    """(ncart(l), 2l+1) block for one shell, in the package's Cartesian order."""
    if l <= 1:
        return np.eye((l + 1) * (l + 2) // 2)
    cart = [tuple(c) for c in CARTESIAN["spdf"[l]]]
    G = np.array([[_monomial_overlap(p, q) for q in cart] for p in cart])
    scale = np.sqrt(np.diag(G))  # monomial m_i = scale_i * (normalised Cartesian function i)
    out = np.zeros((len(cart), 2 * l + 1))
    for m, poly in enumerate(_SOLID[l]):
        c = np.array([poly.get(p, 0.0) for p in cart])
        out[:, m] = c * scale / np.sqrt(c @ G @ c)
    return out


def transform_matrix(shells) -> np.ndarray:
    """Block-diagonal T (n_cartesian, n_spherical) for a list of shells (``Shell`` objects)."""
    blocks = [cart_to_sph(int(np.sum(s.angular_moments[0]))) for s in shells]
    ncart = sum(b.shape[0] for b in blocks)
    nsph = sum(b.shape[1] for b in blocks)
    T = np.zeros((ncart, nsph))
    r = c = 0
    for b in blocks:
        T[r:r + b.shape[0], c:c + b.shape[1]] = b
        r += b.shape[0]
        c += b.shape[1]
    return T


def n_spherical(shells) -> int:
    return int(sum(2 * int(np.sum(s.angular_moments[0])) + 1 for s in shells))
