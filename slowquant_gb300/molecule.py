"""Molecule, atoms, shells and basis reading (host side).

Mirrors the reference's molecule layer so that code written against it keeps
working:

* ``_Molecule(molecule_file, molecular_charge_=0, distance_unit="bohr")``
  (slowquant/molecule/moleculeclass.py:12-80) with ``_set_basis_set``,
  ``shells``, ``number_bf``, ``number_shell``, ``number_electrons``,
  ``nuclear_repulsion``, ``atom_coordinates``, ``atom_charges``...;
* ``Shell`` (moleculeclass.py:269-301) with ``normalization[bf, prim]``;
* ``read_basis(atom_name, basis_set)`` (basis_reader.py:6-75) reading this
  package's JSON tables of published basis-set data.

Geometry, units and error behaviour follow the reference: Angstrom input is
scaled by 1.889725989, unknown units or formats raise ``ValueError``, and an
element missing from a basis raises ``ValueError``.
"""

from __future__ import annotations

import functools
import json
import os

import numpy as np

BASIS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basisset")
ANGSTROM_TO_BOHR = 1.889725989

_SYMBOLS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
    "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn"
).split()
CHARGE = {s: i + 1 for i, s in enumerate(_SYMBOLS)}
# Standard atomic weights as the reference tabulates them (slowquant/molecule/constants.py),
# used for the centre of mass (the origin of the multipole integrals).  Elements the
# reference gives no weight (Tc, Pm, Po, At, Rn) weigh 0 in the centre of mass, as there.
MASS = {
    "H": 1.008, "He": 4.002, "Li": 6.94, "Be": 9.012, "B": 10.81, "C": 12.011, "N": 14.007, "O": 15.999, "F":
    18.998, "Ne": 20.1797, "Na": 22.989, "Mg": 24.305, "Al": 26.981, "Si": 28.085, "P": 30.973, "S": 32.06,
    "Cl": 35.45, "Ar": 39.948, "K": 39.0983, "Ca": 40.078, "Sc": 44.955, "Ti": 47.867, "V": 50.9415, "Cr":
    51.9961, "Mn": 54.938, "Fe": 55.845, "Co": 58.933, "Ni": 58.6934, "Cu": 63.546, "Zn": 65.38, "Ga": 69.723,
    "Ge": 72.63, "As": 74.921, "Se": 78.971, "Br": 79.904, "Kr": 83.798, "Rb": 85.4678, "Sr": 87.62, "Y":
    88.905, "Zr": 91.224, "Nb": 92.906, "Mo": 95.95, "Ru": 101.07, "Rh": 102.905, "Pd": 106.42, "Ag": 107.8682,
    "Cd": 112.414, "In": 114.818, "Sn": 118.71, "Sb": 121.76, "Te": 127.6, "I": 126.904, "Xe": 131.293, "Cs":
    132.905, "Ba": 137.327, "La": 138.905, "Ce": 140.116, "Pr": 140.907, "Nd": 144.242, "Sm": 150.36, "Eu":
    151.964, "Gd": 157.25, "Tb": 158.925, "Dy": 162.5, "Ho": 164.93, "Er": 167.259, "Tm": 168.934, "Yb":
    173.045, "Lu": 174.9668, "Hf": 178.49, "Ta": 180.947, "W": 183.84, "Re": 186.207, "Os": 190.23, "Ir":
    192.217, "Pt": 195.084, "Au": 196.966, "Hg": 200.592, "Tl": 204.38, "Pb": 207.2, "Bi": 208.98,
}

# Cartesian component order per shell (basis_reader.py:50-70).
CARTESIAN = {
    "s": [[0, 0, 0]],
    "p": [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
    "d": [[2, 0, 0], [1, 1, 0], [1, 0, 1], [0, 2, 0], [0, 1, 1], [0, 0, 2]],
    "f": [[3, 0, 0], [2, 1, 0], [2, 0, 1], [1, 2, 0], [1, 1, 1], [1, 0, 2], [0, 3, 0], [0, 2, 1], [0, 1, 2],
          [0, 0, 3]],
}


def atom_to_properties(atom_name: str, atom_property: str) -> float:
    """Nuclear charge or mass of an element (slowquant/molecule/constants.py)."""
    if atom_property == "charge":
        return CHARGE[atom_name]
    if atom_property == "mass":
        return MASS.get(atom_name, 0.0)
    raise ValueError(f"unknown atom property {atom_property}")


def factorial2(number: float) -> float:
    """n!! as a float, 1 for n <= 0 (moleculefunctions.py:7-26)."""
    out = 1.0
    if number > 0:
        for i in range(int(number + 1) // 2):
            out *= number - 2 * i
    return out


def primitive_normalization(exponent: float, angular_moment) -> float:
    """moleculefunctions.py:29-47."""
    l, m, n = angular_moment
    return ((2 / np.pi) ** (3 / 4) * (2 ** (l + m + n) * exponent ** ((2 * l + 2 * m + 2 * n + 3) / 4))
            / (factorial2(2 * l - 1) * factorial2(2 * m - 1) * factorial2(2 * n - 1)) ** (1 / 2))


def contracted_normalization(exponents, coefficients, angular_moments) -> float:
    """moleculefunctions.py:50-88."""
    ax, ay, az = angular_moments
    e = np.asarray(exponents, dtype=np.float64)
    c = np.asarray(coefficients, dtype=np.float64)
    f = float(np.sum(np.outer(c, c) / np.add.outer(e, e) ** (ax + ay + az + 3 / 2)))
    f *= (np.pi ** (3 / 2) * factorial2(2 * ax - 1) * factorial2(2 * ay - 1) * factorial2(2 * az - 1)) / (
        2 ** (ax + ay + az))
    return f ** (-1 / 2)


@functools.lru_cache(maxsize=None)
def _basis_table(basis_set: str) -> dict:
    name = basis_set.replace("*", "_st_").lower()
    path = os.path.join(BASIS_DIR, name + ".json")
    if not os.path.exists(path):
        raise ValueError(f"Unknown basis set: {basis_set}")
    with open(path, encoding="UTF-8") as fh:
        return json.load(fh)["elements"]


def read_basis(atom_name: str, basis_set: str):
    """Exponents, contraction coefficients and Cartesian angular moments per shell."""
    table = _basis_table(basis_set)
    key = atom_name.lower()
    if key not in table:
        raise ValueError(f"Could not find request atom in basisset.\nBasisset: {basis_set}\nAtom: {atom_name}")
    exps, coefs, angs = [], [], []
    for sh in table[key]:
        if sh["l"] not in CARTESIAN:
            raise ValueError(f"None implemented angular moment: {sh['l']}")
        exps.append(np.array(sh["exponents"]))
        coefs.append(np.array(sh["coefficients"]))
        angs.append(np.array(CARTESIAN[sh["l"]]))
    return exps, coefs, angs


class Atom:
    def __init__(self, name: str, coordinate_, charge: int, mass_: float) -> None:
        self.atom_name = name
        self.coordinate = coordinate_
        self.nuclear_charge = charge
        self.mass = mass_


class Shell:
    """Contracted Cartesian shell with per-component normalisation (moleculeclass.py:269-301)."""

    def __init__(self, center_, exponents_, contraction_coefficients_, angular_moments_, bf_idx_: int,
                 origin_atom_: Atom):
        self.center = center_
        self.exponents = exponents_
        self.contraction_coefficients = contraction_coefficients_
        self.normalization = np.zeros((len(angular_moments_), len(exponents_)))
        self.origin_atom = origin_atom_
        for bf_i, ang in enumerate(angular_moments_):
            for i, e in enumerate(exponents_):
                self.normalization[bf_i, i] = primitive_normalization(e, ang)
            self.normalization[bf_i, :] *= contracted_normalization(
                exponents_, contraction_coefficients_ * self.normalization[bf_i, :], ang)
        self.angular_moments = angular_moments_
        self.bf_idx = np.array(range(bf_idx_, bf_idx_ + len(angular_moments_)))

    @property
    def angular_momentum(self) -> int:
        return int(np.max(self.angular_moments))

    def component_independent_coefficients(self) -> np.ndarray:
        """c_i x the part of N[bf, i] shared by every Cartesian component.

        N[bf, i] = g(alpha_i) / sqrt((2x-1)!!(2y-1)!!(2z-1)!!) with g common to
        the shell (the contracted factor of moleculefunctions.py:50-88 is the
        same for every component), so c_i N[0, i] sqrt((2l-1)!!) is g(alpha_i) c_i.
        """
        l0 = self.angular_moments[0]
        df0 = factorial2(2 * l0[0] - 1) * factorial2(2 * l0[1] - 1) * factorial2(2 * l0[2] - 1)
        return self.contraction_coefficients * self.normalization[0, :] * np.sqrt(df0)


class _Molecule:
    def __init__(self, molecule_file: str, molecular_charge_: int = 0, distance_unit: str = "bohr") -> None:
        self.molecular_charge = molecular_charge_
        self.shells: list[Shell] = []
        self.number_bf = 0
        if distance_unit.lower() == "angstrom":
            unit_factor = ANGSTROM_TO_BOHR
        elif distance_unit.lower() in ("au", "bohr"):
            unit_factor = 1.0
        else:
            raise ValueError(f"distance_unit not valid can be 'angstrom' or 'bohr'. Was given: {distance_unit}")
        if ".xyz" in molecule_file:
            with open(molecule_file, encoding="UTF-8") as fh:
                lines = fh.read().splitlines()[2:]
        elif ";" in molecule_file:
            lines = molecule_file.split(";")
        else:
            raise ValueError(
                "Does only support:\n    .xyz files for molecule coordinates.\n"
                "    A string with the elements and coordinates (; delimited)."
            )
        self.atoms: list[Atom] = []
        for line in lines:
            if len(line.strip()) == 0:
                continue
            f = line.split()
            self.atoms.append(Atom(
                f[0],
                np.array([float(f[1]) * unit_factor, float(f[2]) * unit_factor, float(f[3]) * unit_factor]),
                int(atom_to_properties(f[0], "charge")),
                atom_to_properties(f[0], "mass"),
            ))

    def _set_basis_set(self, basis_set: str) -> None:
        self.shells = []
        self.number_bf = 0
        self.basis_set = basis_set
        for atom in self.atoms:
            exps, coefs, angs = read_basis(atom.atom_name, basis_set)
            for e, c, a in zip(exps, coefs, angs):
                self.shells.append(Shell(atom.coordinate, e, c, a, self.number_bf, atom))
                self.number_bf += len(a)

    @property
    def atom_coordinates(self) -> np.ndarray:
        return np.array([a.coordinate for a in self.atoms], dtype=np.float64).reshape(-1, 3)

    @property
    def atom_charges(self) -> np.ndarray:
        return np.array([a.nuclear_charge for a in self.atoms], dtype=np.float64)

    @property
    def number_electrons(self) -> int:
        return int(sum(a.nuclear_charge for a in self.atoms) - self.molecular_charge)

    @property
    def number_electrons_alpha(self) -> int:
        return (self.number_electrons + 1) // 2

    @property
    def number_electrons_beta(self) -> int:
        return self.number_electrons // 2

    @property
    def nuclear_repulsion(self) -> float:
        """sum_{i<j} Z_i Z_j / R_ij (moleculeclass.py:167-184)."""
        Z = self.atom_charges
        R = self.atom_coordinates
        V = 0.0
        for i in range(len(Z)):
            for j in range(i + 1, len(Z)):
                V += Z[i] * Z[j] / np.einsum("k->", (R[i] - R[j]) ** 2) ** 0.5
        return V

    @property
    def center_of_mass(self) -> np.ndarray:
        m = np.array([a.mass for a in self.atoms])
        return np.einsum("ij,i->j", self.atom_coordinates, m) / np.einsum("i->", m)

    @property
    def basis_function_labels(self) -> list[str]:
        return [f"{s.origin_atom.atom_name} {a}" for s in self.shells for a in s.angular_moments]

    @property
    def number_shell(self) -> int:
        return len(self.shells)
