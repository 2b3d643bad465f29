"""Facade with the reference's entry points (slowquant/SlowQuant.py:7-49)."""

from __future__ import annotations

from .hartreefock import _HartreeFock
from .integralclass import _Integral
from .logger import _Logger
from .molecule import _Molecule


class SlowQuant:
    def __init__(self) -> None:
        self.molecule: _Molecule
        self.integral: _Integral
        self.hartree_fock: _HartreeFock
        self.logger = _Logger()

    def set_molecule(self, molecule_file: str, molecular_charge: int = 0, distance_unit: str = "bohr",
                     basis_set: str | None = None, spherical: bool = False) -> None:
        self.molecule = _Molecule(molecule_file, molecular_charge, distance_unit)
        if basis_set is not None:
            self.molecule._set_basis_set(basis_set)
            self.integral = _Integral(self.molecule, spherical)

    def set_basis_set(self, basis_set: str, spherical: bool = False) -> None:
        """``spherical=True`` (not in the reference) works in real solid harmonics."""
        if hasattr(self, "molecule"):
            self.molecule._set_basis_set(basis_set)
            self.integral = _Integral(self.molecule, spherical)
        else:
            self.logger.add_to_log("Cannot set basis set, molecule is not defined.", is_warning=True)

    def init_hartree_fock(self) -> None:
        self.hartree_fock = _HartreeFock(self.molecule, self.integral)
