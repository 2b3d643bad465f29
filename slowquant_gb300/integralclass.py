"""Integral class with the reference's lazy-property API
(slowquant/molecularintegrals/integralclass.py:16-108), backed by the GPU engine.

Properties return numpy float64 arrays owned by the object (cached unless
``force_recompute``), exactly like the reference; ``engine`` exposes the device
engine for the integral-direct Fock build.
"""

from __future__ import annotations

import numpy as np

from .engine import IntegralEngine
from .logger import _Logger
from .molecule import _Molecule


def engine_for(mol: _Molecule) -> IntegralEngine:
    """The molecule's device engine, rebuilt when its basis set changes."""
    eng = getattr(mol, "_gb300_engine", None)
    if eng is None or eng.mol is not mol or getattr(mol, "_gb300_shells_id", None) != id(mol.shells):
        eng = IntegralEngine(mol)
        mol._gb300_engine = eng
        mol._gb300_shells_id = id(mol.shells)
    return eng


class _Integral:
    def __init__(self, molecule_object_: _Molecule) -> None:
        self.molecule_object = molecule_object_
        self.store_1e_int = True
        self.store_2e_int = True
        self.logger = _Logger()
        nbf = self.molecule_object.number_bf
        if nbf**4 * 8 / 10**9 > 6:
            self.logger.add_to_log(
                f"Storing 2-electron integrals in memory will use approx {nbf**4 * 8 / 10**9:3.1f} GB",
                is_warning=True,
            )
        self.force_recompute = False
        self._overlap_int = None
        self._kineticenergy_int = None
        self._nuclearattraction_int = None
        self._electronrepulsion_int = None
        self.engine = engine_for(self.molecule_object)
        # Integral screening: the Schwarz matrix is formed eagerly, as in the reference.
        self._cauchy_schwarz_matrix = self.engine.schwarz_matrix() if self.engine.eri_supported() else None
        self.cauchy_schwarz_threshold = 10**-12
        self._one_e_dev = None

    def one_electron_device(self):
        """(S, T, V) as FP64 device tensors."""
        if self._one_e_dev is None or self.force_recompute:
            self._one_e_dev = self.engine.one_electron()
        return self._one_e_dev

    def _one_e(self, idx: int) -> np.ndarray:
        return self.one_electron_device()[idx].cpu().numpy()

    @property
    def overlap_matrix(self) -> np.ndarray:
        if self.store_1e_int:
            if self._overlap_int is None or self.force_recompute:
                self._overlap_int = self._one_e(0)
            return self._overlap_int
        return self._one_e(0)

    @property
    def kinetic_energy_matrix(self) -> np.ndarray:
        if self.store_1e_int:
            if self._kineticenergy_int is None or self.force_recompute:
                self._kineticenergy_int = self._one_e(1)
            return self._kineticenergy_int
        return self._one_e(1)

    @property
    def nuclear_attraction_matrix(self) -> np.ndarray:
        if self.store_1e_int:
            if self._nuclearattraction_int is None or self.force_recompute:
                self._nuclearattraction_int = self._one_e(2)
            return self._nuclearattraction_int
        return self._one_e(2)

    def _eri(self) -> np.ndarray:
        return self.engine.eri_dense(self.cauchy_schwarz_threshold).cpu().numpy()

    @property
    def electron_repulsion_tensor(self) -> np.ndarray:
        if self.store_2e_int:
            if self._electronrepulsion_int is None or self.force_recompute:
                self._electronrepulsion_int = self._eri()
            return self._electronrepulsion_int
        return self._eri()

    def get_multipole_matrix(self, multipole_order) -> np.ndarray:
        """Only the zeroth moment (the overlap) is provided on this path."""
        if np.any(np.asarray(multipole_order) != 0):
            raise NotImplementedError("multipole integrals beyond the overlap are outside this package")
        return self.overlap_matrix.copy()
