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
    """``spherical=True`` (an option the reference does not have) returns every
    matrix and the ERI tensor in real solid harmonics (2l+1 functions per
    shell, ``slowquant_gb300.spherical``); the default is the reference's
    Cartesian basis."""

    def __init__(self, molecule_object_: _Molecule, spherical: bool = False) -> None:
        self.molecule_object = molecule_object_
        self.spherical = bool(spherical)
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
        self._T = None

    @property
    def number_bf(self) -> int:
        """Basis functions of the matrices this object returns (spherical or Cartesian)."""
        return self.cart_to_sph.shape[1] if self.spherical else self.molecule_object.number_bf

    @property
    def cart_to_sph(self):
        """(n_cartesian, n_spherical) FP64 device matrix of the solid-harmonic transform."""
        if self._T is None:
            import torch

            from .spherical import transform_matrix

            self._T = torch.tensor(transform_matrix(self.molecule_object.shells), dtype=torch.float64,
                                   device=self.engine.device)
        return self._T

    def one_electron_device(self):
        """(S, T, V) as FP64 device tensors (in solid harmonics when ``spherical``)."""
        if self._one_e_dev is None or self.force_recompute:
            mats = self.engine.one_electron()
            if self.spherical:
                Tm = self.cart_to_sph
                mats = tuple(Tm.T @ M @ Tm for M in mats)
            self._one_e_dev = mats
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
        V = self.engine.eri_dense(self.cauchy_schwarz_threshold)
        if self.spherical:
            import torch

            Tm = self.cart_to_sph
            V = torch.einsum("pqrs,pi->iqrs", V, Tm)
            V = torch.einsum("iqrs,qj->ijrs", V, Tm)
            V = torch.einsum("ijrs,rk->ijks", V, Tm)
            V = torch.einsum("ijks,sl->ijkl", V, Tm)
        return V.cpu().numpy()

    @property
    def electron_repulsion_tensor(self) -> np.ndarray:
        if self.store_2e_int:
            if self._electronrepulsion_int is None or self.force_recompute:
                self._electronrepulsion_int = self._eri()
            return self._electronrepulsion_int
        return self._eri()

    def get_multipole_matrix(self, multipole_order) -> np.ndarray:
        """Multipole integrals of Cartesian orders (ex, ey, ez) about the centre of mass
        (integralclass.py:99-108, multipole.py:10-135); (0, 0, 0) is the overlap."""
        M = self.engine.multipole(np.asarray(multipole_order, dtype=np.int64))
        if self.spherical:
            Tm = self.cart_to_sph
            M = Tm.T @ M @ Tm
        return M.cpu().numpy()
