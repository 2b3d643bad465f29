"""Module-level ERI entry points of slowquant/molecularintegrals/electronrepulsion.py."""

from __future__ import annotations

import numpy as np

from .integralclass import engine_for
from .molecule import _Molecule


def electron_repulsion_integral_driver(mol_obj: _Molecule, cauchy_schwarz_matrix: np.ndarray | None = None,
                                       cauchy_schwarz_threshold: float = 10**-10) -> np.ndarray:
    """Dense (nbf,)*4 ERI tensor (electronrepulsion.py:11-104).

    With ``cauchy_schwarz_matrix`` a quartet is skipped when
    cs[i,j] * cs[k,l] < threshold; without it every quartet is computed.
    """
    eng = engine_for(mol_obj)
    if cauchy_schwarz_matrix is None:
        return eng.eri_dense_with_q(None, 0.0).cpu().numpy()
    cs = np.asarray(cauchy_schwarz_matrix, dtype=np.float64)
    q = cs[eng.pair_shells[:, 0], eng.pair_shells[:, 1]]
    return eng.eri_dense_with_q(q, cauchy_schwarz_threshold).cpu().numpy()


def get_cauchy_schwarz_matrix(mol_obj: _Molecule) -> np.ndarray:
    """Shell-pair Cauchy-Schwarz matrix sqrt(max (ij|ij)) (electronrepulsion.py:300-339)."""
    return engine_for(mol_obj).schwarz_matrix()
