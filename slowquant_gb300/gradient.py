"""RHF nuclear gradients through torch.autograd.

``rhf_energy(coords, symbols, basis)`` returns the total RHF energy (electronic
+ nuclear repulsion, Eh) as a differentiable scalar of the nuclear coordinates
(bohr, shape (natom, 3)).  The forward pass runs the integral-direct FP64 SCF
on the GPU; the backward pass calls the adjoint derivative kernels
(sq_grad_1e / sq_grad_2e), which contract the derivative integrals with the
density, the energy-weighted density and the two-particle density on the fly.
The reference has no gradients; its energies are the finite-difference check.
"""

from __future__ import annotations

import numpy as np
import torch

from .engine import IntegralEngine
from .hartreefock import DirectJK, run_hartree_fock
from .logger import _Logger
from .molecule import _Molecule


def molecule_from_coords(symbols, coords_bohr, basis: str) -> _Molecule:
    geom = ";".join(f"{s} {x:.17g} {y:.17g} {z:.17g}" for s, (x, y, z) in zip(symbols, np.asarray(coords_bohr)))
    m = _Molecule(geom, 0, "bohr")
    m._set_basis_set(basis)
    return m


def scf_energy(mol: _Molecule, threshold: float = 1e-12, conv: float = 1e-10, engine: IntegralEngine | None = None):
    """Converged FP64 RHF: (E_total, D device tensor, engine)."""
    eng = engine or IntegralEngine(mol)
    S, T, V = eng.one_electron()
    log = _Logger()
    log.print_output = False
    E, C, F, D = run_hartree_fock(S, T, V, DirectJK(eng, threshold, "fp64"), mol.number_electrons, log, conv,
                                  conv, 200, True)
    return E + mol.nuclear_repulsion, torch.tensor(D, device=eng.device), eng


class _RHFEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coords, symbols, basis, threshold, conv):
        mol = molecule_from_coords(symbols, coords.detach().cpu().numpy(), basis)
        E, D, eng = scf_energy(mol, threshold, conv)
        ctx.state = (eng, D, threshold)
        return torch.tensor(E, dtype=coords.dtype, device=coords.device)

    @staticmethod
    def backward(ctx, grad_out):
        eng, D, threshold = ctx.state
        g = torch.tensor(eng.nuclear_gradient(D, threshold), dtype=grad_out.dtype, device=grad_out.device)
        return grad_out * g, None, None, None, None


def rhf_energy(coords: torch.Tensor, symbols, basis: str, threshold: float = 1e-12, conv: float = 1e-10):
    """Differentiable total RHF energy of the nuclear coordinates (bohr)."""
    return _RHFEnergy.apply(coords, list(symbols), basis, threshold, conv)


def rhf_gradient(mol: _Molecule, threshold: float = 1e-12, conv: float = 1e-10) -> np.ndarray:
    """dE_total/dR (natom x 3, Eh/bohr) for a molecule with its basis set."""
    E, D, eng = scf_energy(mol, threshold, conv)
    return eng.nuclear_gradient(D, threshold)
