"""GB300-native SlowQuant integral / restricted Hartree-Fock hot path.

Entry points mirror the reference: ``SlowQuant`` (facade), ``_Integral``,
``electron_repulsion_integral_driver``, ``get_cauchy_schwarz_matrix``,
``run_hartree_fock``, ``DIIS``, ``_HartreeFock``.  Compute runs in the CUDA
library ``libsqgb300.so`` (built by ``slowquant_gb300.build``); there is no
CPU fallback.
"""

from .molecule import Atom, Shell, _Molecule, read_basis  # noqa: F401

__all__ = ["Atom", "Shell", "_Molecule", "read_basis"]
