"""Route code written against SlowQuant's module names to this package.

``install()`` registers this package's modules under the names SlowQuant's
own code and tests import (``slowquant.SlowQuant``,
``slowquant.molecularintegrals.integralclass`` ... ), so that
``import slowquant.SlowQuant as sq`` gives the GPU implementation with the
reference's classes, functions and signatures.  ``uninstall(saved)`` puts
back whatever those names held before.  Call ``install()`` before anything
imports ``slowquant``.
"""

from __future__ import annotations

import sys
import types


def _aliases() -> dict:
    from . import SlowQuant, electronrepulsion, hartreefock, integralclass, integralfunctions, logger, molecule

    def package(name: str, **children) -> types.ModuleType:
        m = types.ModuleType(name)
        m.__path__ = []  # a package: submodules resolve through sys.modules
        for k, v in children.items():
            setattr(m, k, v)
        return m

    mi = package("slowquant.molecularintegrals", integralclass=integralclass, electronrepulsion=electronrepulsion,
                 integralfunctions=integralfunctions)
    hf = package("slowquant.hartreefock", hartreefock_in_memory=hartreefock, diis=hartreefock,
                 hartreefockclass=hartreefock, unrestricted_hartreefock_in_memory=hartreefock)
    mol = package("slowquant.molecule", moleculeclass=molecule, basis_reader=molecule, moleculefunctions=molecule)
    top = package("slowquant", SlowQuant=SlowQuant, molecularintegrals=mi, hartreefock=hf, molecule=mol,
                  logger=logger)
    return {
        "slowquant": top,
        "slowquant.SlowQuant": SlowQuant,
        "slowquant.logger": logger,
        "slowquant.molecularintegrals": mi,
        "slowquant.molecularintegrals.integralclass": integralclass,
        "slowquant.molecularintegrals.electronrepulsion": electronrepulsion,
        "slowquant.molecularintegrals.integralfunctions": integralfunctions,
        "slowquant.hartreefock": hf,
        "slowquant.hartreefock.hartreefock_in_memory": hartreefock,
        "slowquant.hartreefock.unrestricted_hartreefock_in_memory": hartreefock,
        "slowquant.hartreefock.diis": hartreefock,
        "slowquant.hartreefock.hartreefockclass": hartreefock,
        "slowquant.molecule": mol,
        "slowquant.molecule.moleculeclass": molecule,
        "slowquant.molecule.basis_reader": molecule,
        "slowquant.molecule.moleculefunctions": molecule,
    }


def install() -> dict:
    """Register the aliases; returns the previous sys.modules entries (for uninstall)."""
    new = _aliases()
    saved = {k: sys.modules.get(k) for k in new}
    sys.modules.update(new)
    return saved


def uninstall(saved: dict) -> None:
    for k, v in saved.items():
        if v is None:
            sys.modules.pop(k, None)
        else:
            sys.modules[k] = v
