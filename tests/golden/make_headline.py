"""Oracle fixtures for the two headline water clusters -- TEST INFRASTRUCTURE.

This script runs the oracle (``oracle/sq_oracle.c`` for the integrals and the
direct J/K, ``oracle/oracle.py`` for the SCF loop of
slowquant/hartreefock/hartreefock_in_memory.py:7-94 with the DIIS of
slowquant/hartreefock/diis.py:4-66), not the reference itself: the reference's
pure-Python path would need about 35 h for the smaller cluster.  The oracle is
pinned to the reference's own outputs by ``make_golden.py`` and
``tests/test_oracle_golden.py``.

Systems (seeded, ``slowquant_gb300.systems.water_cluster``), both cc-pVDZ
(Cartesian), Schwarz threshold 1e-12, SCF thresholds dE 1e-9 and rmsd 1e-9,
Boys function to full double precision (the oracle's accurate mode):

* ``headline_c2``: (H2O)_8 in a 9 A cube, seed 8 (200 basis functions);
* ``headline_c3``: (H2O)_16 in an 11 A cube, seed 16 (400 basis functions).

Each ``.npz`` holds the converged SCF energy (electronic, and E_nuc), the
per-iteration energies, the occupied coefficients C_occ of the converged
density D = 2 C_occ C_occ^T, and J, K at that D through size-independent
checks: J @ R and K @ R for R = default_rng(1234).standard_normal((nbf, 8)),
their diagonals, tr(D J), tr(D K) and E(D) = 1/2 tr D (H + F(D)) with
F = H + J - K/2 (one Fock build, no DIIS).

Run:  python tests/golden/make_headline.py [--only headline_c2 ...] [--threads N]
(about 3 minutes for c2 and 16 for c3 on 8 cores).
"""

from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from slowquant_gb300 import systems  # noqa: E402

SYSTEMS = {
    "headline_c2": (8, 9.0, 8),
    "headline_c3": (16, 11.0, 16),
}
SCREEN = 1e-12
PROJ_SEED, NPROJ = 1234, 8


def projections(nbf: int) -> np.ndarray:
    return np.random.default_rng(PROJ_SEED).standard_normal((nbf, NPROJ))


def make(name: str, nthreads: int) -> None:
    nw, box, seed = SYSTEMS[name]
    geom = systems.water_cluster(nw, box, seed)
    o = O.OracleMolecule(geom, "cc-pvdz", "angstrom")
    t0 = time.time()
    S, T, V = o.one_electron()
    O.lib().sqo_set_boys_mode(1)
    cs = o.schwarz(nthreads)
    O.lib().sqo_set_boys_mode(0)
    nbuild = [0]

    def jk(D):
        t = time.time()
        J, K = o.jk_direct(D, SCREEN, nthreads, accurate=True, cs=cs)
        nbuild[0] += 1
        print(f"  {name}: J/K build {nbuild[0]} in {time.time() - t:.1f} s", flush=True)
        return J, K

    E, C, F, D, energies = O.run_hartree_fock(S, T, V, jk, o.number_electrons, 1e-9, 1e-9, 100, True)
    nocc = o.number_electrons // 2
    Cocc = np.ascontiguousarray(C[:, :nocc])
    Dc = 2 * Cocc @ Cocc.T
    J, K = jk(Dc)
    H = T + V
    Fd = H + J - 0.5 * K
    R = projections(o.nbf)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        geometry=np.array(geom), nbf=o.nbf, E_hf=E, E_nuc=o.nuclear_repulsion, energies=np.array(energies),
        C_occ=Cocc, JR=J @ R, KR=K @ R, J_diag=np.diag(J).copy(), K_diag=np.diag(K).copy(),
        trDJ=np.einsum("ij,ij->", Dc, J), trDK=np.einsum("ij,ij->", Dc, K),
        E_at_D=0.5 * np.einsum("ij,ij->", Dc, H + Fd), screen=SCREEN, seed=seed, box=box, waters=nw,
    )
    print(f"{name}: nbf {o.nbf}, E_hf {E:.12f}, {len(energies)} iterations, {time.time() - t0:.0f} s", flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=None)
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    for name in SYSTEMS:
        if args.only is None or name in args.only:
            make(name, args.threads)


if __name__ == "__main__":
    main()
