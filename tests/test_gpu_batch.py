"""Batched SCF over independent molecules of uneven size against single-molecule SCF."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mols(sizes, basis="6-31G*"):
    from slowquant_gb300 import systems
    from slowquant_gb300.molecule import _Molecule

    out = []
    for i, n in enumerate(sizes):
        box = 9.0 * (n / 8.0) ** (1.0 / 3.0) + 1.0
        m = _Molecule(systems.water_cluster(n, box, seed=100 + i), 0, "angstrom")
        m._set_basis_set(basis)
        out.append(m)
    return out


def _single_energy(m):
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.hartreefock import DirectJK, run_hartree_fock
    from slowquant_gb300.logger import _Logger

    eng = IntegralEngine(m)
    S, T, V = eng.one_electron()
    log = _Logger()
    log.print_output = False
    return run_hartree_fock(S, T, V, DirectJK(eng), m.number_electrons, log, 1e-10, 1e-10, 100, True)[0]


@pytest.mark.parametrize("use_graphs", [False, True])
def test_batch_energies_match_single_molecule(gpu_lib, use_graphs):
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    sizes = [2, 1, 3, 1, 2]
    mols = _mols(sizes)
    be = BatchEngine(mols)
    E = BatchSCF(be, "fp64", use_graphs=use_graphs).run(1e-10, 1e-10)
    ref = np.array([_single_energy(m) for m in mols])
    np.testing.assert_allclose(E, ref, atol=1e-8)


def test_batch_one_electron_blocks(gpu_lib):
    from slowquant_gb300.batch import BatchEngine
    from slowquant_gb300.engine import IntegralEngine

    mols = _mols([1, 2])
    be = BatchEngine(mols)
    S, T, V = be.one_electron()
    for mi, m in enumerate(be.mols):
        n = m.number_bf
        blk = slice(be.mol_base[mi], be.mol_base[mi] + n * n)
        Sr, Tr, Vr = IntegralEngine(m).one_electron()
        np.testing.assert_allclose(S[blk].view(n, n).cpu().numpy(), Sr.cpu().numpy(), atol=1e-12)
        np.testing.assert_allclose(T[blk].view(n, n).cpu().numpy(), Tr.cpu().numpy(), atol=1e-12)
        np.testing.assert_allclose(V[blk].view(n, n).cpu().numpy(), Vr.cpu().numpy(), atol=1e-11)


def test_batch_mixed_precision(gpu_lib):
    from slowquant_gb300.batch import BatchEngine, BatchSCF

    mols = _mols([3, 2, 4])
    be = BatchEngine(mols)
    E64 = BatchSCF(be, "fp64").run()
    scf = BatchSCF(be, "mixed", fp32_threshold=1e-4)
    Em = scf.run()
    assert scf.builds[0] == "mixed" and scf.builds[-1] == "fp64"
    assert np.max(np.abs(Em - E64)) < 1e-6
