"""f shells (cc-pVTZ) on the block kernel against the reference's golden blocks and the oracle.

The reference reads f shells (basis_reader.py:50-70) and its integral code is
generic in l; cc-pVTZ puts f shells on O.  Tolerances as for s/p/d: integrals
1e-10 absolute, energies 1e-8 Eh against the oracle's SCF on the oracle's own
tensor, FP32 paths within the FP32 error scale.
"""


import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def _mol(geom, basis, unit):
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(geom, 0, unit)
    m._set_basis_set(basis)
    return m


def _engine(geom, basis, unit):
    from slowquant_gb300.engine import IntegralEngine

    return IntegralEngine(_mol(geom, basis, unit))


def _random_density(n, seed):
    rng = np.random.default_rng(seed)
    C = rng.normal(size=(n, max(1, n // 3))) / np.sqrt(n)
    return 2 * C @ C.T


@pytest.fixture(scope="module")
def h2o2(gpu_lib, golden_energies):
    e = golden_energies["h2o2_ccpvtz_f"]
    return e, _engine(e["geometry"], e["basis"], e["unit"])


def test_boys_high_order_grid(gpu_lib):
    """The high-order grid of the f classes vs the exact series; the reference formula to n = 22."""
    import torch

    from slowquant_gb300 import _lib

    eng = _engine("H 0 0 0;H 0 0 1.4", "sto-3g", "bohr")
    z = np.concatenate([[0.0, 1e-14, 1e-9, 1e-4], np.linspace(0.001, 75, 1501), [59.99, 60.0, 60.01, 100.0, 1e4]])

    def gpu(nmax, mode):
        zt = torch.tensor(z, dtype=torch.float64, device="cuda")
        out = torch.zeros((len(z), nmax + 1), dtype=torch.float64, device="cuda")
        _lib.check(_lib.lib().sq_boys(nmax, zt.data_ptr(), len(z), eng.tab64.data_ptr(), mode, out.data_ptr(),
                                      _lib.stream_handle()), "sq_boys")
        return out.cpu().numpy()

    def oracle(nmax, mode):
        O.lib().sqo_set_boys_mode(mode)
        try:
            return np.array([[O.boys(n, zz) for n in range(nmax + 1)] for zz in z])
        finally:
            O.lib().sqo_set_boys_mode(0)

    # exact F_n: the series below z = 1, else Gamma(n+1/2) P(n+1/2, z) / (2 z^{n+1/2})
    # (an asymptote from z = 40 on would be 4e-7 off at n = 12 there)
    from scipy.special import gamma, gammainc

    exact = oracle(16, 1)
    big = z > 1.0
    for n in range(17):
        exact[big, n] = gamma(n + 0.5) * gammainc(n + 0.5, z[big]) / (2 * z[big] ** (n + 0.5))
    # beyond z = 60 the asymptote drops a term below 2e-13 (n <= 13) / 1e-11 (n <= 16) relative
    hi = gpu(16, 2)
    np.testing.assert_allclose(hi, exact, rtol=1e-11, atol=1e-300)
    np.testing.assert_allclose(hi[:, :14], exact[:, :14], rtol=2e-13, atol=1e-300)
    inside = z < 60.0
    np.testing.assert_allclose(hi[inside], exact[inside], rtol=5e-14, atol=1e-300)
    np.testing.assert_allclose(gpu(22, 1), oracle(22, 0), rtol=1e-13, atol=1e-300)
    # orders beyond the grids are refused
    out = torch.zeros(len(z) * 30, dtype=torch.float64, device="cuda")
    zt = torch.tensor(z, dtype=torch.float64, device="cuda")
    assert _lib.lib().sq_boys(17, zt.data_ptr(), len(z), eng.tab64.data_ptr(), 2, out.data_ptr(),
                              _lib.stream_handle()) == _lib.SQ_ERR_ARG
    assert _lib.lib().sq_boys(9, zt.data_ptr(), len(z), eng.tab64.data_ptr(), 0, out.data_ptr(),
                              _lib.stream_handle()) == _lib.SQ_ERR_ARG


def test_dense_blocks_match_reference_golden(h2o2):
    """Every f class of H2O2/cc-pVTZ (two O centres with f shells) against the reference's own blocks."""
    e, eng = h2o2
    g = load_golden("h2o2_ccpvtz_f")
    V = eng.eri_dense(1e-14)
    shells = eng.mol.shells
    worst = 0.0
    for qi, (a, b, c, d) in enumerate(g["quartets"]):
        sl = [slice(shells[s].bf_idx[0], shells[s].bf_idx[-1] + 1) for s in (a, b, c, d)]
        blk = V[sl[0], sl[1], sl[2], sl[3]].reshape(-1).cpu().numpy()
        ref = g["blocks"][g["block_off"][qi]:g["block_off"][qi + 1]]
        worst = max(worst, float(np.max(np.abs(blk - ref))))
    assert worst < 1e-10, worst
    assert len(g["quartets"]) >= 60  # every f class, two quartets each


def test_dense_schwarz_one_electron_match_oracle():
    """Water/cc-pVTZ: the whole tensor, the Schwarz factors and S, T, V against the oracle."""
    from slowquant_gb300 import systems

    geom = systems.water_monomer()
    o = O.OracleMolecule(geom, "cc-pvtz", "angstrom")
    eng = _engine(geom, "cc-pvtz", "angstrom")
    assert eng.nbf == o.nbf == 65
    np.testing.assert_allclose(eng.schwarz_matrix(), o.schwarz(faithful=True), atol=1e-12)
    V = eng.eri_dense(1e-12).cpu().numpy()
    np.testing.assert_allclose(V, o.eri_dense(1e-12), atol=1e-10)
    S, T, Vn = (x.cpu().numpy() for x in eng.one_electron())
    So, To, Vo = o.one_electron()
    np.testing.assert_allclose(S, So, atol=1e-12)
    np.testing.assert_allclose(T, To, atol=1e-11)
    np.testing.assert_allclose(Vn, Vo, atol=1e-10)


def _oracle_exact_boys(fn):
    """Run fn() with the oracle's accurate Boys mode (the full series, asymptote beyond z = 60)."""
    O.lib().sqo_set_boys_mode(1)
    try:
        return fn()
    finally:
        O.lib().sqo_set_boys_mode(0)


def test_jk_with_f_shells_fp64_and_fp32(h2o2):
    """Direct J/K (tabulated high-order Boys) == the oracle's contraction with the accurate Boys function.

    The reference's own Boys series (integralfunctions.py:74-97) stops once a
    term is below 1e-12 in absolute terms.  The first term is 1/(2n+1)!!, below
    that for n >= 12, so F_12 keeps one term, and f-shell integrals move by up to
    1e-2.  The dense tensor reproduces this (drop-in output); the Fock build does not.
    """
    import torch

    e, eng = h2o2
    o = O.OracleMolecule(e["geometry"], e["basis"], e["unit"])
    D = _random_density(eng.nbf, 11)
    Jr, Kr = O.jk_from_eri(_oracle_exact_boys(lambda: o.eri_dense(1e-14)), D)
    Dt = torch.tensor(D, dtype=torch.float64, device="cuda")
    J, K = (x.cpu().numpy() for x in eng.jk(Dt, 1e-14, "fp64"))
    np.testing.assert_allclose(J, Jr, atol=1e-10)
    np.testing.assert_allclose(K, Kr, atol=1e-10)
    for prec in ("mixed", "mixed_boys32"):
        J3, K3 = (x.cpu().numpy() for x in eng.jk(Dt, 1e-14, prec, fp32_threshold=1e30))
        assert np.max(np.abs(J3 - J)) < 1e-4
        assert np.max(np.abs(K3 - K)) < 1e-4


def test_jk_matches_oracle_einsum_water_ccpvtz():
    import torch

    from slowquant_gb300 import systems

    geom = systems.water_monomer()
    o = O.OracleMolecule(geom, "cc-pvtz", "angstrom")
    eng = _engine(geom, "cc-pvtz", "angstrom")
    D = _random_density(eng.nbf, 3)
    Jr, Kr = O.jk_from_eri(_oracle_exact_boys(lambda: o.eri_dense(1e-12)), D)
    J, K = (x.cpu().numpy() for x in eng.jk(torch.tensor(D, dtype=torch.float64, device="cuda"), 1e-12, "fp64"))
    np.testing.assert_allclose(J, Jr, atol=1e-10)
    np.testing.assert_allclose(K, Kr, atol=1e-10)


def _oracle_rhf(geom, basis, unit, exact_boys):
    o = O.OracleMolecule(geom, basis, unit)
    V = _oracle_exact_boys(lambda: o.eri_dense(1e-12)) if exact_boys else o.eri_dense(1e-12)
    S, T, Vn = o.one_electron()
    return O.run_hartree_fock(S, T, Vn, lambda D: O.jk_from_eri(V, D), o.number_electrons)[0]


def _run(geom, basis, **kw):
    import slowquant_gb300.SlowQuant as sq

    A = sq.SlowQuant()
    A.set_molecule(geom, distance_unit="angstrom")
    A.set_basis_set(basis)
    A.init_hartree_fock()
    A.hartree_fock.logger.print_output = False
    for k, v in kw.items():
        setattr(A.hartree_fock, k, v)
    return A


def test_rhf_energy_water_ccpvtz(gpu_lib):
    """RHF through the reference's public API with f shells on O.

    Direct J/K (accurate Boys) against the oracle's SCF on the accurate tensor;
    the stored-tensor path (reference Boys, as the reference stores it) against
    the oracle's SCF on the reference-faithful tensor; mixed within 1e-6.
    """
    from slowquant_gb300 import systems

    geom = systems.water_monomer()
    A = _run(geom, "cc-pvtz")
    A.hartree_fock.run_restricted_hartree_fock()
    assert abs(A.hartree_fock.E_hf - _oracle_rhf(geom, "cc-pvtz", "angstrom", True)) < 1e-8
    B = _run(geom, "cc-pvtz", direct_jk=False)
    B.hartree_fock.run_restricted_hartree_fock()
    assert abs(B.hartree_fock.E_hf - _oracle_rhf(geom, "cc-pvtz", "angstrom", False)) < 1e-8
    M = _run(geom, "cc-pvtz", precision="mixed", fp32_schwarz_threshold=1e-4)
    M.hartree_fock.run_restricted_hartree_fock()
    assert M.hartree_fock.fock_builds[0] != "fp64" and M.hartree_fock.fock_builds[-1] == "fp64"
    assert abs(M.hartree_fock.E_hf - A.hartree_fock.E_hf) < 1e-6
    # UHF (two densities per integral pass) on the closed shell lands on the RHF energy
    U = _run(geom, "cc-pvtz", uhf_lumo_homo_mix_coeff=0.0)
    U.hartree_fock.run_unrestricted_hartree_fock()
    assert abs(U.hartree_fock.E_uhf - A.hartree_fock.E_hf) < 1e-8


def test_batch_with_f_shells(gpu_lib):
    """Batched SCF of cc-pVTZ molecules of uneven size (one launch per class for the whole batch)."""
    from slowquant_gb300 import systems
    from slowquant_gb300.batch import BatchEngine, BatchSCF
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.hartreefock import DirectJK, run_hartree_fock
    from slowquant_gb300.logger import _Logger

    mols = [_mol(systems.water_cluster(n, 6.0, seed=40 + n), "cc-pvtz", "angstrom") for n in (1, 2)]
    E = BatchSCF(BatchEngine(mols), "fp64", use_graphs=False).run(1e-10, 1e-10)
    ref = []
    for m in mols:
        eng = IntegralEngine(m)
        S, T, V = eng.one_electron()
        log = _Logger()
        log.print_output = False
        ref.append(run_hartree_fock(S, T, V, DirectJK(eng), m.number_electrons, log, 1e-10, 1e-10, 100, True)[0])
    np.testing.assert_allclose(E, np.array(ref), atol=1e-8)


def test_f_classes_agree_across_kernel_shapes(h2o2):
    """(fs|ss), (fs|ps), (fp|ss) on per-thread kernels == on the warp kernel (all precisions)."""
    import torch

    from slowquant_gb300 import _lib

    e, eng = h2o2
    D = torch.tensor(_random_density(eng.nbf, 4), dtype=torch.float64, device="cuda")
    lib = _lib.lib()
    res = {}
    try:
        for min_l in (5, 0):
            lib.sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, min_l)
            res[min_l] = {p: [x.cpu().numpy() for x in eng.jk(D, 1e-12, p, fp32_threshold=1e30)]
                          for p in ("fp64", "mixed", "mixed_boys32")}
    finally:
        lib.sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, 5)
    for p, tol in (("fp64", 1e-11), ("mixed", 2e-4), ("mixed_boys32", 2e-4)):
        for a, b in zip(res[5][p], res[0][p]):
            assert np.max(np.abs(a - b)) < tol, p
