"""GPU integral kernels against the oracle and the reference's golden outputs.

Tolerances: integrals 1e-10 absolute (the parity bar), Boys 1e-12.
"""

import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_golden, unpack_unique

pytestmark = pytest.mark.gpu

SYSTEMS = ["h2o_sto3g_crawford", "h2o_sto3g_c1", "ch4_sto3g", "h2o_631gs", "h2o_dz", "h2o_ccpvdz_c1", "h2o_dzp",
           "h6_dzp"]


def _engine(geom, basis, unit):
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(geom, 0, unit)
    m._set_basis_set(basis)
    return IntegralEngine(m)


@pytest.fixture(autouse=True)
def _lib_ready(gpu_lib):
    from slowquant_gb300 import _lib

    _lib.lib().sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, 5)
    yield
    _lib.lib().sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, 5)


def _gpu_boys(eng, z, nmax, mode):
    import torch

    from slowquant_gb300 import _lib

    zt = torch.tensor(z, dtype=torch.float64, device="cuda")
    out = torch.zeros((len(z), nmax + 1), dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().sq_boys(nmax, zt.data_ptr(), len(z), eng.tab64.data_ptr(), mode, out.data_ptr(),
                                  _lib.stream_handle()), "sq_boys")
    return out.cpu().numpy()


def _oracle_boys(z, nmax, mode):
    O.lib().sqo_set_boys_mode(mode)
    try:
        return np.array([[O.boys(n, zz) for n in range(nmax + 1)] for zz in z])
    finally:
        O.lib().sqo_set_boys_mode(0)


def test_boys_against_oracle():
    """Tabulated Boys vs the exact series; reference-mode Boys vs the reference's formula."""
    eng = _engine("H 0 0 0;H 0 0 1.4", "sto-3g", "bohr")
    z = np.concatenate([[0.0, 1e-14, 1e-9, 1e-4], np.linspace(0.001, 60, 1777), [35.99, 36.0, 36.01, 100.0, 1e4]])
    nmax = 8
    exact = _oracle_boys(z, nmax, 1)
    # T >= 36 drops the e^{-T} term of the upward recursion: < 1e-17 absolute
    np.testing.assert_allclose(_gpu_boys(eng, z, nmax, 0), exact, rtol=2e-14, atol=1e-16)
    ref = _oracle_boys(z, nmax, 0)
    np.testing.assert_allclose(_gpu_boys(eng, z, nmax, 1), ref, rtol=1e-13, atol=1e-300)
    # the reference's own truncation: large relative error for high n at small z
    assert np.max(np.abs(ref - exact) / exact) > 1e-7


@pytest.mark.parametrize("name", SYSTEMS)
def test_schwarz_dense_eri_one_electron(name, golden_energies):
    e = golden_energies[name]
    d = load_golden(name)
    eng = _engine(e["geometry"], e["basis"], e["unit"])
    np.testing.assert_allclose(eng.schwarz_matrix(), d["schwarz"], atol=1e-12)
    V = eng.eri_dense(1e-12).cpu().numpy()
    ref = d["eri"] if "eri" in d else unpack_unique(d["eri_unique"], eng.nbf)
    np.testing.assert_allclose(V, ref, atol=1e-10)
    assert np.max(np.abs(V - ref)) < 1e-11
    S, T, Vn = (x.cpu().numpy() for x in eng.one_electron())
    np.testing.assert_allclose(S, d["S"], atol=1e-12)
    np.testing.assert_allclose(T, d["T"], atol=1e-11)
    np.testing.assert_allclose(Vn, d["V"], atol=1e-10)


def _random_density(n, seed):
    rng = np.random.default_rng(seed)
    C = rng.normal(size=(n, max(1, n // 3))) / np.sqrt(n)
    return 2 * C @ C.T


@pytest.mark.parametrize("geom_kind", ["monomer_ccpvdz", "dimer_ccpvdz", "trimer_631gs"])
def test_direct_jk_matches_oracle_einsum(geom_kind):
    import torch

    from slowquant_gb300 import systems

    geom, basis = {
        "monomer_ccpvdz": (systems.water_monomer(), "cc-pvdz"),
        "dimer_ccpvdz": (systems.water_cluster(2, 5.0, seed=2), "cc-pvdz"),
        "trimer_631gs": (systems.water_cluster(3, 6.0, seed=3), "6-31G*"),
    }[geom_kind]
    o = O.OracleMolecule(geom, basis, "angstrom")
    Vref = o.eri_dense(1e-12)
    eng = _engine(geom, basis, "angstrom")
    D = _random_density(eng.nbf, 5)
    Jr, Kr = O.jk_from_eri(Vref, D)
    Dt = torch.tensor(D, dtype=torch.float64, device="cuda")
    J, K = (x.cpu().numpy() for x in eng.jk(Dt, 1e-12, "fp64"))
    np.testing.assert_allclose(J, Jr, atol=1e-10)
    np.testing.assert_allclose(K, Kr, atol=1e-10)


def test_generic_warp_kernel_matches_per_class_kernels():
    """Every class on the warp kernel == the unrolled per-class kernels (J/K)."""
    import torch

    from slowquant_gb300 import _lib, systems

    eng = _engine(systems.water_cluster(2, 5.0, seed=2), "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 1), dtype=torch.float64, device="cuda")
    J1, K1 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    _lib.lib().sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, 0)
    J2, K2 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    np.testing.assert_allclose(J2, J1, atol=1e-11)
    np.testing.assert_allclose(K2, K1, atol=1e-11)
    # FP32 paths of both kernels agree with FP64 within the FP32 error scale
    for prec in ("mixed", "mixed_boys32"):
        for min_l in (0, 5):
            _lib.lib().sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, min_l)
            J3, K3 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, prec, fp32_threshold=1e30))
            assert np.max(np.abs(J3 - J1)) < 1e-4
            assert np.max(np.abs(K3 - K1)) < 1e-4


def test_driver_entry_points_follow_reference_screening():
    """electronrepulsion.py semantics: no matrix -> all quartets; huge threshold -> zeros."""
    from slowquant_gb300 import electronrepulsion as er
    from slowquant_gb300.molecule import _Molecule

    g = "H 0 0 0;H 1 0 0;H 2 0 0;H 3 0 0;H 4 0 0;H 5 0 0"
    m = _Molecule(g, 0, "bohr")
    m._set_basis_set("dzp")
    cs = er.get_cauchy_schwarz_matrix(m)
    d = load_golden("h6_dzp")
    np.testing.assert_allclose(cs, d["schwarz"], atol=1e-12)
    full = er.electron_repulsion_integral_driver(m)
    ref = unpack_unique(d["eri_unique"], m.number_bf)
    np.testing.assert_allclose(full, ref, atol=1e-10)
    for thr, tol in [(1e-8, 1e-8), (1e-3, 1e-3)]:
        Vs = er.electron_repulsion_integral_driver(m, cs, thr)
        np.testing.assert_allclose(Vs, full, atol=tol)
    assert np.all(er.electron_repulsion_integral_driver(m, cs, 1e10) == 0.0)


def test_primitive_pair_screening(monkeypatch):
    """Dropping primitive pairs with bound q_ij * max q < 1e-17 leaves J/K unchanged (1e-11)."""
    import torch

    from slowquant_gb300 import engine as E
    from slowquant_gb300 import systems

    geom = systems.water_cluster(4, 8.0, seed=4)
    eng = _engine(geom, "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 2), dtype=torch.float64, device="cuda")
    J1, K1 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    kept, total = int(eng.slot_npp[:eng.nslot_base].sum()), int(eng.pair_np.sum())
    assert kept < total
    # primitive Schwarz factors bound the contracted ones: q_P <= sum_ij q_ij
    qp = eng.prim_q
    qsum = np.add.reduceat(qp, eng.pp_off_host[:-1])
    assert np.all(eng.pair_q <= qsum * (1 + 1e-12) + 1e-300)
    monkeypatch.setattr(E, "PRIM_SCREEN", 0.0)
    eng0 = _engine(geom, "cc-pvdz", "angstrom")
    J0, K0 = (x.cpu().numpy() for x in eng0.jk(D, 1e-12, "fp64"))
    assert int(eng0.slot_npp[:eng0.nslot_base].sum()) == total
    np.testing.assert_allclose(J1, J0, atol=1e-11)
    np.testing.assert_allclose(K1, K0, atol=1e-11)


def test_split_quartets_match_whole(monkeypatch):
    """Heavy J/K quartets split into bra sub-slot chunks give the same J/K (both kernels)."""
    import torch

    from slowquant_gb300 import _lib
    from slowquant_gb300 import engine as E
    from slowquant_gb300 import systems

    geom = systems.water_cluster(3, 6.0, seed=3)
    monkeypatch.setattr(E, "SPLIT_TARGET", 64)
    eng = _engine(geom, "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 3), dtype=torch.float64, device="cuda")
    ql = eng.quartets(1e-12)
    whole = eng.quartets(1e-12, split=False)
    assert ql.nquartet > whole.nquartet  # some quartets were split
    assert int((eng.slot_sub != 0).sum()) > 0
    J1, K1 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    lists, precs = [whole], ["fp64"]
    Jw, Kw = eng.jk_accumulate(D, lists, precs)
    Jw = (0.5 * (Jw + Jw.T)).cpu().numpy()
    Kw = (0.5 * (Kw + Kw.T)).cpu().numpy()
    np.testing.assert_allclose(J1, Jw, atol=1e-11)
    np.testing.assert_allclose(K1, Kw, atol=1e-11)
    # the generic warp kernel honours sub-slots too
    _lib.lib().sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, 0)
    J2, K2 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    np.testing.assert_allclose(J2, Jw, atol=1e-11)
    np.testing.assert_allclose(K2, Kw, atol=1e-11)
    # mixed precision lists split as well (FP32 error scale)
    J3, K3 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "mixed", fp32_threshold=1e-4))
    assert np.max(np.abs(J3 - Jw)) < 1e-6 and np.max(np.abs(K3 - Kw)) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_jk_multi_matches_single_density_builds(precision):
    """sq_jk_multi (one integral pass, several densities) == one sq_jk per density."""
    import torch

    from slowquant_gb300 import systems

    eng = _engine(systems.water_cluster(2, 5.0, seed=2), "cc-pvdz", "angstrom")
    Ds = torch.tensor(np.stack([_random_density(eng.nbf, s) for s in (7, 8, 9)]), dtype=torch.float64,
                      device="cuda")
    J, K = eng.jk_multi(Ds, 1e-12, precision, 1e-4)
    for i in range(3):
        Ji, Ki = eng.jk(Ds[i], 1e-12, precision, 1e-4)
        tol = 1e-11 if precision == "fp64" else 1e-9
        np.testing.assert_allclose(J[i].cpu().numpy(), Ji.cpu().numpy(), atol=tol)
        np.testing.assert_allclose(K[i].cpu().numpy(), Ki.cpu().numpy(), atol=tol)


def test_jk_stream_pool_matches_single_stream():
    """Class launches spread over the library's streams == all on the caller's stream."""
    import torch

    from slowquant_gb300 import _lib, systems

    L = _lib.lib()
    eng = _engine(systems.water_cluster(2, 5.0, seed=2), "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 4), dtype=torch.float64, device="cuda")
    default = L.sq_get_option(_lib.SQ_OPT_JK_STREAMS)
    assert default >= 1
    try:
        _lib.check(L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, 1), "sq_set_option")
        J1, K1 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "mixed", 1e-4))
        _lib.check(L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, 8), "sq_set_option")
        J8, K8 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "mixed", 1e-4))
        assert L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, 17) != 0  # out of range is rejected
    finally:
        L.sq_set_option(_lib.SQ_OPT_JK_STREAMS, default)
    np.testing.assert_allclose(J8, J1, atol=1e-11)
    np.testing.assert_allclose(K8, K1, atol=1e-11)


def test_chunk_level_mixed_precision():
    """mixed_chunk: FP64 quartets' small primitive chunks in FP32; J/K at the FP32 error scale."""
    import torch

    from slowquant_gb300 import systems

    eng = _engine(systems.water_cluster(3, 6.0, seed=3), "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 6), dtype=torch.float64, device="cuda")
    J0, K0 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    Jm, Km = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "mixed", 1e-4))
    Jc, Kc = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "mixed_chunk", 1e-4))
    assert np.max(np.abs(Jc - J0)) < 1e-6 and np.max(np.abs(Kc - K0)) < 1e-6
    # the chunk lists keep fewer primitive quartets in FP64 than the quartet-level lists
    npp = eng.slot_npp.astype(np.int64)

    def prims(ql):
        p = ql.pairs[: ql.nquartet].cpu().numpy()
        return int((npp[p[:, 0]] * npp[p[:, 1]]).sum())

    q64, q32 = eng.quartets(1e-12, 1e-4)
    c64, c32 = eng.quartets(1e-12, 1e-4, chunks=True)
    assert prims(c64) < prims(q64)
    assert prims(c64) + prims(c32) == prims(q64) + prims(q32)  # same primitive quartets, re-partitioned
    # every chunk kept in FP64 (per-thread classes 0-18) has a large bound
    p = c64.pairs[: int(c64.class_off[19])].cpu().numpy()
    assert np.all(eng.slot_qsum[p[:, 0]] * eng.slot_qsum[p[:, 1]] >= 1e-4)
    assert np.max(np.abs(Jm - J0)) < 1e-6


def test_chunk_lists_partition_exactly_in_fp64():
    """The chunk lists (bra and ket sub-slots) run both in FP64 reproduce the FP64 J/K,
    on the per-thread kernels and on the generic warp kernel."""
    import torch

    from slowquant_gb300 import _lib, systems

    eng = _engine(systems.water_cluster(3, 6.0, seed=3), "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 9), dtype=torch.float64, device="cuda")
    J0, K0 = (x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64"))
    c64, c32 = eng.quartets(1e-12, 1e-4, chunks=True)
    assert (eng.slot_sub[c64.pairs[: c64.nquartet, 1].cpu().numpy()] != 0).any()  # some kets were cut
    for min_l in (5, 0):
        _lib.lib().sq_set_option(_lib.SQ_OPT_GENERIC_MIN_L, min_l)
        Ja, Ka = eng.jk_accumulate(D, [c64, c32], ["fp64", "fp64"])
        J = (0.5 * (Ja + Ja.T)).cpu().numpy()
        K = (0.5 * (Ka + Ka.T)).cpu().numpy()
        np.testing.assert_allclose(J, J0, atol=1e-11)
        np.testing.assert_allclose(K, K0, atol=1e-11)


def test_ket_split_lists_give_the_same_jk(monkeypatch):
    """Short heavy-class segments cut into ket sub-slot chunks: the same J and K, more list entries."""
    import torch

    from slowquant_gb300 import engine, systems

    geom = systems.water_cluster(3, 6.0, seed=3)
    eng = _engine(geom, "cc-pvdz", "angstrom")
    D = torch.tensor(_random_density(eng.nbf, 7), dtype=torch.float64, device="cuda")
    res = {}
    for per_sm in (0, 256):
        monkeypatch.setattr(engine, "KET_SPLIT_PER_SM", per_sm)
        eng._quartet_cache.clear()
        ql = eng.quartets(1e-12)
        res[per_sm] = (ql.class_counts(), [x.cpu().numpy() for x in eng.jk(D, 1e-12, "fp64")],
                       [x.cpu().numpy() for x in eng.jk(D, 1e-12, "mixed_prim", 1e-3)])
    (c0, jk0, jp0), (c1, jk1, jp1) = res[0], res[256]
    assert sum(c1[12:19]) > sum(c0[12:19]) and (c1[:12] == c0[:12]).all()
    for a, b in zip(jk0, jk1):
        np.testing.assert_allclose(b, a, atol=1e-12)
    for a, b in zip(jp0, jp1):  # the FP32 parts are summed in other groupings: FP32 rounding of terms < 1e-3
        np.testing.assert_allclose(b, a, atol=1e-8)
