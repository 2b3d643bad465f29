"""Double-float J/K kernels (sq_jk_df): FP64-level results from FP32-pipe arithmetic.

The classes (ss|ss) to (dd|ds) carry every FP64 quantity as a pair of floats
(about 46 significant bits) and run on the FP32 pipe; the other classes run
as in sq_jk_prim.  Checks: J and K at a fixed density against the FP64
kernels and against the oracle's direct J/K (tolerance 1e-10, the bar of the
FP64 kernels against the oracle); the double-float Boys rows against the
FP64 ones; SCF energies against the FP64 SCF (1e-9 Eh) and the reference's
golden energies (1e-8 Eh); the mixed mode (FP32 below the primitive bound,
double-float above) within the error its bound allows; argument refusal.
"""

import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _geom(n=2, seed=2):
    from slowquant_gb300 import systems

    return systems.water_cluster(n, 3.0 + 2.0 * n, seed=seed)


def _engine(n=2, basis="cc-pvdz", seed=2):
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(_geom(n, seed), 0, "angstrom")
    m._set_basis_set(basis)
    return IntegralEngine(m)


def _density(eng, seed=5):
    import torch

    rng = np.random.default_rng(seed)
    C = rng.normal(size=(eng.nbf, eng.nbf // 4)) / np.sqrt(eng.nbf)
    return torch.tensor(2 * C @ C.T, dtype=torch.float64, device="cuda")


def _jk(eng, D, ql, prec, tau=0.0):
    Jacc, Kacc = eng.jk_accumulate(D, [ql], [prec], prim_tau=tau)
    return (0.5 * (Jacc + Jacc.T)).cpu().numpy(), (0.5 * (Kacc + Kacc.T)).cpu().numpy()


@pytest.mark.parametrize("basis", ["sto-3g", "6-31G*", "cc-pvdz"])
def test_df64_jk_matches_fp64_kernels_and_oracle(gpu_lib, basis):
    eng = _engine(2, basis)
    D = _density(eng)
    ql = eng.quartets(1e-12)
    J64, K64 = _jk(eng, D, ql, "fp64")
    Jd, Kd = _jk(eng, D, ql, "df64")
    np.testing.assert_allclose(Jd, J64, atol=1e-10)
    np.testing.assert_allclose(Kd, K64, atol=1e-10)
    assert np.abs(Jd - J64).max() > 0.0  # a different arithmetic, not the FP64 launch
    om = O.OracleMolecule(_geom(2), basis, "angstrom")
    Jo, Ko = om.jk_direct(D.cpu().numpy(), 1e-12)
    np.testing.assert_allclose(Jd, Jo, atol=1e-10)
    np.testing.assert_allclose(Kd, Ko, atol=1e-10)


def test_df64_boys_rows_match_fp64_table(gpu_lib):
    """The double-float Taylor rows are the FP64 rows split into (hi, lo)."""
    from slowquant_gb300 import _lib

    eng = _engine(1, "sto-3g")
    t64 = eng.tab64.cpu().numpy()
    t32 = eng.tab32.cpu().numpy()
    ng = _lib.SQ_BOYS_NGRID
    tay = t64[_lib.SQ_BOYS_TAY64_OFF: _lib.SQ_BOYS_TAY64_OFF + 16 * ng * 8].reshape(16, ng, 8)
    df = t32[_lib.SQ_BOYS_DF_OFF: _lib.SQ_BOYS_DF_OFF + 16 * ng * 12].reshape(16, ng, 12).astype(np.float64)
    for j in range(4):
        np.testing.assert_allclose(df[:, :, 2 * j] + df[:, :, 2 * j + 1], tay[:, :, j], rtol=2e-15, atol=1e-300)
    for j in range(4, 7):
        np.testing.assert_allclose(df[:, :, 4 + j], tay[:, :, j].astype(np.float32), rtol=0, atol=0)
    assert not df[:, :, 11].any()


@pytest.mark.parametrize("n_max", [0, 1, 2, 5, 8])
def test_double_float_boys_against_fp64_table_and_exact(gpu_lib, n_max):
    """boys_df (float-pair Taylor rows, downward recursion in float pairs) against the FP64
    tabulated function (rtol 1e-12, all T) and the exact F_m(T) = 1F1(m+1/2; m+3/2; -T)/(2m+1)
    (rtol 1e-12 below T = 36, where both expand about the grid; above it both use the
    same asymptote, whose own error is up to 1e-8 for m = 8 at T = 36)."""
    import torch
    from scipy.special import hyp1f1

    from slowquant_gb300 import _lib

    eng = _engine(1, "sto-3g")
    rng = np.random.default_rng(11)
    z = np.concatenate([np.arange(0, 60, 1 / 16.0), rng.uniform(0, 60, 4000), [0.0, 1e-9, 35.999, 36.0, 36.001]])
    zt = torch.tensor(z, dtype=torch.float64, device="cuda")
    out_df = torch.empty((len(z), n_max + 1), dtype=torch.float64, device="cuda")
    out64 = torch.empty_like(out_df)
    L = _lib.lib()
    s = _lib.stream_handle()
    _lib.check(L.sq_boys_df(n_max, zt.data_ptr(), len(z), eng.tab32.data_ptr(), out_df.data_ptr(), s), "sq_boys_df")
    _lib.check(L.sq_boys(n_max, zt.data_ptr(), len(z), eng.tab64.data_ptr(), 0, out64.data_ptr(), s), "sq_boys")
    Fd, F64 = out_df.cpu().numpy(), out64.cpu().numpy()
    np.testing.assert_allclose(Fd, F64, rtol=1e-12, atol=0)
    low = z < 36.0
    m = np.arange(n_max + 1)
    exact = hyp1f1(m[None, :] + 0.5, m[None, :] + 1.5, -z[low, None]) / (2 * m[None, :] + 1)
    np.testing.assert_allclose(Fd[low], exact, rtol=1e-12, atol=0)
    assert L.sq_boys_df(9, zt.data_ptr(), 1, eng.tab32.data_ptr(), out_df.data_ptr(), s) == _lib.SQ_ERR_ARG


@pytest.mark.parametrize("name", ["h2o_sto3g_c1", "ch4_sto3g", "h2o_631gs", "h2o_ccpvdz_c1", "h6_dzp"])
def test_df64_scf_matches_reference_energies(gpu_lib, golden_energies, name):
    from tests.test_gpu_scf import _run

    e = golden_energies[name]
    A = _run(e["geometry"], e["basis"], e["unit"], precision="df64")
    assert set(A.hartree_fock.fock_builds) == {"df64"}
    assert abs(A.hartree_fock.E_hf - e["E_hf"]) < 1e-8


def test_df64_scf_matches_fp64_scf_on_a_cluster(gpu_lib):
    from slowquant_gb300 import systems

    from tests.test_gpu_scf import _run

    g = systems.water_cluster(3, 6.0, seed=3)
    ref = _run(g, "cc-pvdz", "angstrom").hartree_fock.E_hf
    A = _run(g, "cc-pvdz", "angstrom", precision="df64")
    assert abs(A.hartree_fock.E_hf - ref) < 1e-9


@pytest.mark.parametrize("tau", [1e-4, 1e-3])
def test_mixed_df_error_is_bounded_by_the_primitive_bound(gpu_lib, tau):
    eng = _engine(3, seed=3)
    D = _density(eng)
    q64, q32 = eng.quartets(1e-12, tau)
    Jr, Kr = _jk(eng, D, eng.quartets(1e-12), "fp64")
    Jacc, Kacc = eng.jk_accumulate(D, [q64, q32], ["df64_prim", "fp32"], prim_tau=tau)
    J = (0.5 * (Jacc + Jacc.T)).cpu().numpy()
    K = (0.5 * (Kacc + Kacc.T)).cpu().numpy()
    tol = 2e-5 * max(tau, 1e-4)
    assert np.abs(J - Jr).max() < tol and np.abs(K - Kr).max() < tol
    Dn = D.cpu().numpy()
    assert abs(0.5 * np.sum(Dn * (J - Jr)) - 0.25 * np.sum(Dn * (K - Kr))) < 1e-6


def test_mixed_df_scf_ends_in_double_float_at_the_fp64_energy(gpu_lib):
    from slowquant_gb300 import systems

    from tests.test_gpu_scf import _run

    g = systems.water_cluster(2, 5.0, seed=2)
    ref = _run(g, "cc-pvdz", "angstrom").hartree_fock.E_hf
    A = _run(g, "cc-pvdz", "angstrom", precision="mixed_df", fp32_schwarz_threshold=1e-3)
    builds = A.hartree_fock.fock_builds
    assert builds[0] == "mixed_df" and builds[-1] == "df64"
    assert abs(A.hartree_fock.E_hf - ref) < 1e-8


def test_df_entry_point_refuses_missing_double_float_data(gpu_lib):
    import torch

    from slowquant_gb300 import _lib

    eng = _engine(1)
    ql = eng.quartets(1e-12)
    slots = _lib.SqSlots.from_buffer_copy(eng.slots)
    slots.hermdf = None
    n = eng.nbf
    J = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    Ddf = torch.zeros(2 * n * n, dtype=torch.float32, device="cuda")
    rc = _lib.lib().sq_jk_df(ctypes.byref(eng.cbasis), ctypes.byref(eng.cpairs), ctypes.byref(slots),
                             ctypes.byref(ql.cstruct()), eng.tab64.data_ptr(), eng.tab32.data_ptr(), J.data_ptr(),
                             Ddf.data_ptr(), J.data_ptr(), J.data_ptr(), 0.0, _lib.stream_handle())
    assert rc == _lib.SQ_ERR_ARG and b"hermdf" in _lib.lib().sq_last_error()
    assert float(J.abs().sum()) == 0.0
