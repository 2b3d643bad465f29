"""Primitive-level precision inside the FP64 J/K launches (sq_jk_prim).

The large-bound quartets of a mixed build keep their FP64 launch, but each of
their primitive quartets whose primitive Schwarz bound q_ij q_kl falls below
the bound runs in FP32 (with the FP64 Boys recursion) and is added into the
FP64 block.  Checks: a zero bound reproduces the plain FP64 launch; a bound
above every primitive quartet gives the FP32 launch's numbers; in between, the
error of J, K and of the one-build energy stays within what FP32 arithmetic on
primitive quartets of that size can cause; a mixed SCF in this mode finishes
in FP64 at the FP64 energy.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(n=2, basis="cc-pvdz", seed=2):
    from slowquant_gb300 import systems
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(systems.water_cluster(n, 3.0 + 2.0 * n, seed=seed), 0, "angstrom")
    m._set_basis_set(basis)
    return IntegralEngine(m)


def _density(eng, seed=5):
    import torch

    rng = np.random.default_rng(seed)
    C = rng.normal(size=(eng.nbf, eng.nbf // 4)) / np.sqrt(eng.nbf)
    return torch.tensor(2 * C @ C.T, dtype=torch.float64, device="cuda")


def _jk(eng, D, ql, prec, tau=0.0):
    Jacc, Kacc = eng.jk_accumulate(D, [ql], [prec], prim_tau=tau)
    J = 0.5 * (Jacc + Jacc.T)
    K = 0.5 * (Kacc + Kacc.T)
    return J.cpu().numpy(), K.cpu().numpy()


def test_zero_bound_is_the_fp64_launch(gpu_lib):
    eng = _engine()
    D = _density(eng)
    ql = eng.quartets(1e-12)
    J64, K64 = _jk(eng, D, ql, "fp64")
    J, K = _jk(eng, D, ql, "fp64_prim", 0.0)
    np.testing.assert_allclose(J, J64, atol=1e-12)
    np.testing.assert_allclose(K, K64, atol=1e-12)


def test_bound_above_everything_is_the_fp32_launch(gpu_lib):
    eng = _engine()
    D = _density(eng)
    ql = eng.quartets(1e-12)
    J64, K64 = _jk(eng, D, ql, "fp64")
    J32, K32 = _jk(eng, D, ql, "fp32")
    J, K = _jk(eng, D, ql, "fp64_prim", 1e30)
    scale = max(np.abs(J64).max(), np.abs(K64).max())
    # the same FP32 arithmetic per primitive quartet in the per-thread classes;
    # the other classes (warp kernel) run FP64 in the split launch
    assert np.abs(J - J32).max() < 1e-5 * scale and np.abs(K - K32).max() < 1e-5 * scale
    assert np.abs(J - J64).max() > 1e-12  # really not the FP64 path


@pytest.mark.parametrize("tau", [1e-5, 1e-4, 1e-3, 1e-2])
def test_error_is_bounded_by_the_primitive_bound(gpu_lib, tau):
    eng = _engine(3, seed=3)
    D = _density(eng)
    q64, q32 = eng.quartets(1e-12, tau)
    Jr, Kr = _jk(eng, D, eng.quartets(1e-12), "fp64")
    Jacc, Kacc = eng.jk_accumulate(D, [q64, q32], ["fp64_prim", "fp32"], prim_tau=tau)
    J = (0.5 * (Jacc + Jacc.T)).cpu().numpy()
    K = (0.5 * (Kacc + Kacc.T)).cpu().numpy()
    # FP32 relative error (~1e-6 after the recurrences) on contributions of size <= tau
    tol = 2e-5 * max(tau, 1e-4)
    assert np.abs(J - Jr).max() < tol, (tau, np.abs(J - Jr).max())
    assert np.abs(K - Kr).max() < tol, (tau, np.abs(K - Kr).max())
    Dn = D.cpu().numpy()
    dE = 0.5 * np.sum(Dn * (J - Jr)) - 0.25 * np.sum(Dn * (K - Kr))
    assert abs(dE) < 1e-6


def test_mixed_prim_scf_ends_at_the_fp64_energy(gpu_lib):
    from slowquant_gb300 import systems

    from tests.test_gpu_scf import _run

    g = systems.water_cluster(2, 5.0, seed=2)
    ref = _run(g, "cc-pvdz", "angstrom").hartree_fock.E_hf
    A = _run(g, "cc-pvdz", "angstrom", precision="mixed_prim", fp32_schwarz_threshold=1e-3)
    builds = A.hartree_fock.fock_builds
    assert builds[0] == "mixed_prim" and builds[-1] == "fp64"
    assert abs(A.hartree_fock.E_hf - ref) < 1e-8


def test_prim_entry_point_refuses_missing_primitive_factors(gpu_lib):
    import torch

    from slowquant_gb300 import _lib

    eng = _engine(1)
    ql = eng.quartets(1e-12)
    pairs = _lib.SqPairs.from_buffer_copy(eng.cpairs)
    pairs.pq = None
    n = eng.nbf
    J = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    rc = _lib.lib().sq_jk_prim(ctypes.byref(eng.cbasis), ctypes.byref(pairs), ctypes.byref(eng.slots),
                               ctypes.byref(ql.cstruct()), eng.tab64.data_ptr(), eng.tab32.data_ptr(), J.data_ptr(),
                               J.data_ptr(), J.data_ptr(), 1e-4, _lib.stream_handle())
    assert rc == _lib.SQ_ERR_ARG and b"pairs->pq" in _lib.lib().sq_last_error()
