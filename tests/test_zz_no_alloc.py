"""The allocation-free J/K entry point (sq_jk_noalloc) against sq_jk.

sq_jk_noalloc is for callers that cannot allocate device memory (a host that
owns the whole device pool, a stream being captured in a mode that forbids
allocation, latency-critical SCF loops): its FP32 density scratch lives in a
fixed array inside the library instead of caller memory.  This file runs last
(pytest collects test files in name order) so that a failure here stops a -x
run only after every other test has run; it also passes on its own in a fresh
process.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine():
    from slowquant_gb300 import systems
    from slowquant_gb300.engine import IntegralEngine
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(systems.water_cluster(2, 5.0, seed=2), 0, "angstrom")
    m._set_basis_set("cc-pvdz")
    return IntegralEngine(m)


def _noalloc_calls(eng, D, lists, precs, J, K):
    """sq_jk_noalloc for each list, accumulating into the caller's J, K (current stream)."""
    from slowquant_gb300 import _lib

    for ql, prec in zip(lists, precs):
        qs = ql.cstruct()
        rc = _lib.lib().sq_jk_noalloc(ctypes.byref(eng.cbasis), ctypes.byref(eng.cpairs), ctypes.byref(eng.slots),
                                      ctypes.byref(qs), eng.tab64.data_ptr(), eng.tab32.data_ptr(), D.data_ptr(),
                                      J.data_ptr(), K.data_ptr(), _lib.PRECISIONS[prec], _lib.stream_handle())
        _lib.check(rc, "sq_jk_noalloc")


def _noalloc_jk(eng, D, lists, precs):
    import torch

    n = eng.nbf
    J = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    K = torch.zeros_like(J)
    _noalloc_calls(eng, D, lists, precs, J, K)
    torch.cuda.synchronize()
    return J.cpu().numpy(), K.cpu().numpy()


def _setup():
    import torch

    eng = _engine()
    rng = np.random.default_rng(11)
    C = rng.normal(size=(eng.nbf, eng.nbf // 3)) / np.sqrt(eng.nbf)
    D = torch.tensor(2 * C @ C.T, dtype=torch.float64, device="cuda")
    q64, q32 = eng.quartets(1e-12, 1e-4)
    lists, precs = [q64, q32], ["fp64", "fp32"]
    Jr, Kr = (x.cpu().numpy() for x in eng.jk_accumulate(D, lists, precs))
    return eng, D, lists, precs, Jr, Kr


def test_noalloc_matches_sq_jk_two_calls_in_a_row(gpu_lib):
    eng, D, lists, precs, Jr, Kr = _setup()
    for _ in range(2):
        J, K = _noalloc_jk(eng, D, lists, precs)
        np.testing.assert_allclose(J, Jr, atol=1e-10)
        np.testing.assert_allclose(K, Kr, atol=1e-10)


def test_noalloc_rejects_basis_beyond_limit(gpu_lib):
    from slowquant_gb300 import _lib

    eng = _engine()
    big = _lib.SqBasis.from_buffer_copy(eng.cbasis)
    big.nbf = _lib.SQ_NOALLOC_MAX_NBF + 1
    q64 = eng.quartets(1e-12)
    qs = q64.cstruct()
    rc = _lib.lib().sq_jk_noalloc(ctypes.byref(big), ctypes.byref(eng.cpairs), ctypes.byref(eng.slots),
                                  ctypes.byref(qs), eng.tab64.data_ptr(), eng.tab32.data_ptr(), None, None, None,
                                  _lib.SQ_FP32, _lib.stream_handle())
    assert rc == 1  # SQ_ERR_ARG
    assert b"exceeds the static scratch limit" in _lib.lib().sq_last_error()


def test_noalloc_allocates_nothing_and_runs_under_a_global_capture(gpu_lib):
    """The property callers rely on: no device memory is taken by the calls,
    and after one call on the device (which looks up the array's address) the
    calls can be recorded by a stream capture in global mode, where any
    cudaMalloc from any thread would fail the capture."""
    import torch

    eng, D, lists, precs, Jr, Kr = _setup()
    n = eng.nbf
    J = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    K = torch.zeros_like(J)
    _noalloc_calls(eng, D, lists, precs, J, K)  # first call on this device
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        J.zero_()
        K.zero_()
        _noalloc_calls(eng, D, lists, precs, J, K)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    np.testing.assert_allclose(J.cpu().numpy(), Jr, atol=1e-10)

    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="global"):
        J.zero_()
        K.zero_()
        _noalloc_calls(eng, D, lists, precs, J, K)
    for _ in range(2):
        J.fill_(1.0)  # replay must overwrite: the graph zeroes and re-accumulates
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_allclose(J.cpu().numpy(), Jr, atol=1e-10)
        np.testing.assert_allclose(K.cpu().numpy(), Kr, atol=1e-10)
