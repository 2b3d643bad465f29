"""Shared test configuration.

Markers: ``gpu`` -- needs a CUDA device and the built libsqgb300.so.
The golden fixtures in tests/golden were produced by running the reference
itself (tests/golden/make_golden.py).
"""

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled CUDA library")


@pytest.fixture(scope="session")
def golden_energies():
    with open(os.path.join(GOLDEN, "golden_energies.json")) as fh:
        return json.load(fh)


def load_golden(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def unpack_unique(vals: np.ndarray, n: int) -> np.ndarray:
    """Inverse of make_golden.unique_eri: fill the dense 8-fold symmetric tensor."""
    V = np.zeros((n, n, n, n))
    ii, jj = np.tril_indices(n)
    P, Q = np.tril_indices(len(ii))
    a, b, c, d = ii[P], jj[P], ii[Q], jj[Q]
    for (p, q_, r, s) in [(a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                          (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)]:
        V[p, q_, r, s] = vals
    return V


@pytest.fixture(scope="session")
def gpu_lib():
    """Built library + a CUDA device, else the GPU test fails loudly."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is available")
    from slowquant_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.lib()
