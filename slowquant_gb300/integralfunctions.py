"""AO -> MO integral transforms on the GPU (slowquant/molecularintegrals/integralfunctions.py:186-211).

The reference contracts with numpy einsum along a fixed path, one AO index at
a time.  Here the same quarter-transform chain runs as FP64 GEMMs on the
device (cuBLAS through torch): for the two-electron tensor four successive
(n^3 x n) @ (n x m) products, O(n^4 m) work each, instead of one n^8 loop.
Inputs may be numpy arrays or torch tensors; numpy in gives numpy out.
"""

from __future__ import annotations

import numpy as np
import torch


def _device_pair(C, X):
    if not torch.cuda.is_available():
        raise RuntimeError("slowquant_gb300 needs a CUDA device; there is no CPU fallback")
    dev = torch.device("cuda", torch.cuda.current_device())
    as_numpy = not isinstance(X, torch.Tensor)
    Ct = torch.as_tensor(np.asarray(C, dtype=np.float64)) if not isinstance(C, torch.Tensor) else C
    Xt = torch.as_tensor(np.asarray(X, dtype=np.float64)) if as_numpy else X
    return Ct.to(device=dev, dtype=torch.float64), Xt.to(device=dev, dtype=torch.float64), as_numpy


def one_electron_integral_transform(C, int1e):
    """h_ij = sum_ab C_ai C_bj h_ab (integralfunctions.py:186-196)."""
    Ct, Ht, as_numpy = _device_pair(C, int1e)
    out = Ct.T @ Ht @ Ct
    return out.cpu().numpy() if as_numpy else out


def two_electron_integral_transform(C, int2e):
    """g_ijkl = sum_abcd C_ai C_bj C_ck C_dl g_abcd (integralfunctions.py:199-211)."""
    Ct, Gt, as_numpy = _device_pair(C, int2e)
    n, m = Ct.shape
    # transform the last AO index, then rotate it to the front; four times
    g = Gt.reshape(n, n, n, n)
    for _ in range(4):
        a0, a1, a2, a3 = g.shape
        g = (g.reshape(a0 * a1 * a2, a3) @ Ct).reshape(a0, a1, a2, m)
        g = g.permute(3, 0, 1, 2).contiguous()
    return g.cpu().numpy() if as_numpy else g
