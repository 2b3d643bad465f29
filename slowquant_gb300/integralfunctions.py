"""AO -> MO integral transforms on the GPU (slowquant/molecularintegrals/integralfunctions.py:186-211).

The reference contracts with numpy einsum along a fixed path, one AO index at
a time.  Here the same quarter-transform chain runs through the library's
FP64 kernel ``sq_ao2mo_rotate``: each pass transforms the last AO index and
writes it as the first index, so that four passes give g[i][j][k][l] (two
give C^T h C) with no separate permutation.  Inputs may be numpy arrays or
torch tensors; numpy in gives numpy out.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr


def _device_pair(C, X):
    if not torch.cuda.is_available():
        raise RuntimeError("slowquant_gb300 needs a CUDA device; there is no CPU fallback")
    dev = torch.device("cuda", torch.cuda.current_device())
    as_numpy = not isinstance(X, torch.Tensor)
    Ct = torch.as_tensor(np.asarray(C, dtype=np.float64)) if not isinstance(C, torch.Tensor) else C
    Xt = torch.as_tensor(np.asarray(X, dtype=np.float64)) if as_numpy else X
    return (Ct.to(device=dev, dtype=torch.float64).contiguous(), Xt.to(device=dev, dtype=torch.float64).contiguous(),
            as_numpy)


def _rotate_passes(X: torch.Tensor, Ct: torch.Tensor, npass: int) -> torch.Tensor:
    """Apply ``npass`` transform-last-index-and-rotate passes to an n^npass tensor."""
    lib = _lib.lib()
    n, m = Ct.shape
    shape = [n] * npass
    cur = X.reshape(-1)
    for k in range(npass):
        rows = cur.numel() // n
        out = torch.empty(rows * m, dtype=torch.float64, device=X.device)
        check(lib.sq_ao2mo_rotate(rows, n, m, ptr(cur), ptr(Ct), ptr(out), _lib.stream_handle()), "sq_ao2mo_rotate")
        shape = [m] + shape[:-1]
        cur = out
    return cur.reshape(shape)


def one_electron_integral_transform(C, int1e):
    """h_ij = sum_ab C_ai C_bj h_ab (integralfunctions.py:186-196)."""
    Ct, Ht, as_numpy = _device_pair(C, int1e)
    out = _rotate_passes(Ht, Ct, 2)
    return out.cpu().numpy() if as_numpy else out


def two_electron_integral_transform(C, int2e):
    """g_ijkl = sum_abcd C_ai C_bj C_ck C_dl g_abcd (integralfunctions.py:199-211)."""
    Ct, Gt, as_numpy = _device_pair(C, int2e)
    out = _rotate_passes(Gt, Ct, 4)
    return out.cpu().numpy() if as_numpy else out
