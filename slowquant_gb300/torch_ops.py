"""The library's entry points as torch operators (``torch.ops.slowquant_gb300.*``).

The compute goes through the same C ABI (libsqgb300.so) as the rest of the
package; registering the calls with ``torch.library`` lets torch code use them
as operators on CUDA tensors, with shape rules for fake tensors:

* ``jk_dense(V, D) -> (J, K)``: the einsum J/K of a stored tensor (sq_jk_dense);
* ``ao2mo(C, G) -> G_mo``: the four-index AO -> MO transformation (sq_ao2mo_rotate);
* ``direct_jk(handle, D, threshold, precision, fp32_threshold) -> (J, K)``: the
  integral-direct J/K of a registered ``IntegralEngine`` (``register_engine``
  returns its handle), i.e. sq_jk / sq_jk_prim over its screened quartets.

Importing this module registers the operators once per process.
"""

from __future__ import annotations

import torch

_engines: dict = {}


def register_engine(engine) -> int:
    """Make an IntegralEngine reachable from ``direct_jk``; returns its handle."""
    h = len(_engines) + 1
    _engines[h] = engine
    return h


@torch.library.custom_op("slowquant_gb300::jk_dense", mutates_args=())
def jk_dense(V: torch.Tensor, D: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    from .hartreefock import dense_jk

    return dense_jk(V, D)


@jk_dense.register_fake
def _(V, D):
    n = V.shape[0]
    return V.new_empty((n, n)), V.new_empty((n, n))


@torch.library.custom_op("slowquant_gb300::ao2mo", mutates_args=())
def ao2mo(C: torch.Tensor, G: torch.Tensor) -> torch.Tensor:
    from .integralfunctions import two_electron_integral_transform

    return two_electron_integral_transform(C, G)


@ao2mo.register_fake
def _(C, G):
    m = C.shape[1]
    return G.new_empty((m, m, m, m))


@torch.library.custom_op("slowquant_gb300::direct_jk", mutates_args=())
def direct_jk(handle: int, D: torch.Tensor, threshold: float, precision: str,
              fp32_threshold: float) -> tuple[torch.Tensor, torch.Tensor]:
    eng = _engines[handle]
    J, K = eng.jk(D, threshold, precision, fp32_threshold)
    return J, K


@direct_jk.register_fake
def _(handle, D, threshold, precision, fp32_threshold):
    return D.new_empty(D.shape), D.new_empty(D.shape)
