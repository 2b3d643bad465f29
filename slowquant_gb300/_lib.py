"""ctypes binding of the C ABI declared in include/slowquant_gb300.h.

The shared library ``libsqgb300.so`` is built in-tree by
``slowquant_gb300.build``.  There is no fallback: if the library is missing or
no CUDA device is present, every entry point raises.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsqgb300.so")

SQ_OK = 0
SQ_ERR_ARG = 1
SQ_ERR_UNSUPPORTED = 2
SQ_ERR_CUDA = 3
SQ_ERR_NONFINITE = 4
SQ_MAX_L = 3
SQ_MAX_QCLASS = 55
SQ_MAX_L_GRAD = 3
SQ_BOYS_NGRID = 580
SQ_BOYS_STEP_INV = 16
SQ_BOYS_NCOL = 16
SQ_BOYS_TMAX = 36.0
SQ_BOYS_HI_NGRID = 968
SQ_BOYS_HI_NCOL = 24
SQ_BOYS_HI_TMAX = 60.0
SQ_BOYS_TAY64_OFF = SQ_BOYS_NGRID * SQ_BOYS_NCOL
SQ_BOYS_HI64_OFF = SQ_BOYS_TAY64_OFF + 16 * SQ_BOYS_NGRID * 8
SQ_BOYS_TAB64_SIZE = SQ_BOYS_HI64_OFF + SQ_BOYS_HI_NGRID * SQ_BOYS_HI_NCOL
SQ_BOYS_TAY32_5_OFF = SQ_BOYS_NGRID * SQ_BOYS_NCOL + 16 * SQ_BOYS_NGRID * 4
SQ_BOYS_DF_OFF = SQ_BOYS_TAY32_5_OFF + 16 * SQ_BOYS_NGRID
SQ_BOYS_TAB32_SIZE = SQ_BOYS_DF_OFF + 16 * SQ_BOYS_NGRID * 12
SQ_FP64 = 0
SQ_FP32 = 1
SQ_FP32_BOYS32 = 2
SQ_FP64_PRIM = 3
SQ_DF64 = 4
SQ_OPT_GENERIC_MIN_L = 1
SQ_OPT_JK_STREAMS = 2
SQ_OPT_FP64_UNROLLED_HIGH = 3
SQ_OPT_GRAD_THREAD = 4
SQ_OPT_DF_CLASSES = 5
SQ_NOALLOC_MAX_NBF = 1024
SQ_NOALLOC_MAX_ELEMS = SQ_NOALLOC_MAX_NBF * SQ_NOALLOC_MAX_NBF

PRECISIONS = {"fp64": SQ_FP64, "fp32": SQ_FP32, "fp32_boys32": SQ_FP32_BOYS32, "fp64_prim": SQ_FP64_PRIM,
              "df64": SQ_DF64}

_p = ctypes.c_void_p


class SqBasis(ctypes.Structure):
    _fields_ = [
        ("nshell", ctypes.c_int), ("nbf", ctypes.c_int), ("natom", ctypes.c_int), ("nprim_total", ctypes.c_int),
        ("center", _p), ("l", _p), ("nprim", _p), ("prim_off", _p), ("bf_off", _p), ("exps", _p),
        ("coefs", _p), ("atom_xyz", _p), ("atom_charge", _p), ("shell_atom", _p),
        ("mat_base", _p), ("mat_ld", _p), ("mat_total", ctypes.c_longlong), ("atom_begin", _p), ("atom_end", _p),
    ]


class SqPairs(ctypes.Structure):
    _fields_ = [
        ("npair", ctypes.c_int), ("nprimpair", ctypes.c_int), ("shells", _p), ("pp_off", _p),
        ("herm_off", _p), ("prim", _p), ("herm", _p), ("prim32", _p), ("herm32", _p), ("pq", _p),
    ]


class SqSlots(ctypes.Structure):
    _fields_ = [
        ("nslot", ctypes.c_int), ("npp_total", ctypes.c_longlong), ("nherm_total", ctypes.c_longlong),
        ("pair", _p), ("npp", _p), ("pbase", _p), ("pstride", _p), ("hbase", _p),
        ("prim", _p), ("herm", _p), ("prim32", _p), ("herm32", _p),
        ("prim_src", _p), ("prim_src_off", _p), ("sub", _p), ("desc", _p), ("mbase", _p), ("prim32v", _p),
        ("primdf", _p), ("hermdf", _p),
    ]


class SqQuartets(ctypes.Structure):
    _fields_ = [
        ("nquartet", ctypes.c_longlong), ("pairs", _p),
        ("class_off", ctypes.c_longlong * (SQ_MAX_QCLASS + 1)),
    ]


_lib = None


def _preload_torch_linalg() -> None:
    """Load torch's CUDA linear-algebra library by absolute path, once.

    torch opens libtorch_cuda_linalg.so by bare name on the first torch.linalg
    call on a CUDA tensor.  Under a profiler that interposes dlopen (ncu) that
    name no longer resolves through torch's run path and the call fails;
    loaded here by path with RTLD_GLOBAL, the later dlopen finds this copy.
    """
    try:
        import torch

        path = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
        if os.path.exists(path):
            ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    except OSError:
        pass


def lib() -> ctypes.CDLL:
    """Load libsqgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -m slowquant_gb300.build); there is no CPU fallback"
            )
        _preload_torch_linalg()
        L = ctypes.CDLL(LIB_PATH)
        L.sq_last_error.restype = ctypes.c_char_p
        L.sq_version.restype = ctypes.c_int
        L.sq_get_option.restype = ctypes.c_longlong
        L.sq_get_option.argtypes = [ctypes.c_int]
        L.sq_set_option.argtypes = [ctypes.c_int, ctypes.c_longlong]
        L.sq_set_launch_config.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_longlong]
        L.sq_boys_table.argtypes = [_p, _p, _p]
        L.sq_boys.argtypes = [ctypes.c_int, _p, ctypes.c_longlong, _p, ctypes.c_int, _p, _p]
        L.sq_pair_prep.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), _p]
        L.sq_schwarz.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqQuartets), _p,
                                 _p, _p]
        L.sq_eri_dense.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                                   ctypes.POINTER(SqQuartets), _p, _p, _p]
        L.sq_jk.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                            ctypes.POINTER(SqQuartets), _p, _p, _p, _p, _p, _p, ctypes.c_int, _p]
        L.sq_jk_multi.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                                  ctypes.POINTER(SqQuartets), _p, _p, ctypes.c_int, _p, _p, _p, _p, ctypes.c_int, _p]
        L.sq_slots_fill.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots), _p]
        L.sq_slots_describe.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                                        _p]
        L.sq_grad_2e.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                                 ctypes.POINTER(SqQuartets), _p, _p, _p, _p]
        L.sq_grad_1e.argtypes = [ctypes.POINTER(SqBasis), _p, _p, _p, _p, _p]
        L.sq_ao2mo_rotate.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, _p, _p, _p, _p]
        L.sq_multipole.argtypes = [ctypes.POINTER(SqBasis), _p, _p, _p, _p]
        L.sq_jk_dense.argtypes = [ctypes.c_int, _p, _p, _p, _p, _p]
        L.sq_jk_prim.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                                 ctypes.POINTER(SqQuartets), _p, _p, _p, _p, _p, ctypes.c_double, _p]
        L.sq_jk_df.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                               ctypes.POINTER(SqQuartets), _p, _p, _p, _p, _p, _p, ctypes.c_double, _p]
        L.sq_df_class.argtypes = [ctypes.c_int, ctypes.c_longlong]
        L.sq_boys_df.argtypes = [ctypes.c_int, _p, ctypes.c_longlong, _p, _p, _p]
        L.sq_jk_noalloc.argtypes = [ctypes.POINTER(SqBasis), ctypes.POINTER(SqPairs), ctypes.POINTER(SqSlots),
                                    ctypes.POINTER(SqQuartets), _p, _p, _p, _p, _p, ctypes.c_int, _p]
        L.sq_fock_build.argtypes = [ctypes.c_int, _p, _p, _p, _p, _p, _p, _p]
        L.sq_one_electron.argtypes = [ctypes.POINTER(SqBasis), _p, _p, _p, _p, _p]
        L.sq_quartets_expand.argtypes = [ctypes.c_longlong, _p, _p, _p, _p, _p, _p, ctypes.c_longlong, _p]
        L.sq_fma_probe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _p, _p]
        L.sq_batched_eigh.argtypes = [ctypes.c_int, _p, _p, ctypes.c_int, _p, _p, _p, _p, ctypes.c_double,
                                      ctypes.c_int, _p, _p]
        _lib = L
    return _lib


EXPORTED = [
    "sq_version", "sq_last_error", "sq_set_option", "sq_get_option", "sq_set_launch_config", "sq_boys_table", "sq_boys",
    "sq_pair_prep", "sq_schwarz", "sq_eri_dense", "sq_jk", "sq_fock_build", "sq_one_electron",
    "sq_quartets_expand", "sq_fma_probe", "sq_slots_fill", "sq_slots_describe", "sq_jk_prim", "sq_jk_df", "sq_df_class", "sq_boys_df", "sq_ao2mo_rotate", "sq_multipole", "sq_jk_dense", "sq_jk_noalloc", "sq_grad_2e", "sq_grad_1e",
    "sq_batched_eigh", "sq_jk_multi",
]


def check(rc: int, what: str = "") -> None:
    """Raise RuntimeError carrying sq_last_error() when rc != SQ_OK."""
    if rc != SQ_OK:
        msg = lib().sq_last_error().decode(errors="replace")
        raise RuntimeError(f"slowquant_gb300 {what} failed (status {rc}): {msg}")


def ptr(t) -> int | None:
    """Device pointer of a torch tensor (None for None)."""
    return None if t is None else t.data_ptr()


def stream_handle(device=None) -> int:
    import torch

    return torch.cuda.current_stream(device).cuda_stream
