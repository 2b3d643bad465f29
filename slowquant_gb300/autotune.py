"""Autotuner for the J/K kernels' launch shape per quartet class and precision.

For every class present in a workload's quartet lists it times the class's
launch alone (CUDA events, median of 3) over candidate shapes -- threads per
block and the grid cap, i.e. how many quartets each thread or warp takes in
its grid-stride loop -- and installs the fastest through
sq_set_launch_config.  The result is returned as a table
{(class, precision): (threads, blocks, ms)} and can be re-applied with
``apply``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .engine import QuartetList

THREADS = (64, 128)
WAVES = (1, 2, 4, 8, 16, 64, 128)


def _time(fn, reps: int = 3) -> float:
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def apply(table: dict) -> None:
    lib = _lib.lib()
    for (c, prec), (threads, blocks, _) in table.items():
        _lib.check(lib.sq_set_launch_config(c, _lib.PRECISIONS[prec], threads, blocks), "sq_set_launch_config")


def reset() -> None:
    lib = _lib.lib()
    for c in range(_lib.SQ_MAX_QCLASS):
        for p in range(3):
            lib.sq_set_launch_config(c, p, 0, 0)


def tune(run_class, lists, precs, threads=THREADS, waves=WAVES) -> dict:
    """run_class(sub_list, prec) launches one class; lists/precs as for jk_accumulate."""
    lib = _lib.lib()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    table = {}
    for ql, prec in zip(lists, precs):
        p = _lib.PRECISIONS[prec]
        for c in range(_lib.SQ_MAX_QCLASS):
            n = int(ql.class_off[c + 1] - ql.class_off[c])
            if n == 0:
                continue
            off = np.zeros(_lib.SQ_MAX_QCLASS + 1, dtype=np.int64)
            off[c + 1:] = n
            sub = QuartetList(ql.pairs[ql.class_off[c]:ql.class_off[c + 1]], off)
            lib.sq_set_launch_config(c, p, 0, 0)
            best = (0, 0, _time(lambda: run_class(sub, prec)))
            for t in threads:
                for w in waves:
                    blocks = sms * w * (128 // t)
                    _lib.check(lib.sq_set_launch_config(c, p, t, blocks), "sq_set_launch_config")
                    ms = _time(lambda: run_class(sub, prec))
                    if ms < best[2]:
                        best = (t, blocks, ms)
            _lib.check(lib.sq_set_launch_config(c, p, best[0], best[1]), "sq_set_launch_config")
            table[(c, prec)] = best
    return table
