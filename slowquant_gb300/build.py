"""Build the CUDA library ``libsqgb300.so`` in-tree for sm_103a.

Every ``csrc/*.cu`` is compiled to an object in parallel (one nvcc per
translation unit), then linked into ``slowquant_gb300/libsqgb300.so`` with the
static CUDA runtime.  Objects are rebuilt only when a source or header is newer.

    python -m slowquant_gb300.build [--jobs N] [--force]
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsqgb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _nvcc() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        nvcc = "/usr/local/cuda/bin/nvcc"
    if nvcc is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build slowquant_gb300")
    return nvcc


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, obj: str, extra: list[str]) -> tuple[str, float, str]:
    t0 = time.time()
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{proc.stderr}")
    return os.path.basename(src), time.time() - t0, proc.stderr


def build(jobs: int | None = None, force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile and link; returns the path of the shared library."""
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = _newest_header()
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr):
            todo.append((s, o))
    jobs = jobs or max(1, os.cpu_count() or 1)
    # longest translation units first: the per-class kernels of the high classes
    # (eri_q12..q18 and their FP64 variants) take 1-2 minutes each, the rest seconds
    def cost(so):
        base = os.path.basename(so[0])[:-3]
        if base.startswith("eri_q"):
            num = base[5:].split("_")[0]
            if num.isdigit():
                return 100 * int(num) + (50 if base.endswith("_f64") else 0)
        return os.path.getsize(so[0]) / 1e4

    todo.sort(key=lambda so: -cost(so))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = [ex.submit(_compile, s, o, extra) for s, o in todo]
            for f in cf.as_completed(futs):
                name, dt, err = f.result()
                if verbose:
                    print(f"  nvcc {name}: {dt:.1f}s", flush=True)
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [_nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-cudart", "static", "-o", tmp, *objs]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{proc.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args()
    t0 = time.time()
    path = build(args.jobs, args.force, verbose=True)
    print(f"built {path} in {time.time() - t0:.1f}s")


if __name__ == "__main__":
    sys.exit(main())
