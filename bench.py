"""Benchmark: integral-direct Fock build of a (H2O)_16 cluster in cc-pVDZ.

One step = one Fock build F = H + J - K/2 of the seeded (H2O)_16 cluster
(11 A cube, seed 16; 400 Cartesian basis functions) directly from the
Schwarz-screened ERIs (threshold 1e-12), in mixed precision (quartets with
Schwarz bound < 1e-4 in FP32 with FP64 Boys recursion; FP64 above), the
headline configuration.  The FP64 plain build of the same workload is timed in
the same run and reported beside it, with the SCF energy error of the mixed
scheme against the FP64 SCF.

Prints ONE JSON line (rank 0).  ``--impl reference`` times the reference's CPU
algorithm (the oracle's C restatement of electronrepulsion.py, faithful loop
structure, all host threads) on bounded samples of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ERI quartets/s & Fock-build ms, mixed vs FP64 plain on GPU at |ΔE|≤1e-6 Eh"
WATERS, BOX, SEED, BASIS = 16, 11.0, 16, "cc-pvdz"
BOXES = {16: 11.0, 8: 9.0}
# Cartesian basis functions per water and the basis's name as printed
BASES = {"cc-pvdz": (25, "cc-pVDZ"), "cc-pvtz": (65, "cc-pVTZ")}
SCREEN, FP32_THR = 1e-12, 1e-3
# precision mode of the headline build, and the launch precision of its large-bound list
HEADLINE = "mixed_df"
ACCURATE_LIST = {"mixed": "fp64", "mixed_prim": "fp64_prim", "mixed_df": "df64_prim"}
HEADLINE_TEXT = {
    "mixed": "mixed (quartets with Schwarz bound below {tau:g} in FP32 with the FP64 Boys recursion; FP64 above)",
    "mixed_prim": "mixed_prim (FP64 for the large-bound quartets, their primitive quartets below {tau:g} in FP32; "
                  "FP32 quartets below the bound)",
    "mixed_df": "mixed_df (double-float arithmetic on the FP32 pipe, about 46 bits, for the large-bound quartets of "
                "the classes where it is faster, FP64 for the others; their primitive quartets below {tau:g} and "
                "the quartets below {tau:g} in FP32)",
}


def workload_geometry() -> str:
    from slowquant_gb300 import systems

    return systems.water_cluster(WATERS, BOXES.get(WATERS, BOX), SEED)


def oracle_fixture():
    """The oracle's SCF fixture for the configured cluster (tests/golden/make_headline.py), or None."""
    name = {(16, "cc-pvdz"): "headline_c3", (8, "cc-pvdz"): "headline_c2"}.get((WATERS, BASIS))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", f"{name}.npz")
    if name is None or not os.path.exists(path):
        return None
    g = np.load(path)
    if str(g["geometry"]) != workload_geometry():
        return None
    return {"E_hf": float(g["E_hf"]), "E_at_D": float(g["E_at_D"])}


def config(extra=None) -> dict:
    nbf_w, label = BASES[BASIS]
    c = {
        "workload": f"(H2O)_{WATERS} {label} Fock build (J+K), {nbf_w * WATERS} Cartesian bf, "
                    f"{BOXES.get(WATERS, BOX):g} A cube seed {SEED}",
        "molecule": f"(H2O)_{WATERS}",
        "basis": f"{label} (Cartesian, {nbf_w * WATERS} bf)",
        "schwarz_threshold": SCREEN,
        "fp32_schwarz_threshold": FP32_THR,
        "precision": HEADLINE_TEXT[HEADLINE].format(tau=FP32_THR),
        "step": "one Fock build F = H + J - K/2 from a converged-SCF density",
        "l2": "flushed between timed steps (512 MB write); quartet list > L2",
        "parallelism": "replicas only",
    }
    if extra:
        c.update(extra)
    return c


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- helpers
def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def fma_peak(lib, torch, precision: int) -> float:
    """Measured FMA throughput (FLOP/s) of one pipe via the library's probe kernel."""
    from slowquant_gb300 import _lib

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, iters = sms * 8, {_lib.SQ_FP64: 20000, _lib.SQ_DF64: 30000}.get(precision, 400000)
    out = torch.empty(blocks * 256, dtype=torch.float64, device="cuda")
    s = _lib.stream_handle()
    _lib.check(lib.sq_fma_probe(precision, blocks, 100, out.data_ptr(), s), "sq_fma_probe")
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(lib.sq_fma_probe(precision, blocks, iters, out.data_ptr(), s), "sq_fma_probe")
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 16.0 * iters * 256 * blocks / (e0.elapsed_time(e1) * 1e-3))
    return best


def class_work(eng, ql, precision: str = "fp64") -> dict:
    """Per quartet class: contracted quartets, primitive quartets, model FLOPs.

    Primitive quartets are the ones the launch computes: the per-thread class
    kernels (classes 0-18, 21, 22, 28) loop over the slots' screened
    primitive pairs, the generic warp kernel over all of a pair's primitives.
    """
    import torch

    from slowquant_gb300 import _lib, flops

    # quartet entries are slot ids: primitive pairs per slot
    npp_slot = torch.tensor(eng.slot_npp, dtype=torch.int64, device=eng.device)
    npp_all = torch.tensor(eng.pair_np[eng.slot_pair], dtype=torch.int64, device=eng.device)
    sub = torch.tensor(eng.slot_sub, dtype=torch.int64, device=eng.device)
    # the warp kernel's share of a sub-slot: its chunk of all the pair's primitive pairs
    S = torch.clamp(sub & 0xFFFF, min=1)
    kk = sub >> 16
    npp_all = (npp_all * (kk + 1)) // S - (npp_all * kk) // S
    out = {}
    for c in range(_lib.SQ_MAX_QCLASS):
        a, b = int(ql.class_off[c]), int(ql.class_off[c + 1])
        if b == a:
            continue
        per_thread = c <= 18 or c in (21, 22, 28)  # the per-thread kernels (f: (fs|ss), (fs|ps), (fp|ss))
        npp = npp_slot if per_thread else npp_all
        seg = ql.pairs[a:b].long()
        nprim = int((npp[seg[:, 0]] * npp[seg[:, 1]]).sum())
        nuniq = int(((sub[seg[:, 0]] >> 16) == 0).sum())
        la, lb, lc, ld = flops.quartet_class_l(c)
        f = nprim * flops.flops_per_primitive_quartet(la, lb, lc, ld) + nuniq * flops.flops_per_contracted_quartet_jk(
            la, lb, lc, ld)
        out[c] = {"quartets": nuniq, "list_entries": b - a, "prim_quartets": nprim, "flops": float(f),
                  "class": f"{la}{lb}{lc}{ld}"}
    return out


def time_events(torch, fn, n: int, flush=None, preroll: bool = False) -> list[float]:
    """CUDA-event times (ms) of n calls of fn, L2 flushed before each.  preroll
    queues a ~2 ms device sleep before the start event, so that the host has
    issued all of fn's launches before the GPU reaches it: the time is then the
    device's alone (used for the per-class launches, whose host-side issue
    time would otherwise count)."""
    ts = []
    for _ in range(n):
        if flush is not None:
            flush()
        if preroll:
            torch.cuda._sleep(4_000_000)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return ts


def max_over_ranks(value: float, world: int, device: str = "cpu") -> float:
    """The largest of every rank's value (the slowest replica sets the timed region)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------- CPU arm
def cpu_sample(eng_or_none, target_seconds: float, seed: int = 0, pairs_host=None, mol_geom=None, n_fixed=None):
    """Time the oracle (faithful restatement of the reference) on random surviving quartets.

    Without n_fixed the sample size is calibrated upward until one sample takes
    about 0.3-1x target_seconds; with n_fixed exactly that many quartets are timed.
    """
    from oracle import oracle as O

    o = O.OracleMolecule(mol_geom, BASIS, "angstrom")
    rng = np.random.default_rng(seed)
    pair_shells, quartets = pairs_host
    nthreads = os.cpu_count() or 1
    n = 64 if n_fixed is None else int(n_fixed)
    while True:
        idx = rng.integers(0, len(quartets), n)
        sq = np.concatenate([pair_shells[quartets[idx, 0]], pair_shells[quartets[idx, 1]]], axis=1)
        t0 = time.time()
        o.eri_quartets(sq, nthreads=nthreads, faithful=True)
        dt = time.time() - t0
        if n_fixed is not None or dt > 0.3 * target_seconds or n >= 2_000_000:
            return n / dt, nthreads, n, dt
        n = int(n * min(16.0, max(2.0, 0.5 * target_seconds / max(dt, 1e-3))))


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # Build the workload's screened quartet list on the host (the oracle's own Schwarz factors).
    from oracle import oracle as O
    from slowquant_gb300 import screening
    from slowquant_gb300.molecule import _Molecule

    geom = workload_geometry()
    m = _Molecule(geom, 0, "angstrom")
    m._set_basis_set(BASIS)
    o = O.OracleMolecule(geom, BASIS, "angstrom")
    cs = o.schwarz(nthreads=os.cpu_count() or 1)
    pair_shells, pc, npa, npb, q = _host_pairs(m, cs)
    lists, ket = screening.build_tasks(pc, npa, npb, q, SCREEN)
    quartets = screening.expand_host(*screening.flatten_tasks(lists[0])[:3], ket)
    rates = []
    t_start = time.time()
    # calibrate once, then every step times the same number of random quartets
    # (about cpu_seconds / 2 each, so the whole run stays within a few minutes)
    rate0, _, n0, dt0 = cpu_sample(None, args.cpu_seconds, seed=12345, pairs_host=(pair_shells, quartets),
                                   mol_geom=geom)
    n_step = max(64, int(rate0 * args.cpu_seconds / 2))
    for step in range(args.warmup + args.steps):
        rate, nthreads, n, dt = cpu_sample(None, args.cpu_seconds, seed=step, pairs_host=(pair_shells, quartets),
                                           mol_geom=geom, n_fixed=n_step)
        if step >= args.warmup:
            rates.append(rate)
    value = float(np.median(rates))
    timings = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "reference_timings.json")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "quartets/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": n_step / value * 1e3,
        "ms_per_step_is": "one timed sample of the workload (the step)",
        "full_build_ms_extrapolated": len(quartets) / value * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config({"total_quartets": len(quartets)}),
        "cpu_baseline": {"value": value, "unit": "quartets/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"per step {n_step} (~{args.cpu_seconds / 2:.0f} s) uniformly random surviving unique shell "
                                   f"quartets of the workload through the oracle's faithful C restatement of "
                                   f"electron_repulsion_integral; full_build_ms_extrapolated scales the rate to "
                                   f"the {len(quartets)}-quartet build"},
        "reference_python": json.load(open(timings)) if os.path.exists(timings) else None,
        "reference_python_is": "the unmodified pure-Python reference timed single-threaded in the build container "
                               "(tests/golden/time_reference.py); it cannot be installed on the GPU host",
        "e2e": {"value": value, "unit": "quartets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": round(time.time() - t_start, 1),
    }
    print(json.dumps(line), flush=True)


def _host_pairs(m, cs):
    """Pair table in the engine's order (host restatement, for the CPU arm)."""
    from slowquant_gb300 import screening  # noqa: F401

    l = np.array([s.angular_momentum for s in m.shells])
    nprim = np.array([len(s.exponents) for s in m.shells])
    i, j = np.triu_indices(len(l))
    a = np.where(l[i] >= l[j], i, j)
    b = np.where(l[i] >= l[j], j, i)
    pc = l[a] * (l[a] + 1) // 2 + l[b]
    order = np.argsort(pc, kind="stable")
    a, b, pc = a[order], b[order], pc[order]
    return np.stack([a, b], 1).astype(np.int32), pc, nprim[a], nprim[b], cs[a, b]


# ----------------------------------------------------------------- GPU arm
def gpu_arm(args) -> None:
    import torch
    import torch.distributed as dist

    from slowquant_gb300 import _lib
    from slowquant_gb300.engine import IntegralEngine, QuartetList
    from slowquant_gb300.hartreefock import DirectJK, run_hartree_fock
    from slowquant_gb300.logger import _Logger
    from slowquant_gb300.molecule import _Molecule

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    lib = _lib.lib()
    if args.jk_streams:
        _lib.check(lib.sq_set_option(_lib.SQ_OPT_JK_STREAMS, args.jk_streams), "sq_set_option")

    geom = workload_geometry()
    mol = _Molecule(geom, 0, "angstrom")
    mol._set_basis_set(BASIS)
    t0 = time.time()
    eng = IntegralEngine(mol)
    q_all = eng.quartets(SCREEN)
    q64, q32 = eng.quartets(SCREEN, FP32_THR)
    # unique contracted quartets (the J/K lists split the heaviest ones into chunks)
    nq_unique = eng.quartets(SCREEN, split=False).nquartet
    n64_unique, n32_unique = (x.nquartet for x in eng.quartets(SCREEN, FP32_THR, split=False))
    S, T, V = eng.one_electron()
    H = T + V
    torch.cuda.synchronize()
    setup_s = time.time() - t0

    # SCF in FP64 and in mixed precision: energies and the converged density
    log = _Logger()
    log.print_output = False
    ne = mol.number_electrons
    jk64 = DirectJK(eng, SCREEN, "fp64")
    t0 = time.time()
    E64, C64, F64, D64 = run_hartree_fock(S, T, V, jk64, ne, log, 1e-9, 1e-9, 100, True)
    scf64_s = time.time() - t0
    jkm = DirectJK(eng, SCREEN, HEADLINE, FP32_THR, 1e-5)
    t0 = time.time()
    Em, _, _, _ = run_hartree_fock(S, T, V, jkm, ne, log, 1e-9, 1e-9, 100, True)
    scfm_s = time.time() - t0
    n_mixed_builds = sum(1 for b in jkm.builds if b != "fp64")
    D = torch.tensor(D64, dtype=torch.float64, device="cuda")

    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.zero_()

    def step_mixed():
        eng.fock(H, D, SCREEN, HEADLINE, FP32_THR)

    def step_fp64():
        eng.fock(H, D, SCREEN, "fp64")

    for _ in range(args.warmup):
        step_mixed()
        step_fp64()
    torch.cuda.synchronize()

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.time()
        torch.cuda.nvtx.range_push("timed_mixed")
        ms_mixed = time_events(torch, step_mixed, args.steps, flush)
        torch.cuda.nvtx.range_pop()
        wall_mixed = time.time() - t_wall
    torch.cuda.nvtx.range_push("timed_fp64")
    ms_fp64 = time_events(torch, step_fp64, max(3, min(args.steps, 5)), flush)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    tot_mixed = sum(ms_mixed)
    tot_mixed = max_over_ranks(tot_mixed, world, "cuda")

    ms_step = tot_mixed / args.steps
    nq = nq_unique
    value = world * nq / (ms_step * 1e-3)
    ms64 = float(np.median(ms_fp64))

    # e2e through the public API: pinned host D -> device, Fock build, F -> pinned host
    D_host = torch.empty_like(D, device="cpu").pin_memory()
    D_host.copy_(D)
    F_host = torch.empty_like(D_host).pin_memory()

    def step_e2e():
        Dd = D_host.to("cuda", non_blocking=True)
        F = eng.fock(H, Dd, SCREEN, HEADLINE, FP32_THR)
        F_host.copy_(F, non_blocking=True)

    for _ in range(2):
        step_e2e()
    ms_e2e = time_events(torch, step_e2e, args.steps, flush)
    e2e_ms = float(np.mean(ms_e2e))

    orc = oracle_fixture()
    # precision threshold sweep: build time, one-build energy error at the FP64
    # density, and the SCF energy error (mixed SCF switches to FP64 at the end)
    Ffp = eng.fock(H, D, SCREEN, "fp64")
    E_build64 = float(0.5 * torch.sum(D * (H + Ffp)))
    sweep = []
    for tau in args.tau_sweep:
        eng.fock(H, D, SCREEN, "mixed", tau)
        ms_tau = float(np.median(time_events(torch, lambda: eng.fock(H, D, SCREEN, "mixed", tau), 3, flush)))
        Fm = eng.fock(H, D, SCREEN, "mixed", tau)
        dE_build = float(0.5 * torch.sum(D * (H + Fm))) - E_build64
        jkt = DirectJK(eng, SCREEN, "mixed", tau, 1e-5)
        Et, _, _, _ = run_hartree_fock(S, T, V, jkt, ne, log, 1e-9, 1e-9, 100, True)
        sweep.append({"fp32_threshold": tau, "fock_build_ms": ms_tau, "speedup_vs_fp64": ms64 / ms_tau,
                      "dE_one_build": dE_build, "dE_scf": Et - E64,
                      "dE_scf_vs_oracle": None if orc is None else Et - orc["E_hf"],
                      "mixed_builds": sum(1 for b in jkt.builds if b != "fp64"), "builds": len(jkt.builds)})

    # primitive-chunk granularity of the same precision test (beside the headline)
    chunk_modes = []
    for tau in (1e-4, 1e-3, 1e-2):
        eng.fock(H, D, SCREEN, "mixed_chunk", tau)
        ms_c = float(np.median(time_events(torch, lambda: eng.fock(H, D, SCREEN, "mixed_chunk", tau), 5, flush)))
        Fc = eng.fock(H, D, SCREEN, "mixed_chunk", tau)
        jkc = DirectJK(eng, SCREEN, "mixed_chunk", tau, 1e-5)
        Ec, _, _, _ = run_hartree_fock(S, T, V, jkc, ne, log, 1e-9, 1e-9, 100, True)
        c64, c32 = eng.quartets(SCREEN, tau, chunks=True)
        chunk_modes.append({"fp32_threshold": tau, "fock_build_ms": ms_c, "speedup_vs_fp64": ms64 / ms_c,
                            "dE_one_build": float(0.5 * torch.sum(D * (H + Fc))) - E_build64, "dE_scf": Ec - E64,
                            "fp64_entries": c64.nquartet, "fp32_entries": c32.nquartet})

    # primitive-level precision inside the FP64 launches (sq_jk_prim) at the same bounds
    prim_modes = []
    for tau in args.prim_sweep:
        eng.fock(H, D, SCREEN, "mixed_prim", tau)
        torch.cuda.nvtx.range_push(f"timed_prim_{tau:g}")
        ms_p = float(np.median(time_events(torch, lambda: eng.fock(H, D, SCREEN, "mixed_prim", tau), 5, flush)))
        torch.cuda.nvtx.range_pop()
        Fp = eng.fock(H, D, SCREEN, "mixed_prim", tau)
        jkp = DirectJK(eng, SCREEN, "mixed_prim", tau, 1e-5)
        Ep, _, _, _ = run_hartree_fock(S, T, V, jkp, ne, log, 1e-9, 1e-9, 100, True)
        p64, p32 = eng.quartets(SCREEN, tau)
        eng.jk_accumulate(D, [p64], ["fp64_prim"], prim_tau=tau)
        ms_p64 = float(np.median(time_events(
            torch, lambda: eng.jk_accumulate(D, [p64], ["fp64_prim"], prim_tau=tau), 5, flush)))
        prim_modes.append({"fp32_threshold": tau, "fock_build_ms": ms_p, "speedup_vs_fp64": ms64 / ms_p,
                           "dE_one_build": float(0.5 * torch.sum(D * (H + Fp))) - E_build64, "dE_scf": Ep - E64,
                           "dE_scf_vs_oracle": None if orc is None else Ep - orc["E_hf"],
                           "fp64_list_alone_ms": ms_p64, "fp64_list_quartets": p64.nquartet,
                           "fp32_list_quartets": p32.nquartet,
                           "mixed_builds": sum(1 for b in jkp.builds if b != "fp64"), "builds": len(jkp.builds)})

    # double-float arithmetic on the FP32 pipe (sq_jk_df) in place of FP64: the
    # whole build, then the primitive-level mixed mode with double-float above the bound
    df_full, df_modes = None, []
    if args.df:
        eng.fock(H, D, SCREEN, "df64")
        torch.cuda.nvtx.range_push("timed_df64")
        ms_df = float(np.median(time_events(torch, lambda: eng.fock(H, D, SCREEN, "df64"), 5, flush)))
        torch.cuda.nvtx.range_pop()
        Fd = eng.fock(H, D, SCREEN, "df64")
        jkd = DirectJK(eng, SCREEN, "df64")
        Ed, _, _, _ = run_hartree_fock(S, T, V, jkd, ne, log, 1e-9, 1e-9, 100, True)
        J64, K64 = eng.jk(D, SCREEN, "fp64")
        Jd, Kd = eng.jk(D, SCREEN, "df64")
        df_full = {"fock_build_ms": ms_df, "speedup_vs_fp64": ms64 / ms_df,
                   "dE_one_build": float(0.5 * torch.sum(D * (H + Fd))) - E_build64, "dE_scf": Ed - E64,
                   "dE_scf_vs_oracle": None if orc is None else Ed - orc["E_hf"],
                   "max_abs_dJ_vs_fp64": float((Jd - J64).abs().max()),
                   "max_abs_dK_vs_fp64": float((Kd - K64).abs().max()), "builds": len(jkd.builds)}
        for tau in args.prim_sweep:
            eng.fock(H, D, SCREEN, "mixed_df", tau)
            torch.cuda.nvtx.range_push(f"timed_mixed_df_{tau:g}")
            ms_q = float(np.median(time_events(torch, lambda: eng.fock(H, D, SCREEN, "mixed_df", tau), 5, flush)))
            torch.cuda.nvtx.range_pop()
            Fq = eng.fock(H, D, SCREEN, "mixed_df", tau)
            jkq = DirectJK(eng, SCREEN, "mixed_df", tau, 1e-5)
            Eq, _, _, _ = run_hartree_fock(S, T, V, jkq, ne, log, 1e-9, 1e-9, 100, True)
            d64, _ = eng.quartets(SCREEN, tau)
            eng.jk_accumulate(D, [d64], ["df64_prim"], prim_tau=tau)
            ms_d64 = float(np.median(time_events(
                torch, lambda: eng.jk_accumulate(D, [d64], ["df64_prim"], prim_tau=tau), 5, flush)))
            df_modes.append({"fp32_threshold": tau, "fock_build_ms": ms_q, "speedup_vs_fp64": ms64 / ms_q,
                             "dE_one_build": float(0.5 * torch.sum(D * (H + Fq))) - E_build64, "dE_scf": Eq - E64,
                             "dE_scf_vs_oracle": None if orc is None else Eq - orc["E_hf"],
                             "df64_list_alone_ms": ms_d64,
                             "mixed_builds": sum(1 for b in jkq.builds if b == "mixed_df"),
                             "builds": len(jkq.builds)})

    # launch shapes from the project's autotuner on this workload's lists, timed beside the defaults
    tuned = None
    if args.autotune:
        from slowquant_gb300 import autotune

        def run_class(sub, prec):
            eng.jk_accumulate(D, [sub], [prec], prim_tau=FP32_THR)

        t0 = time.time()
        table = autotune.tune(run_class, [q64, q32], ["fp64", "fp32"])
        tune_s = time.time() - t0
        ms_tuned = float(np.median(time_events(torch, step_mixed, 5, flush)))
        ms64_tuned = float(np.median(time_events(torch, step_fp64, 3, flush)))
        autotune.reset()
        tuned = {"mixed_ms": ms_tuned, "fp64_ms": ms64_tuned, "tune_s": round(tune_s, 1),
                 "shapes": {f"{c}:{p}": [t, b] for (c, p), (t, b, _) in sorted(table.items()) if t}}

    # the two halves of the mixed build, each timed alone (all its classes, stream pool)
    ms_part = {}
    for name, lst, prec in (("fp64_list", q64, ACCURATE_LIST[HEADLINE]), ("fp32_list", q32, "fp32")):
        eng.jk_accumulate(D, [lst], [prec], prim_tau=FP32_THR)
        ms_part[name] = float(np.median(time_events(
            torch, lambda: eng.jk_accumulate(D, [lst], [prec], prim_tau=FP32_THR), 5, flush, preroll=True)))

    # roofline of the dominant kernel (per-class launches timed alone)
    peak64 = fma_peak(lib, torch, _lib.SQ_FP64)
    peak32 = fma_peak(lib, torch, _lib.SQ_FP32)
    peakdf = fma_peak(lib, torch, _lib.SQ_DF64)
    work64 = class_work(eng, q64)
    work32 = class_work(eng, q32, "fp32")
    work_all = class_work(eng, q_all)
    rows = []
    for lst, prec, work in ((q64, ACCURATE_LIST[HEADLINE], work64), (q32, "fp32", work32)):
        for c, w in work.items():
            off = np.zeros(_lib.SQ_MAX_QCLASS + 1, dtype=np.int64)
            off[c + 1:] = w["list_entries"]
            sub = QuartetList(lst.pairs[lst.class_off[c]:lst.class_off[c + 1]], off)
            eng.jk_accumulate(D, [sub], [prec], prim_tau=FP32_THR)
            t = float(np.median(time_events(
                torch, lambda: eng.jk_accumulate(D, [sub], [prec], prim_tau=FP32_THR), 3, flush, preroll=True)))
            # the arithmetic the launch ran in (the library's per-class double-float policy)
            ran = prec if prec in ("fp64", "fp32") else (
                "df64" if prec == "df64_prim" and eng.df_class(c, w["list_entries"]) else "fp64")
            rows.append({"class": w["class"], "precision": ran, "ms": t, "flops": w["flops"],
                         "quartets": w["quartets"]})
    rows.sort(key=lambda r: -r["ms"])
    dom = rows[0]
    # the launch that carries the most model FLOPs of the build (the longest
    # launches timed alone are short heavy-class lists, which overlap the others)
    big = max(rows, key=lambda r: r["flops"])
    # DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
    # capture of the same launch in this workload: the FP64 (dp|dp) launch of the
    # mixed_df large-bound list at 1e-3, the longest launch of that build
    ncu_traffic = {("2121", "fp64", "mixed_df", 1e-3, 16, "cc-pvdz"): 4.17e6}
    traffic = ncu_traffic.get((dom["class"], dom["precision"], HEADLINE, FP32_THR, WATERS, BASIS))
    # The J/K launch also zeroes two nbf^2 accumulators (negligible at 400 bf).
    peak = {"fp64": peak64, "fp32": peak32, "df64": peakdf}[dom["precision"]]
    achieved = dom["flops"] / (dom["ms"] * 1e-3) / 1e12
    fl64 = sum(w["flops"] for w in work_all.values())
    launches = sum(1 for c in range(_lib.SQ_MAX_QCLASS) if q64.class_off[c + 1] > q64.class_off[c]) + sum(
        1 for c in range(_lib.SQ_MAX_QCLASS) if q32.class_off[c + 1] > q32.class_off[c]) + 2

    # the small configurations of the reference timings (tests/golden/reference_timings.json),
    # through the public facade: ERI tensor and RHF SCF of one water (each the median of 3)
    small = []
    for basis in ("sto-3g", "cc-pvdz"):
        import slowquant_gb300.SlowQuant as sqm
        from slowquant_gb300 import systems as _sys

        te, ts = [], []
        for _ in range(3):
            A = sqm.SlowQuant()
            A.set_molecule(_sys.water_monomer(), distance_unit="angstrom")
            A.set_basis_set(basis)
            torch.cuda.synchronize()
            t0 = time.time()
            A.integral.electron_repulsion_tensor
            torch.cuda.synchronize()
            te.append(time.time() - t0)
            A.init_hartree_fock()
            A.hartree_fock.logger.print_output = False
            t0 = time.time()
            A.hartree_fock.run_restricted_hartree_fock()
            torch.cuda.synchronize()
            ts.append(time.time() - t0)
        small.append({"system": "H2O", "basis": basis, "eri_tensor_s": float(np.median(te)),
                      "scf_s": float(np.median(ts)), "E_hf": A.hartree_fock.E_hf})

    # AO -> MO transform (integralfunctions.py:199-211) on an n = m = 128 tensor: the four
    # rotate passes of sq_ao2mo_rotate, 2 n^4 m + 2 n^3 m^2 + 2 n^2 m^3 + 2 n m^4 FLOPs
    from slowquant_gb300.integralfunctions import two_electron_integral_transform

    na = 128
    gA = torch.randn((na, na, na, na), dtype=torch.float64, device="cuda")
    cA = torch.randn((na, na), dtype=torch.float64, device="cuda")
    two_electron_integral_transform(cA, gA)
    ms_ao2mo = float(np.median(time_events(torch, lambda: two_electron_integral_transform(cA, gA), 5, flush)))
    fl_ao2mo = 8.0 * na ** 5
    ao2mo = {"n": na, "m": na, "ms": ms_ao2mo, "tflops": fl_ao2mo / (ms_ao2mo * 1e-3) / 1e12,
             "frac_of_fp64_fma_peak": fl_ao2mo / (ms_ao2mo * 1e-3) / peak64}
    del gA

    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "quartets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"mixed_df": "df64+f64+f32 (mixed)"}.get(HEADLINE, "f64+f32 (mixed)"),
        "data": "synthetic",
        "config": config({"nbf": eng.nbf, "surviving_quartets": nq, "fp64_quartets": n64_unique,
                          "fp32_quartets": n32_unique, "list_entries_after_split": q_all.nquartet}),
        "fock_build_ms": {"mixed": ms_step, "mixed_precision_mode": HEADLINE, "fp64": ms64,
                          "speedup_mixed_vs_fp64": ms64 / ms_step,
                          "mixed_fp64_list_alone": ms_part["fp64_list"], "mixed_fp32_list_alone": ms_part["fp32_list"]},
        "quartets_per_s": {"mixed": nq / (ms_step * 1e-3), "fp64": nq / (ms64 * 1e-3)},
        "energy": {"E_hf_fp64": E64, "E_hf_mixed": Em, "abs_dE_mixed_vs_fp64": abs(Em - E64),
                   "E_hf_oracle": None if orc is None else orc["E_hf"],
                   "dE_fp64_vs_oracle": None if orc is None else E64 - orc["E_hf"],
                   "dE_mixed_vs_oracle": None if orc is None else Em - orc["E_hf"],
                   "oracle": "tests/golden/make_headline.py: the oracle's direct J/K and SCF, FP64, accurate Boys",
                   "mixed_builds": n_mixed_builds, "total_builds_mixed": len(jkm.builds),
                   "scf_iterations_fp64": len(jk64.builds), "scf_s_fp64": round(scf64_s, 2),
                   "scf_s_mixed": round(scfm_s, 2)},
        "e2e": {"value": world * nq / (e2e_ms * 1e-3), "unit": "quartets/s",
                "h2d_bytes_per_step": int(D.numel() * 8), "d2h_bytes_per_step": int(D.numel() * 8),
                "ms_per_step": e2e_ms},
        "roofline": {"bound": {"fp64": "fp64", "fp32": "fp32", "df64": "fp32 (double-float)"}[dom["precision"]],
                     "kernel": f"J/K class ({dom['class'][0]}{dom['class'][1]}|{dom['class'][2]}{dom['class'][3]}) "
                               f"{dom['precision']}",
                     "achieved": achieved, "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / (peak / 1e12),
                     "peak_source": "measured by sq_fma_probe (FMA loop, in the kernel's arithmetic) in this run",
                     "peaks_tflops": {"fp64": peak64 / 1e12, "df64": peakdf / 1e12, "fp32": peak32 / 1e12},
                     "traffic": traffic,
                     "traffic_source": None if traffic is None else
                     "ncu dram__bytes_read.sum + dram__bytes_write.sum, one capture of this launch in this workload",
                     "flops_per_launch": dom["flops"], "ms_per_launch": dom["ms"]},
        "roofline_by_work": {
            "kernel": f"J/K class ({big['class'][0]}{big['class'][1]}|{big['class'][2]}{big['class'][3]}) "
                      f"{big['precision']}",
            "bound": {"fp64": "fp64", "fp32": "fp32", "df64": "fp32 (double-float)"}[big["precision"]],
            "flops_per_launch": big["flops"], "ms_per_launch": big["ms"],
            "achieved": big["flops"] / (big["ms"] * 1e-3) / 1e12,
            "peak": {"fp64": peak64, "fp32": peak32, "df64": peakdf}[big["precision"]] / 1e12, "unit": "TFLOP/s",
            "frac": big["flops"] / (big["ms"] * 1e-3) / {"fp64": peak64, "fp32": peak32, "df64": peakdf}[big["precision"]]},
        "roofline_fp64_build": {"flops": fl64, "ms": ms64, "achieved_tflops": fl64 / (ms64 * 1e-3) / 1e12,
                                "peak_tflops": peak64 / 1e12, "frac": fl64 / (ms64 * 1e-3) / peak64},
        "small_systems": small,
        "ao2mo": ao2mo,
        "tau_sweep": sweep,
        "chunk_precision": chunk_modes,
        "prim_precision": prim_modes,
        "df64": df_full,
        "mixed_df": df_modes,
        "autotuned_launch_shapes": tuned,
        "kernels_by_time": rows[:8],
        "fp32_kernels_by_time": [r for r in rows if r["precision"] == "fp32"][:8],
        "gpu_launches": launches * args.steps,
        "clocks": clocks,
        "setup_s": round(setup_s, 2),
        "wall_timed_s": round(wall_mixed, 3),
        "hbm_peak_gbs": measured_peaks().get("hbm_gbs"),
        "jk_streams": int(lib.sq_get_option(_lib.SQ_OPT_JK_STREAMS)),
    }
    if rank == 0 and not args.no_cpu:
        pairs_host = (eng.pair_shells[eng.slot_pair], q_all.pairs[: q_all.nquartet].cpu().numpy())
        rate, nthreads, n, dt = cpu_sample(None, args.cpu_seconds, 0, pairs_host, geom)
        line["gpu_vs_cpu_baseline"] = {"mixed": value / rate, "fp64": nq / (ms64 * 1e-3) / rate,
                                       "mixed_e2e": line["e2e"]["value"] / rate}
        line["cpu_baseline"] = {
            "value": rate, "unit": "quartets/s", "cores": nthreads, "kind": "port",
            "sample": f"{n} uniformly random surviving unique shell quartets of the workload "
                      f"({dt:.1f} s) through the oracle's faithful C restatement of electron_repulsion_integral"}
    if rank == 0 and args.secondary:
        line["secondary"] = {"batch": batch_quick(), "gradient": gradient_quick()}
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- secondary workloads
def batch_quick() -> dict:
    """The batched-SCF workload (256 water clusters, 6-31G*) once in FP64 and once in mixed_df,
    each after a warm-up run that captures its iteration graphs (the full sweep: --workload batch)."""
    import torch

    from slowquant_gb300.batch import BatchEngine, BatchSCF

    mols, sizes = _batch_molecules(256)
    be = BatchEngine(mols)
    out, E = {}, {}
    for prec in ("fp64", "mixed_df"):
        scf = BatchSCF(be, prec)
        scf.run()
        torch.cuda.synchronize()
        t0 = time.time()
        E[prec] = scf.run()
        torch.cuda.synchronize()
        dt = time.time() - t0
        out[prec] = {"molecules_per_s": len(mols) / dt, "scf_s": round(dt, 3), "iterations": scf.iterations}
    return {"workload": f"{len(mols)} water clusters (H2O)_k, k~U{{1..6}} (seed 256), 6-31G*, full RHF SCF, "
                        f"{int(sum(m.number_bf for m in mols))} bf in total",
            **out, "max_abs_dE_mixed_df_vs_fp64": float(np.max(np.abs(E["mixed_df"] - E["fp64"])))}


def gradient_quick() -> dict:
    """SCF and adjoint RHF gradient of n-octane / cc-pVDZ (the full line with finite-difference checks:
    --workload gradient)."""
    import torch

    from slowquant_gb300 import systems
    from slowquant_gb300.gradient import rhf_gradient, scf_energy
    from slowquant_gb300.molecule import _Molecule

    m = _Molecule(systems.octane(), 0, "angstrom")
    m._set_basis_set("cc-pvdz")
    rhf_gradient(m)  # warm-up
    torch.cuda.synchronize()
    t0 = time.time()
    E, D, eng = scf_energy(m)
    torch.cuda.synchronize()
    t_scf = time.time() - t0
    t0 = time.time()
    g = eng.nuclear_gradient(D, 1e-12)
    torch.cuda.synchronize()
    return {"workload": "n-octane cc-pVDZ (210 bf), FP64", "scf_s": round(t_scf, 3),
            "gradient_s": round(time.time() - t0, 3), "max_abs_grad": float(np.abs(g).max())}
def _batch_molecules(n: int, seed: int = 256):
    """n seeded water clusters (H2O)_k, k uniform in 1..6, 6-31G*."""
    from slowquant_gb300 import systems
    from slowquant_gb300.molecule import _Molecule

    rng = np.random.default_rng(seed)
    sizes = rng.integers(1, 7, n)
    mols = []
    for i, k in enumerate(sizes):
        box = 9.0 * (k / 8.0) ** (1.0 / 3.0) + 1.0
        m = _Molecule(systems.water_cluster(int(k), box, seed=1000 + i), 0, "angstrom")
        m._set_basis_set("6-31G*")
        mols.append(m)
    return mols, sizes


def batch_arm(args) -> None:
    """Batched RHF of many small molecules: molecules/s over whole SCF runs, FP64 and mixed."""
    import torch

    from slowquant_gb300.batch import BatchEngine, BatchSCF

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mols, sizes = _batch_molecules(args.batch_size)
    t0 = time.time()
    be = BatchEngine(mols)
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    res = {}
    # launch shapes of every class and precision from the project's autotuner,
    # tuned once on this batch's lists (the mixed lists include the FP64 ones)
    from slowquant_gb300 import autotune

    t0 = time.time()
    tuning = BatchSCF(be, "mixed").autotune()
    tune_s = time.time() - t0
    steps = max(1, min(args.steps, 3))

    def timed_runs(scf):
        scf.run()  # warm-up run: captures the iteration graphs, which later runs replay
        torch.cuda.synchronize()
        t0 = time.time()
        for _ in range(steps):
            E = scf.run()
        torch.cuda.synchronize()
        return E, (time.time() - t0) / steps

    # FP64 and mixed, and the same with double-float arithmetic in place of FP64
    taus = {"fp64": 1e-4, "mixed": 1e-4, "df64": 1e-4, "mixed_df": 1e-4}
    for prec in ("fp64", "mixed", "df64", "mixed_df"):
        t0 = time.time()
        scf = BatchSCF(be, prec, fp32_threshold=taus[prec])
        torch.cuda.synchronize()
        prep_s = time.time() - t0
        E, scf_s = timed_runs(scf)
        mode = "fp64" if prec in ("fp64", "df64") else "mixed"
        ms_fock = float(np.median(time_events(torch, lambda: scf.fock(mode), 5)))
        # the same SCF with the built-in launch shapes, and with eager iterations (no graphs)
        autotune.reset()
        _, scf_default_s = timed_runs(BatchSCF(be, prec, fp32_threshold=taus[prec]))
        _, scf_eager_s = timed_runs(BatchSCF(be, prec, fp32_threshold=taus[prec], use_graphs=False))
        autotune.apply(tuning)
        res[prec] = {"molecules_per_s": len(mols) / scf_s, "scf_s": scf_s,
                     "per_molecule_scf_ms": scf_s * 1e3 / len(mols), "iterations": scf.iterations,
                     "host_syncs_per_scf": scf.host_syncs, "fock_build_ms": ms_fock,
                     "molecules_per_s_default_launch_shapes": len(mols) / scf_default_s,
                     "molecules_per_s_eager_iterations": len(mols) / scf_eager_s,
                     "list_prep_s": round(prep_s, 2), "fp32_threshold": taus[prec], "E": E}
    dE = {p: float(np.max(np.abs(res[p]["E"] - res["fp64"]["E"]))) for p in ("mixed", "df64", "mixed_df")}
    for r in res.values():
        r.pop("E")
    line = {
        "metric": "molecules/s, batched RHF (FP64 vs mixed)", "value": res["mixed_df"]["molecules_per_s"],
        "unit": "molecules/s", "n_gpus": 1, "steps": max(1, min(args.steps, 3)), "warmup": 1,
        "ms_per_step": res["mixed_df"]["scf_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "df64+f32 (mixed_df)", "data": "synthetic",
        "precision_mode": "mixed_df (quartets with bound below 1e-4 in FP32, the others in double-float; "
                          "the SCF ends in double-float)",
        "config": {"workload": f"{len(mols)} water clusters (H2O)_k, k~U{{1..6}} (seed 256), 6-31G*, full RHF SCF",
                   "total_bf": int(sum(m.number_bf for m in mols)), "waters": int(sizes.sum()),
                   "step": "one batched SCF to convergence (dE, rmsD < 1e-9) of every molecule, each iteration "
                           "replayed from a CUDA graph"},
        "fp64": res["fp64"], "mixed": res["mixed"], "df64": res["df64"], "mixed_df": res["mixed_df"],
        "max_abs_dE_mixed_vs_fp64": dE["mixed"], "max_abs_dE_vs_fp64": dE,
        "setup_s": round(setup_s, 2), "autotune_s": round(tune_s, 2),
        "launch_shapes": {f"{c}:{p}": [t, b] for (c, p), (t, b, _) in sorted(tuning.items()) if t},
    }
    autotune.reset()
    print(json.dumps(line), flush=True)


def gradient_arm(args) -> None:
    """RHF nuclear gradient (SCF + adjoint gradient) timings for H24 STO-3G and n-octane cc-pVDZ."""
    import torch

    from slowquant_gb300 import systems
    from slowquant_gb300.gradient import rhf_gradient, scf_energy
    from slowquant_gb300.molecule import _Molecule

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    out = {}
    for name, geom, basis in (("H24 chain STO-3G", systems.hydrogen_chain(24, seed=24), "sto-3g"),
                              ("n-octane cc-pVDZ", systems.octane(), "cc-pvdz")):
        m = _Molecule(geom, 0, "angstrom")
        m._set_basis_set(basis)
        rhf_gradient(m)  # warm-up
        torch.cuda.synchronize()
        t0 = time.time()
        E, D, eng = scf_energy(m)
        torch.cuda.synchronize()
        t_scf = time.time() - t0
        t0 = time.time()
        g = eng.nuclear_gradient(D, 1e-12)
        torch.cuda.synchronize()
        t_grad = time.time() - t0
        # central finite differences (step 1e-4 bohr) of the FP64 GPU energy
        from slowquant_gb300.gradient import molecule_from_coords
        from slowquant_gb300.molecule import ANGSTROM_TO_BOHR

        symbols = [a.split()[0] for a in geom.split(";") if a.strip()]
        xyz = np.array([[float(v) * ANGSTROM_TO_BOHR for v in a.split()[1:]] for a in geom.split(";") if a.strip()])
        if basis == "sto-3g":
            comps = [(a, 0) for a in range(len(xyz))]
        else:
            comps = [(0, 0), (3, 1), (9, 2), (20, 0)]
        h = 1e-4
        dev = []
        for a, d in comps:
            xp, xm = xyz.copy(), xyz.copy()
            xp[a, d] += h
            xm[a, d] -= h
            Ep = scf_energy(molecule_from_coords(symbols, xp, basis), conv=1e-11)[0]
            Em = scf_energy(molecule_from_coords(symbols, xm, basis), conv=1e-11)[0]
            dev.append(abs((Ep - Em) / (2 * h) - g[a, d]))
        out[name] = {"nbf": m.number_bf, "scf_s": round(t_scf, 3), "gradient_s": round(t_grad, 3),
                     "max_abs_grad": float(np.abs(g).max()),
                     "fd_check": {"components": len(comps), "step_bohr": h,
                                  "max_abs_dev_eh_per_bohr": float(max(dev))}}
    line = {"metric": "RHF nuclear gradient wall time (s)", "value": out["n-octane cc-pVDZ"]["gradient_s"],
            "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 1, "higher_is_better": False, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "adjoint RHF gradient after SCF"}, "systems": out}
    print(json.dumps(line), flush=True)


def main() -> None:
    global WATERS, SEED, BASIS, HEADLINE, FP32_THR
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--waters", type=int, default=16, choices=[8, 16],
                    help="cluster size (16 is the benchmark workload; 8 for quick profiling)")
    ap.add_argument("--basis", default="cc-pvdz", choices=sorted(BASES),
                    help="cc-pvdz is the benchmark workload; cc-pvtz adds f shells on O (secondary line)")
    ap.add_argument("--workload", default="fock", choices=["fock", "batch", "gradient"],
                    help="fock: the headline Fock-build line; batch / gradient: secondary measurements")
    ap.add_argument("--batch-size", type=int, default=256)
    ap.add_argument("--jk-streams", type=int, default=0, help="J/K class launch streams (0: library default)")
    ap.add_argument("--tau-sweep", type=float, nargs="*", default=[1e-5, 1e-4, 1e-3, 1e-2, 1e-1],
                    help="FP32 Schwarz thresholds reported beside the headline (empty: skip)")
    ap.add_argument("--autotune", action="store_true",
                    help="also time the build with the autotuner's launch shapes for this workload")
    ap.add_argument("--prim-sweep", type=float, nargs="*", default=[1e-4, 1e-3, 1e-2],
                    help="bounds of the primitive-level precision mode reported beside the headline (empty: skip)")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false",
                    help="skip the short batched-SCF and gradient measurements appended to the headline line")
    ap.add_argument("--no-df", dest="df", action="store_false",
                    help="skip the double-float (df64, mixed_df) measurements")
    ap.add_argument("--precision", default=HEADLINE, choices=sorted(ACCURATE_LIST),
                    help="precision mode of the headline mixed build")
    ap.add_argument("--fp32-threshold", type=float, default=FP32_THR,
                    help="bound below which quartets (and, in mixed_prim / mixed_df, primitive quartets) run in FP32")
    args = ap.parse_args()
    WATERS = SEED = args.waters
    BASIS = args.basis
    HEADLINE, FP32_THR = args.precision, args.fp32_threshold
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "batch":
        batch_arm(args)
    elif args.workload == "gradient":
        gradient_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
