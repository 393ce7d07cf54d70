#!/usr/bin/env python3
"""Benchmark of the linear-optics hot path on GB300.

Headline workload (one step = one pass over one batch): exact permanents of 8192
complex128 Haar submatrices, n uniform in 8..24, rows/columns drawn without
replacement from a 1024x1024 Haar unitary (seed 0), computed in native FP64 (the
reference's arithmetic) by one permanent plan (one CUDA graph: prepare, the size bins
as concurrent branches, reduce).  `value` is perms/s with the matrices resident in
HBM; `e2e` is the same through the C ABI from pinned host buffers with both copies
inside the timed region.  The float-float arithmetic (opt-in) is a secondary line.

Secondary lines in the same JSON: SLOS full distribution m=24/n=12 (amplitudes/s,
HBM roofline), batched SLOS forward+adjoint on 256 Clements meshes m=16/n=8,
Clifford & Clifford sampling n=20/m=400, and the small m=12/n=6 SLOS + 1000 Naive
amplitudes case.

`--impl reference` times the CPU restatement of the reference path (the C oracle,
OpenMP on every host core) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Haar perms/s & SLOS amps/s (frac. of roofline); ESS/s MCMC vs exact sampler"
WORKLOAD = ("8192 Haar-submatrix permanents, n~U{8..24}, rows/cols without replacement from a "
            "1024x1024 Haar unitary (numpy legacy seed 0; sizes/rows/cols from default_rng(seed))")
N_MATS, BIG = 8192, 1024


def make_batch(seed: int):
    from perceval_gb300.utils.matrix import random_unitary
    U = random_unitary(BIG, seed=0)
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(N_MATS):
        n = int(rng.integers(8, 25))
        mats.append(np.ascontiguousarray(U[np.ix_(rng.choice(BIG, n, False), rng.choice(BIG, n, False))]))
    sizes = np.array([a.shape[0] for a in mats], dtype=np.int32)
    offs = np.zeros(N_MATS, dtype=np.int64)
    offs[1:] = np.cumsum([a.size for a in mats])[:-1]
    flat = np.concatenate([a.reshape(-1) for a in mats])
    return mats, flat, offs, sizes


def glynn_flops(n) -> float:
    """Algorithmic FP64 flops of one n x n Glynn permanent: 2^(n-1) (8n - 4)."""
    return (2.0 ** (n - 1)) * (8 * n - 4)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, out: Path):
        self.out = out
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.out, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self) -> dict:
        try:
            rows = [r.split(",") for r in self.out.read_text().strip().splitlines() if r.strip()]
        except OSError:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows)
        power = [float(r[3]) for r in rows if r[3].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        loaded = [s for s, p in zip(sm, power) if p > 0.5 * max(power)] if power else sm
        return {"sm_mhz": statistics.median(loaded or sm), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(power) if power else None}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def max_over_ranks(x: float, device="cpu") -> float:
    """Max of x over the ranks of the default process group (x itself without one):
    the job's time is its slowest replica's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step: float, world: int, steps: int, seconds: float) -> float:
    """Units per second of the whole job: every rank processes units_per_rank_step per step
    (weak scaling, independent replicas), timed by the slowest rank."""
    return world * units_per_rank_step * steps / seconds


def measured_fp64_peak(torch) -> float:
    """cuBLAS DGEMM 4096^3, best of 5, TFLOP/s (the FP64 roofline denominator)."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        s, e = torch.cuda.Event(True), torch.cuda.Event(True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2 * 4096 ** 3 / (best * 1e-3) / 1e12


def traffic_from_profile(name: str):
    p = ROOT / "profiles" / f"{name}.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            return None
    return None


# ----------------------------------------------------------------------------- CPU
def _cpu_perm_rate(oracle, budget_s: float) -> tuple[float, dict, float]:
    """Whole-batch perms/s of the host-tuned Glynn, extrapolated from a stratified sample:
    per size n, batches of the batch's own matrices of that size, doubling until they take
    about budget / 17 seconds; the full-batch time is the per-size times x the size counts."""
    _, flat, offs, sizes = make_batch(seed=0)
    counts = np.bincount(sizes, minlength=25)
    per_n, used = {}, {}
    spent = 0.0
    for n in range(8, 25):
        idx = np.nonzero(sizes == n)[0]
        k, dt = 1, 0.0
        while True:
            sel = idx[:k]
            sub = np.concatenate([flat[offs[i]:offs[i] + n * n] for i in sel])
            t0 = time.perf_counter()
            oracle.perm_batch_fast(sub, np.arange(len(sel), dtype=np.int64) * n * n, np.full(len(sel), n, np.int32))
            dt = time.perf_counter() - t0
            spent += dt
            if dt >= budget_s / 17 / 2 or k >= len(idx):
                break
            k = min(len(idx), 2 * k)
        per_n[n] = dt / len(sel)
        used[n] = len(sel)
    total = sum(counts[n] * per_n[n] for n in range(8, 25))
    return N_MATS / total, used, spent


def cpu_perm_baseline(budget_s: float = 15.0, single_thread_s: float = 0.0) -> dict:
    """The host-tuned FP64 Glynn of the CPU restatement (C, OpenMP over every (matrix,
    chunk) task on all host threads, sixteen Gray-code steps at once in vector lanes) on a
    stratified sample of the batch (``_cpu_perm_rate``); with ``single_thread_s`` also the
    same on one thread, on a sample of about that many seconds."""
    from oracle import oracle
    value, used, spent = _cpu_perm_rate(oracle, budget_s)
    threads = oracle.num_threads()
    extra = {}
    if single_thread_s > 0:
        oracle.set_threads(1)
        try:
            extra["single_thread_value"] = _cpu_perm_rate(oracle, single_thread_s)[0]
        finally:
            oracle.set_threads(threads)
    return {"value": value, "unit": "perms/s", "cores": threads, "kind": "port", **extra,
            "flags": "gcc -O3 -std=c11 -fopenmp (portable: on the Arm host NEON, 128-bit like its SVE, is the "
                     "baseline ISA), multiply-adds fused in the timed kernel",
            "sample": f"{sum(used.values())} matrices of the batch, every size n=8..24 "
                      f"({used[24]} of n=24), {spent:.1f} s of CPU work in batched calls; full-batch time "
                      f"extrapolated from the per-size times and the size counts"}


def cpu_context() -> dict:
    """The oracle's host-tuned paths (C, OpenMP on all host threads: SLOS and its gradient,
    the exact sampler, Gurvits estimates; SLOS and the sampler also on one thread) on bounded
    samples of the secondary workloads, for context beside the GPU lines: a few seconds of
    host time."""
    from oracle import oracle
    from perceval_gb300.utils.matrix import random_unitary
    out = {"threads_openmp": oracle.num_threads()}

    def t(fn):
        t0 = time.perf_counter()
        fn()
        return time.perf_counter() - t0
    U12 = random_unitary(12, seed=0)
    out["slos_m12_n6_ms"] = 1e3 * t(lambda: oracle.slos_fast(U12, [1] * 6 + [0] * 6))
    U20 = random_unitary(20, seed=0)
    out["slos_m20_n10_ms"] = 1e3 * t(lambda: oracle.slos_fast(U20, [1] * 10 + [0] * 10))
    U16 = random_unitary(16, seed=0)
    inp16 = [1] * 8 + [0] * 8
    out["slos_m16_n8_one_circuit_ms"] = 1e3 * t(lambda: oracle.slos_fast(U16, inp16))
    w = np.random.default_rng(1).normal(size=math.comb(23, 8))
    out["slos_grad_m16_n8_one_circuit_ms"] = 1e3 * t(lambda: oracle.slos_grad_fast(U16, inp16, w))
    U64 = random_unitary(64, seed=0)
    out["all_outputs_m64_n4_ms"] = 1e3 * t(lambda: oracle.slos_fast(U64, [1] * 4 + [0] * 60))
    U400 = random_unitary(400, seed=0)
    ns = 32 * oracle.num_threads()
    # the sampler in parallel over samples, all k sub-permanents of a step from one Glynn sum
    out["cc2017_n20_m400_samples_per_s"] = ns / t(lambda: oracle.cc2017_fast(U400, [1] * 20 + [0] * 380, ns, seed=1))
    Ubig = random_unitary(1024, seed=0)
    rng = np.random.default_rng(11)
    gm = [Ubig[np.ix_(rng.choice(1024, 20, False), rng.choice(1024, 20, False))] for _ in range(20)]
    draws = 100000
    dt = t(lambda: oracle.gurvits_batch_fast(gm, draws, 1, [i * draws for i in range(len(gm))]))
    out["gurvits_n20_draws_per_s"] = 20 * draws / dt
    # single-thread rates of the SLOS and sampler legs
    threads = oracle.num_threads()
    oracle.set_threads(1)
    try:
        out["slos_m20_n10_ms_1thread"] = 1e3 * t(lambda: oracle.slos_fast(U20, [1] * 10 + [0] * 10))
        out["cc2017_n20_m400_samples_per_s_1thread"] = 16 / t(
            lambda: oracle.cc2017_fast(U400, [1] * 20 + [0] * 380, 16, seed=1))
    finally:
        oracle.set_threads(threads)
    return out


def run_reference(args):
    ws, rank = dist_setup()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    vals = []
    for _ in range(args.warmup):
        cpu_perm_baseline(budget_s=1.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_perm_baseline(budget_s=8.0))
    wall = time.perf_counter() - t0
    v = statistics.median(x["value"] for x in vals)
    cb = dict(vals[0])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "perms/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex128 (FP64)",
            "data": "synthetic", "config": {"workload": WORKLOAD, "implementation": "CPU oracle restating the "
                                            "reference path (exqalibur is closed and absent)"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "perms/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU
def run_ours(args):
    import torch
    ws, rank = dist_setup()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    from perceval_gb300 import _native, autotune
    from perceval_gb300.utils.matrix import random_unitary
    _native.load()
    dev = torch.device("cuda")
    # the nvidia-smi clock samples of the timed region are logged here (the JSON line carries
    # their summary)
    out_dir = Path(os.environ.get("PCVL_BENCH_OUT", str(ROOT / "bench_out")))
    out_dir.mkdir(parents=True, exist_ok=True)
    # launch shapes of the permanent bins: the cached autotuner table for this GPU, or a
    # fresh tuning run (about 20 s, untimed) that is then cached
    t_tune = time.perf_counter()
    table = autotune.ensure_tuned(range(8, 25), log=lambda s: print(s, file=sys.stderr), precision="fp64")
    tuning = {"sizes": "8..24", "arithmetic": "fp64",
              "source": "cached table" if table is None else "tuned in this run",
              "seconds": round(time.perf_counter() - t_tune, 1)}

    mats, flat, offs, sizes = make_batch(seed=rank)
    flops_total = float(sum(glynn_flops(int(n)) for n in sizes))
    flat_d = torch.from_numpy(flat).to(dev)
    out_d = torch.empty(N_MATS, dtype=torch.complex128, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    bins = len(set(int(n) for n in sizes))
    launches_per_step = bins + 2  # graph nodes: prepare + one per size bin + reduce
    plan = _native.PermPlan(offs, sizes, precision="fp64")  # fixed batch shape: one CUDA graph per step

    def step():
        plan(flat_d, out_d)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    ev = [(torch.cuda.Event(True), torch.cuda.Event(True)) for _ in range(args.steps)]
    clocks = Clocks(out_dir / "bench_clocks.csv")
    with clocks:
        barrier()
        for s, e in ev:
            flush.zero_()  # L2 flush between timed steps, outside the events
            s.record()
            step()
            e.record()
        barrier()
    ms = max_over_ranks(sum(s.elapsed_time(e) for s, e in ev), dev)
    value = whole_job_rate(N_MATS, ws, args.steps, ms * 1e-3)

    # e2e through the C ABI from pinned host buffers (copies inside the timed region)
    host_in = torch.from_numpy(flat).pin_memory()
    host_out = torch.empty(N_MATS, dtype=torch.complex128).pin_memory()
    dev_in = torch.empty_like(flat_d)

    def e2e_step():
        dev_in.copy_(host_in, non_blocking=True)
        plan(dev_in, out_d)
        host_out.copy_(out_d, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dev)
    e2e = {"value": whole_job_rate(N_MATS, ws, args.steps, e2e_s), "unit": "perms/s",
           "h2d_bytes_per_step": int(flat.nbytes),
           "d2h_bytes_per_step": int(N_MATS * 16)}

    # dominant kernel alone: the n = 24 bin (its CTAs' share of the step is largest), FP64
    sel = [i for i in range(N_MATS) if sizes[i] == 24]
    sub = np.concatenate([mats[i].reshape(-1) for i in sel])
    sub_d = torch.from_numpy(sub).to(dev)
    sub_out = torch.empty(len(sel), dtype=torch.complex128, device=dev)
    sub_offs = np.arange(len(sel), dtype=np.int64) * 576
    sub_sizes = np.full(len(sel), 24, dtype=np.int32)
    _native.permanent_batch(sub_d, sub_offs, sub_sizes, sub_out, precision="fp64")
    torch.cuda.synchronize()
    kt = []
    for _ in range(3):
        flush.zero_()
        s, e = torch.cuda.Event(True), torch.cuda.Event(True)
        s.record()
        _native.permanent_batch(sub_d, sub_offs, sub_sizes, sub_out, precision="fp64")
        e.record()
        e.synchronize()
        kt.append(s.elapsed_time(e))
    k_ms = statistics.median(kt)
    fp64_peak = measured_fp64_peak(torch)
    achieved = len(sel) * glynn_flops(24) / (k_ms * 1e-3) / 1e12
    ki = (2 * 24) // 3  # rows of each n = 24 product multiplied on the integer pipes
    roofline = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": traffic_from_profile("perm_bin_fx_n24"),
                "kernel": "perm_bin_fx<24> (the n=24 bin of the batch)",
                "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 on this GPU (the measured peaks file "
                               "has no FP64 entry)",
                "algorithmic_flops_per_permanent": "2^(n-1) (8n - 4)",
                "note": f"FP64-class arithmetic on two pipes at once: exact fixed-point row sums on the "
                        f"integer pipe; of each sign vector's product of 24 row sums, {24 - ki} are multiplied "
                        f"in FP64 and {ki} in 64-bit block floating point on the integer pipes (62 significant "
                        f"bits, finer than FP64), and the halves meet in the compensated FP64 accumulation. "
                        f"The FP64 pipe issues 4 (n - {ki}) = {4 * (24 - ki)} instructions per sign vector for "
                        f"8n - 4 = 188 algorithmic flops, so frac above 1 is the integer pipes' share; with "
                        f"every product in FP64 the kernel reached 1.04 of this peak, with FP64 row sums "
                        f"(secondary perm_batch_fp64_dadd) 6n - 4 instructions, frac <= 0.67",
                "step_tflops": flops_total / (ms / args.steps * 1e-3) / 1e12}

    line = {"metric": METRIC, "value": value, "unit": "perms/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex128 (FP64)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas x{ws}",
                       "launch": f"one CUDA graph per step (pcvl_perm_plan_execute: prepare, {bins} size bins as "
                                 "concurrent branches, reduce)",
                       "tuning": tuning},
            "e2e": e2e, "gpu_launches": launches_per_step * args.steps, "roofline": roofline,
            "clocks": clocks.summary()}

    if rank == 0 and not args.skip_secondary:
        sec = {}
        # the same batch through the plan-free call (host planning, staged descriptors and
        # one launch per bin on the stream), device-timed like the headline
        kb = []
        for _ in range(3):
            flush.zero_()
            s, e = torch.cuda.Event(True), torch.cuda.Event(True)
            s.record()
            _native.permanent_batch(flat_d, offs, sizes, out_d, precision="fp64")
            e.record()
            e.synchronize()
            kb.append(s.elapsed_time(e))
        sec["perm_batch_call_8192"] = {"ms": statistics.median(kb), "arithmetic": "fp64",
                                       "perms_per_s": N_MATS / (statistics.median(kb) * 1e-3)}
        # the same batch in float-float (opt-in) and in FP64 with FP64 row sums: plans of
        # their own, their own tuned shapes
        ref64 = out_d.clone()
        for prec, key in (("float-float", "perm_batch_float_float"), ("fp64-dadd", "perm_batch_fp64_dadd")):
            autotune.ensure_tuned(range(8, 25), log=lambda s: print(s, file=sys.stderr), precision=prec)
            o_plan = _native.PermPlan(offs, sizes, precision=prec)
            o_out = torch.empty_like(out_d)
            for _ in range(args.warmup):
                o_plan(flat_d, o_out)
            torch.cuda.synchronize()
            kf = []
            for _ in range(args.steps):
                flush.zero_()
                s, e = torch.cuda.Event(True), torch.cuda.Event(True)
                s.record()
                o_plan(flat_d, o_out)
                e.record()
                e.synchronize()
                kf.append(s.elapsed_time(e))
            o_ms = statistics.mean(kf)
            sec[key] = {"arithmetic": prec, "ms_per_step": o_ms, "perms_per_s": N_MATS / (o_ms * 1e-3),
                        "speedup_vs_fp64": (ms / args.steps) / o_ms,
                        "max_rel_diff_vs_fp64": float(((o_out - ref64).abs() / ref64.abs()).max()),
                        "step_tflops": flops_total / (o_ms * 1e-3) / 1e12}
            del o_plan
        sec.update(secondary(torch, _native, random_unitary, dev, flush, fp64_peak))
        line["secondary"] = sec
    if rank == 0 and ws == 1 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_perm_baseline(single_thread_s=4.0)
        if "secondary" in line:
            line["secondary"]["cpu_context"] = cpu_context()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def secondary(torch, _native, random_unitary, dev, flush, fp64_peak_tflops):
    res = {}

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            flush.zero_()
            s, e = torch.cuda.Event(True), torch.cuda.Event(True)
            s.record()
            fn()
            e.record()
            e.synchronize()
            ts.append(s.elapsed_time(e))
        return statistics.median(ts)

    hbm = None
    try:
        hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]
    except (OSError, ValueError, KeyError):
        hbm = 6800.0
    # SLOS m=24, n=12 in both arithmetics
    m, n = 24, 12
    Ud = torch.from_numpy(random_unitary(m, seed=0)).to(dev)
    Ls = [math.comb(m + k - 1, k) for k in range(n + 1)]
    alg_bytes = 16 * sum(Ls[k - 1] + Ls[k] for k in range(1, n + 1))
    # the arithmetic floors: layer k has m L_{k-1} (state, occupied mode) terms (the states with
    # mode 0 occupied number L_{k-1}); an FP64 complex multiply-add is 4 DFMA (8 flops), at the
    # FP64 rate measured in this run; a float-float one is 48 FP32 operations, at the 36.8 T
    # FP32 operations/s measured on this part
    terms = m * sum(Ls[k - 1] for k in range(1, n + 1))
    fp64_floor_ms = terms * 8 / (fp64_peak_tflops * 1e12) * 1e3
    fp32_floor_ms = terms * 48 / 36.8e12 * 1e3
    p64 = None
    for prec, key in (("fp64", "slos_m24_n12"), ("float-float", "slos_m24_n12_float_float")):
        plan = _native.SlosPlan(m, [1] * n + [0] * (m - n), precision=prec)
        t_fwd = timed(lambda: plan.forward(Ud), reps=2)
        probs = plan.probabilities()
        t_prob = timed(lambda: plan.probabilities(probs), reps=2)
        # every probability without storing the last layer (its probabilities written directly)
        t_fused = timed(lambda: plan.forward_probabilities(Ud, probs), reps=2)
        row = {"arithmetic": prec, "amps_per_s": Ls[n] / (t_fwd * 1e-3), "forward_ms": t_fwd,
               "probabilities_ms": t_prob, "forward_probabilities_ms": t_fused, "multiply_add_terms": terms,
               "algorithmic_gb": alg_bytes / 1e9, "hbm_frac": alg_bytes / (t_fwd * 1e-3) / 1e9 / hbm,
               "hbm_peak_gbs": hbm, "sum_p": float(probs.sum())}
        if prec == "fp64":
            row.update({"fp64_floor_ms": fp64_floor_ms, "fp64_frac": fp64_floor_ms / t_fwd,
                        "fp64_peak_tflops": fp64_peak_tflops})
            p64 = probs[::997].clone()
        else:
            row.update({"fp32_floor_ms": fp32_floor_ms, "fp32_frac": fp32_floor_ms / t_fwd,
                        "max_abs_diff_vs_fp64_sampled": float((probs[::997] - p64).abs().max())})
        res[key] = row
        del plan, probs
        torch.cuda.empty_cache()
    t_fwd = res["slos_m24_n12"]["forward_ms"]
    # the same circuit heralded: modes 20..23 detected as 1, 1, 0, 0 (a masked plan keeps only
    # the states that can still end with that pattern)
    from perceval_gb300.utils import FSMask
    herald = "*" * 20 + "1100"
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan = _native.SlosPlan(m, [1] * n + [0] * (m - n), mask=FSMask(m, n, [herald]))
    torch.cuda.synchronize()
    t_build = 1e3 * (time.perf_counter() - t0)
    t_fm = timed(lambda: plan.forward(Ud), reps=3)
    pm = plan.probabilities()
    t_pm = timed(lambda: plan.probabilities(pm), reps=3)
    res["slos_masked_m24_n12_heralded"] = {
        "mask": herald, "kept_outputs": plan.count, "full_outputs": Ls[n], "plan_build_ms": t_build,
        "forward_ms": t_fm, "probabilities_ms": t_pm, "full_forward_ms": t_fwd, "speedup_vs_full": t_fwd / t_fm,
        "kept_amps_per_s": plan.count / (t_fm * 1e-3), "device_gb": plan.device_bytes / 1e9,
        "heralded_probability": float(pm.sum())}
    del plan, pm
    torch.cuda.empty_cache()
    plan = _native.SlosPlan(20, [1] * 10 + [0] * 10)
    U20 = torch.from_numpy(random_unitary(20, seed=0)).to(dev)
    t_f20 = timed(lambda: plan.forward(U20), reps=3)
    p20 = plan.probabilities()
    t_p20 = timed(lambda: plan.probabilities(p20), reps=3)
    res["slos_m20_n10"] = {"forward_ms": t_f20, "probabilities_ms": t_p20, "outputs": plan.count}
    del plan, p20
    # SLAP: every output of one input without intermediate layers, many modes and few photons
    # (SLOS plans stop at 32 modes); one line where both run
    for (ms, ns) in [(1024, 3), (256, 4), (64, 6), (64, 4)]:
        inp = [1] * ns + [0] * (ms - ns)
        Us = torch.from_numpy(random_unitary(ms, seed=0)).to(dev)
        cnt = _native.slap_output_count(ms, inp)
        ps = torch.empty(cnt, dtype=torch.float64, device=dev)
        t_s = timed(lambda: _native.slap_all(Us, inp, out=ps), reps=3)
        res[f"slap_m{ms}_n{ns}"] = {"outputs": cnt, "ms": t_s, "outputs_per_s": cnt / (t_s * 1e-3),
                                    "written_gbs": 8 * cnt / (t_s * 1e-3) / 1e9, "sum_p": float(ps.sum())}
        del ps
    torch.cuda.empty_cache()
    inp = [1] * 6 + [0] * 26
    U32 = torch.from_numpy(random_unitary(32, seed=0)).to(dev)
    plan = _native.SlosPlan(32, inp)
    p32 = torch.empty(plan.count, dtype=torch.float64, device=dev)

    def slos32():
        plan.forward(U32)
        plan.probabilities(p32)
    t_slos32 = timed(slos32, reps=3)
    ps = torch.empty_like(p32)
    t_slap32 = timed(lambda: _native.slap_all(U32, inp, out=ps), reps=3)
    res["slap_vs_slos_m32_n6"] = {"outputs": plan.count, "slos_ms": t_slos32, "slap_ms": t_slap32,
                                  "max_abs_diff": float((ps - p32).abs().max())}
    del plan, p32, ps
    # batched forward + adjoint, 256 Clements meshes m=16, n=8
    from perceval_gb300.components.mesh import clements_mesh_unitary
    ph = torch.from_numpy(np.random.default_rng(0).uniform(0, 2 * math.pi, (256, 240)))
    Um = clements_mesh_unitary(ph, 16).contiguous().to(dev)
    Ls = [math.comb(16 + k - 1, k) for k in range(9)]
    fb = 16 * 256 * sum(Ls[k - 1] + Ls[k] for k in range(1, 9))
    fterms = 256 * 16 * sum(Ls[k - 1] for k in range(1, 9))  # forward complex multiply-adds
    for prec, key in (("fp64", "slos_grad_m16_n8_b256"), ("float-float", "slos_grad_m16_n8_b256_float_float")):
        plan = _native.SlosPlan(16, [1] * 8 + [0] * 8, batch=256, keep_layers=True, precision=prec)
        w = torch.from_numpy(np.random.default_rng(1).normal(size=plan.count * 256)).to(dev)
        t_f = timed(lambda: plan.forward(Um), reps=2)
        t_b = timed(lambda: plan.backward(w), reps=2)
        row = {"arithmetic": prec, "forward_ms": t_f, "backward_ms": t_b,
               "circuits_per_s": 256 / ((t_f + t_b) * 1e-3), "forward_hbm_frac": fb / (t_f * 1e-3) / 1e9 / hbm}
        if prec == "fp64":
            row["forward_fp64_frac"] = fterms * 8 / (t_f * 1e-3) / (fp64_peak_tflops * 1e12)
        res[key] = row
        del plan
    torch.cuda.empty_cache()
    # single large permanents spread over the whole chip (Haar submatrices of a 1024x1024
    # unitary), Glynn and Ryser, with their relative difference
    Ubig = random_unitary(1024, seed=0)
    rng = np.random.default_rng(5)
    # n = 32 and 36 in both arithmetics (FP64 Ryser at 32 only: 3x Glynn's time); n = 40 in
    # float-float, its FP64 time extrapolated from n = 36 by the 2^(n-1) (8n - 4) flop count
    for n in (32, 36, 40):
        a = np.ascontiguousarray(Ubig[np.ix_(rng.choice(1024, n, False), rng.choice(1024, n, False))])
        ad = torch.from_numpy(a).to(dev)
        o = torch.empty(1, dtype=torch.complex128, device=dev)
        res_n = {}
        runs = [("glynn_fp64", 0, "fp64"), ("ryser_fp64", 1, "fp64"), ("glynn_ff", 0, "float-float"),
                ("ryser_ff", 1, "float-float")]
        if n == 36:
            runs = [r for r in runs if r[0] != "ryser_fp64"]
        if n == 40:
            runs = [("glynn_ff", 0, "float-float")]
        for name, method, prec in runs:
            s0, e0 = torch.cuda.Event(True), torch.cuda.Event(True)
            s0.record()
            _native.permanent_batch(ad, np.array([0]), np.array([n]), o, method, precision=prec)
            e0.record()
            e0.synchronize()
            v = complex(o.cpu().item())
            res_n[name] = [v.real, v.imag]
            res_n[f"{name}_ms"] = s0.elapsed_time(e0)
            res_n[f"{name}_tflops"] = glynn_flops(n) / (res_n[f"{name}_ms"] * 1e-3) / 1e12
        if "glynn_fp64" in res_n:
            ref = complex(*res_n["glynn_fp64"])
            for name in ("ryser_fp64", "glynn_ff", "ryser_ff"):
                if name in res_n:
                    res_n[f"{name}_rel_diff_vs_glynn_fp64"] = abs(complex(*res_n[name]) - ref) / abs(ref)
        res[f"perm_single_n{n}"] = res_n
    t36 = res["perm_single_n36"]["glynn_fp64_ms"]
    res["perm_single_n40"]["glynn_fp64_ms_extrapolated"] = t36 * glynn_flops(40) / glynn_flops(36)
    # Clifford & Clifford, n=20, m=400
    U4 = torch.from_numpy(random_unitary(400, seed=0)).to(dev)
    cnt = 100000  # the configuration's 1e5 samples
    t_cc = timed(lambda: _native.cc2017_sample(U4, [1] * 20 + [0] * 380, cnt, seed=1), reps=1)
    res["cc2017_n20_m400"] = {"samples_per_s": cnt / (t_cc * 1e-3), "samples": cnt, "precision": "float-float"}
    # the same in the FP64 mode (fixed-point column sums, block-floating products), 1e4 samples
    t_cc64 = timed(lambda: _native.cc2017_sample(U4, [1] * 20 + [0] * 380, 10000, seed=1, precision=2), reps=1)
    res["cc2017_n20_m400"]["fp64"] = {"samples_per_s": 10000 / (t_cc64 * 1e-3), "samples": 10000}
    # many input states (the per-input loop of a samples provider): 64 distinct 6-photon inputs
    # on m = 64, 1000 samples each, one wavefront against one call per input
    rng = np.random.default_rng(5)
    U64 = torch.from_numpy(random_unitary(64, seed=1)).to(dev)
    states = np.zeros((64, 64), dtype=np.int32)
    for b in range(64):
        states[b, rng.choice(64, 6, replace=False)] = 1
    per = [1000] * 64
    t_many = timed(lambda: _native.cc2017_sample_multi(U64, states, per, seed=3), reps=2)

    def loop():
        off = 0
        for b in range(64):
            _native.cc2017_sample(U64, states[b], per[b], seed=3, first_sample=off)
            off += per[b]
    t_loop = timed(loop, reps=2)
    res["cc2017_64_inputs_m64_n6"] = {"samples": 64000, "one_wavefront_ms": t_many, "per_input_loop_ms": t_loop,
                                      "samples_per_s": 64000 / (t_many * 1e-3)}
    # the learned-proposal sampler, bounded for the default run: n = 30, m = 900 trained on
    # 1024 exact samples (FP32 sampler), 8 chains x 16 steps of FP64-permanent acceptances
    # against 96 exact float-float samples and 32 exact FP64 samples; and the n = 8, m = 64
    # companion
    res["learned_mis_n30_m900"] = learned_case(torch, _native, random_unitary, 900, 30, 1024, 4, 8, 16, 96,
                                               tvd=False, n_ref64=32)
    # n = 8, m = 64 with enough samples of both samplers to resolve the marginals to 1e-3:
    # 2048 chains x 4096 steps (8.4 M proposals) and 4 M exact samples; and the exact TVD of
    # both samplers' empirical distributions
    res["learned_mis_n8_m64"] = learned_case(torch, _native, random_unitary, 64, 8, 20000, 10, 2048, 4096,
                                             4_000_000, mis_batch=16384, exact_tvd=True)
    # small case: SLOS m=12, n=6 and 1000 Naive amplitudes (latency-bound)
    from perceval_gb300 import BackendFactory, BasicState
    U12 = random_unitary(12, seed=0)

    def slos_call():
        b = BackendFactory.get_backend("SLOS")
        b.set_circuit(U12)
        b.set_input_state(BasicState([1] * 6 + [0] * 6))
        return b.all_prob()
    slos_call()  # loads the kernels once; each timed call is a fresh backend (plan, launches, copy)
    t0 = time.perf_counter()
    p = slos_call()
    t_slos = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    outs = []
    for _ in range(1000):
        o = np.zeros(12, dtype=int)
        o[rng.choice(12, 6, replace=False)] = 1
        outs.append(BasicState(o))
    nb = BackendFactory.get_backend("Naive")
    nb.set_circuit(U12)
    nb.set_input_state(BasicState([1] * 6 + [0] * 6))
    nb.prob_amplitudes(outs[:10])
    t0 = time.perf_counter()
    nb.prob_amplitudes(outs)
    t_naive = time.perf_counter() - t0
    res["small_m12_n6"] = {"slos_all_prob_ms": t_slos * 1e3, "outputs": len(p), "naive_1000_amplitudes_ms": t_naive * 1e3}
    # many input states of one circuit (the per-input loop of Simulator._probs_svd_fast):
    # 500 distinct 6-photon inputs on m = 12, one batched plan against one plan per input
    rng3 = np.random.default_rng(4)
    many = set()
    while len(many) < 500:
        st = np.zeros(12, dtype=int)
        np.add.at(st, rng3.integers(0, 12, 6), 1)
        many.add(tuple(int(v) for v in st))
    many = [BasicState(list(st)) for st in sorted(many)]
    bm = BackendFactory.get_backend("SLOS")
    bm.set_circuit(U12)
    bm.all_probs_many(many[:8])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pm = bm.all_probs_many(many)
    t_many = time.perf_counter() - t0
    bl = BackendFactory.get_backend("SLOS")
    bl.set_circuit(U12)
    t0 = time.perf_counter()
    dev_max = 0.0
    for st, pref in zip(many, pm):
        bl.set_input_state(st)
        dev_max = max(dev_max, float(np.abs(np.asarray(bl.all_prob()) - pref).max()))
    t_loop = time.perf_counter() - t0
    res["slos_500_inputs_m12_n6"] = {"batched_ms": t_many * 1e3, "per_input_loop_ms": t_loop * 1e3,
                                     "max_abs_diff": dev_max}
    # a noisy source through Simulator.probs_svd: |1,1,1,1,1,1,0,...> on m = 12, each photon
    # lost (0.1), indistinguishable (0.8) or distinguishable (0.1): 729 separable inputs,
    # distinct parts simulated in batched plans, against the same simulator taking one
    # plan per distinct part (the reference's loop)
    from perceval_gb300.simulators import Simulator

    noisy = {}
    for code in range(3 ** 6):
        p, same, parts, c = 1.0, [0] * 12, [], code
        for ph in range(6):
            kind, c = c % 3, c // 3
            p *= (0.1, 0.8, 0.1)[kind]
            if kind == 1:
                same[ph] = 1
            elif kind == 2:
                solo = [0] * 12
                solo[ph] = 1
                parts.append(BasicState(solo))
        noisy[tuple([BasicState(same)] + parts)] = p

    class _PerInput:
        """The SLOS backend without its batched entry point."""

        def __init__(self, be):
            self._be, self._masks_str = be, None

        def set_input_state(self, s):
            self._be.set_input_state(s)

        def prob_iterator(self, min_p):
            return self._be.prob_iterator(min_p)

        def prob_distribution(self):
            return self._be.prob_distribution()

    sim_b = Simulator(BackendFactory.get_backend("SLOS"))
    sim_b.set_circuit(U12)
    sim_b.probs_svd(dict(list(noisy.items())[:8]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out_b = sim_b.probs_svd(noisy)
    t_svd = time.perf_counter() - t0
    be_l = BackendFactory.get_backend("SLOS")
    be_l.set_circuit(U12)
    sim_l = Simulator(_PerInput(be_l))
    t0 = time.perf_counter()
    out_l = sim_l.probs_svd(noisy)
    t_svd_loop = time.perf_counter() - t0
    n_parts = len({s for key in noisy for s in key})
    res["probs_svd_noisy_m12_n6"] = {
        "inputs": len(noisy), "distinct_parts": n_parts, "outputs": len(out_b["results"]),
        "batched_ms": t_svd * 1e3, "per_part_loop_ms": t_svd_loop * 1e3,
        "max_abs_diff": max(abs(out_b["results"][k] - out_l["results"].get(k, 0.0)) for k in out_b["results"]),
        "logical_perf": out_b["logical_perf"]}
    # launch latency of a small batch (1000 permanents of 6x6 Haar submatrices): the
    # plan-free call against one graph launch of a plan, wall clock per call
    sub = np.stack([U12[np.ix_(rng.choice(12, 6, replace=False), rng.choice(12, 6, replace=False))]
                    for _ in range(1000)])
    sd = torch.from_numpy(sub.reshape(-1)).to(dev)
    so = torch.empty(1000, dtype=torch.complex128, device=dev)
    s_offs = np.arange(1000, dtype=np.int64) * 36
    s_sizes = np.full(1000, 6, dtype=np.int32)
    small_plan = _native.PermPlan(s_offs, s_sizes)

    def wall_us(fn, reps=200):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps * 1e6

    # Gurvits estimates (NaiveApprox): 1000 Haar submatrices n = 20, 10^4 draws each;
    # a draw is 2n^2 real FMAs of column sums plus n complex products (FP32)
    rng2 = np.random.default_rng(11)
    gm = np.stack([Ubig[np.ix_(rng2.choice(1024, 20, False), rng2.choice(1024, 20, False))] for _ in range(1000)])
    gd = torch.from_numpy(gm.reshape(-1)).to(dev)
    g_offs = np.arange(1000, dtype=np.int64) * 400
    g_sizes = np.full(1000, 20, dtype=np.int32)
    g_out = torch.empty(1000, dtype=torch.complex128, device=dev)
    g_err = torch.empty(1000, dtype=torch.float64, device=dev)
    g_iters = 10000
    t_g = timed(lambda: _native.permanent_estimate_batch(gd, g_offs, g_sizes, g_out, g_err, g_iters, 1, 0), reps=3)
    draws = 1000 * g_iters
    res["gurvits_1000x20_1e4"] = {"ms": t_g, "draws_per_s": draws / (t_g * 1e-3),
                                  "fp32_tflops": draws * (4 * 20 * 20 + 6 * 20) / (t_g * 1e-3) / 1e12,
                                  "median_err_bound": float(g_err.median())}
    res["perm_1000x6_latency"] = {"batch_call_us": wall_us(lambda: _native.permanent_batch(sd, s_offs, s_sizes, so)),
                                  "plan_graph_us": wall_us(lambda: small_plan(sd, so))}
    return res


def learned_case(torch, _native, random_unitary, m, n, n_train, epochs, chains, steps, n_ref, tvd=True,
                 marginal_modes=8, n_ref64=None, mis_batch=512, tvd_samples=25600, exact_tvd=False):
    """Learned-proposal Metropolised sampler against the plain GPU exact sampler on one
    Haar unitary (seed 0, input photons in modes 0..n-1).

    Training data: exact Clifford & Clifford samples from this library's sampler in its
    FP32 mode.  Acceptance ratios: exact FP64 permanents (permanent plans, FP64 arithmetic).
    ESS: Geyer's initial positive sequence on each chain's log pi trace, summed over
    chains; the exact sampler's samples are independent (ESS = N).  Marginals: the exact
    one-mode distributions P(n_i = a) of the most occupied modes and two-mode
    distributions P(n_i = a, n_j = b) of pairs among them (generating-function
    permanents, perceval_gb300.marginals) against each sampler's empirical ones, with
    the binomial standard error of the largest probability at that sample count (for the
    MIS, at its ESS).  With ``exact_tvd``: the exact TVD between each sampler's empirical
    output distribution and the exact law (every observed output's probability from an FP64
    permanent, the unobserved mass as one minus their sum), for the MIS's chain states and
    for the exact sampler at its full count and at the MIS's ESS."""
    from perceval_gb300.learned import (ProposalMLP, counts_to_sorted_modes, ess, exact_empirical_tvd,
                                        exact_moments, run_mis, tvd_estimate)
    from perceval_gb300.marginals import (empirical_one_mode, empirical_two_mode, one_mode_marginal,
                                          two_mode_marginal)
    U = random_unitary(m, seed=0)
    inp = [1] * n + [0] * (m - n)
    Ud = torch.from_numpy(U).cuda()
    A, E2 = exact_moments(U, inp)
    modes = [int(i) for i in np.argsort(-A)[:marginal_modes]]
    t0 = time.perf_counter()
    train = _native.cc2017_sample(Ud, inp, n_train, seed=101, precision=1).cpu().numpy()
    t_train_samples = time.perf_counter() - t0
    net = ProposalMLP(m, n, D=128, H=512, layers=3, seed=0)
    t0 = time.perf_counter()
    n_val = max(1, len(train) // 10)  # held-out tenth: early stopping on its NLL
    losses = net.train(train[n_val:], epochs=epochs, batch=256, lr=1e-3, val=train[:n_val])
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    res = run_mis(net, U, inp, chains=chains, steps=steps, seed=7, batch=mis_batch)
    ess_mis = float(sum(ess(x) for x in res.log_pi))
    seqs = res.sequences.reshape(-1, n)
    mis_occ = np.stack([(seqs == i).sum(axis=1) for i in modes], axis=1)
    mis_mean = np.bincount(seqs.reshape(-1).astype(np.int64), minlength=m)[:m] / len(seqs)

    ref_sorted = []

    def exact(count, seed, precision):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x = _native.cc2017_sample(Ud, inp, count, seed=seed, precision=precision)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if exact_tvd and not ref_sorted:
            ref_sorted.append(counts_to_sorted_modes(x, n).cpu().numpy())
        return dt, x[:, modes].cpu().numpy(), x.double().mean(0).cpu().numpy(), x[:tvd_samples].cpu().numpy()
    t_ref, ref_occ, ref_mean, ref_head = exact(n_ref, 202, 0)
    # the same sampler in its FP64 mode, the acceptance's arithmetic
    n_ref64 = n_ref if n_ref64 is None else n_ref64
    t_ref64, ref64_occ, ref64_mean, _ = exact(n_ref64, 303, 2)
    one = {i: one_mode_marginal(U, inp, i) for i in modes}
    pairs = [(a, b) for a in range(len(modes)) for b in range(a + 1, len(modes))][:12]
    two = {p: two_mode_marginal(U, inp, modes[p[0]], modes[p[1]]) for p in pairs}

    def marg_err(occ, eff=None):
        # occ: occupations of the selected modes (column k = mode modes[k])
        e1 = max(float(np.abs(empirical_one_mode(occ, k, n) - one[i]).max()) for k, i in enumerate(modes))
        e2 = max(float(np.abs(empirical_two_mode(occ, a, b, n) - two[(a, b)]).max()) for a, b in pairs)
        pmax = max(float(one[i].max()) for i in modes)
        neff = len(occ) if eff is None else eff
        return {"max_abs_err_one_mode": e1, "max_abs_err_two_mode": e2, "samples": int(len(occ)),
                "binomial_stderr_at_max_p": math.sqrt(pmax * (1 - pmax) / neff)}
    row = {"m": m, "n": n, "train_samples": n_train, "train_sampling_s": t_train_samples,
           "fit_s": t_fit, "nll_first_last": [losses[0], losses[-1]],
           "held_out_nll": net.val_nll, "kept_epoch": net.best_epoch,
           "mis": {"chains": chains, "steps": steps, "proposals": res.proposals, "seconds": res.seconds,
                   "acceptance_arithmetic": "fp64 permanents",
                   "accept_rate": res.accept_rate, "ess": ess_mis, "ess_per_s": ess_mis / res.seconds,
                   "max_abs_err_E_n": float(np.abs(mis_mean - A).max()),
                   "marginals": marg_err(mis_occ, ess_mis)},
           "exact_sampler": {"samples": n_ref, "seconds": t_ref, "ess_per_s": n_ref / t_ref,
                             "arithmetic": "float-float",
                             "max_abs_err_E_n": float(np.abs(ref_mean - A).max()),
                             "marginals": marg_err(ref_occ)},
           "exact_sampler_fp64": {"samples": n_ref64, "seconds": t_ref64, "ess_per_s": n_ref64 / t_ref64,
                                  "arithmetic": "fp64",
                                  "max_abs_err_E_n": float(np.abs(ref64_mean - A).max()),
                                  "marginals": marg_err(ref64_occ)},
           "marginal_modes": modes, "marginal_pairs": [[modes[a], modes[b]] for a, b in pairs]}
    row["ess_per_s_ratio"] = row["mis"]["ess_per_s"] / row["exact_sampler"]["ess_per_s"]
    row["ess_per_s_ratio_vs_fp64_exact"] = row["mis"]["ess_per_s"] / row["exact_sampler_fp64"]["ess_per_s"]
    if exact_tvd:
        n_ess = max(1, min(n_ref, int(round(ess_mis))))
        row["exact_tvd"] = {"mis": exact_empirical_tvd(U, inp, seqs),
                            "exact_sampler": exact_empirical_tvd(U, inp, ref_sorted[0]),
                            "exact_sampler_at_mis_ess": exact_empirical_tvd(U, inp, ref_sorted[0][:n_ess])}
    if tvd:
        # TVD(q, pi) on photon sequences from the exact samples: trained vs untrained network
        untrained = ProposalMLP(m, n, D=128, H=512, layers=3, seed=0)
        t, te = tvd_estimate(net, U, inp, ref_head, seed=5)
        u0, ue = tvd_estimate(untrained, U, inp, ref_head, seed=5)
        row["tvd_q_pi_sequences"] = {"samples": int(len(ref_head)), "trained": t, "trained_stderr": te,
                                     "untrained": u0, "untrained_stderr": ue}
    return row


def run_learned(args):
    """Learned-proposal Metropolised sampler vs the plain GPU exact sampler at
    n = 30, m = 900, plus the n = 8, m = 64 companion (``learned_case``), and the
    tensor-pipe rate of the network's GEMM kernel."""
    import torch
    from perceval_gb300 import _native
    from perceval_gb300.utils.matrix import random_unitary
    _native.load()
    out = {}
    for (m, n, n_train, epochs, chains, steps, n_ref) in ((900, 30, args.learned_train, 6, 16, 32, 152),
                                                           (64, 8, 20000, 10, 64, 400, 25600)):
        out[f"n{n}_m{m}"] = learned_case(torch, _native, random_unitary, m, n, n_train, epochs, chains, steps, n_ref,
                                         exact_tvd=(n == 8))
    # tensor-pipe rate of the network's GEMM kernel (pcvl_gemm_bf16: tcgen05 MMA from TMA-staged
    # tiles, FP32 accumulation in tensor memory) at the training shapes of n = 30, m = 900 (256 sequences x 30 steps)
    # and at 8192^3, against the measured cuBLAS BF16 burst peak
    try:
        peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"]
    except (OSError, ValueError, KeyError):
        peak = 1900.0
    gemm = {}
    for (M, N, K) in ((7680, 512, 512), (7680, 900, 512), (7680, 512, 128), (8192, 8192, 8192)):
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
        C = torch.empty(M, N, device="cuda", dtype=torch.float32)
        f = lambda: _native.gemm_bf16(A, B, M, N, K, K, K, C=C)
        f()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(5):
            s0, e0 = torch.cuda.Event(True), torch.cuda.Event(True)
            s0.record()
            f()
            e0.record()
            e0.synchronize()
            best = min(best, s0.elapsed_time(e0))
        tf = 2.0 * M * N * K / (best * 1e-3) / 1e12
        row = {"ms": best, "tflops": tf, "frac_of_bf16_peak": tf / peak,
               "timing": "one call between two events (includes the host's launch latency)"}
        # 20 back-to-back calls captured in one CUDA graph: the device time per call
        reps = 20 if M * N * K < 1 << 33 else 4
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(side):
            f()
            with torch.cuda.graph(graph, stream=side):
                for _ in range(reps):
                    f()
        torch.cuda.current_stream().wait_stream(side)
        graph.replay()
        torch.cuda.synchronize()
        gbest = float("inf")
        for _ in range(5):
            s0, e0 = torch.cuda.Event(True), torch.cuda.Event(True)
            s0.record()
            graph.replay()
            e0.record()
            e0.synchronize()
            gbest = min(gbest, s0.elapsed_time(e0) / reps)
        gtf = 2.0 * M * N * K / (gbest * 1e-3) / 1e12
        row.update({"graph_ms_per_call": gbest, "graph_tflops": gtf, "graph_frac_of_bf16_peak": gtf / peak,
                    "graph_calls": reps})
        del graph
        gemm[f"{M}x{N}x{K}"] = row
    print(json.dumps({"learned_proposal": out, "mlp_gemm": gemm, "bf16_peak_tflops": peak}), flush=True)


def run_large_perm(args):
    """One n = 40 Haar-submatrix permanent (Glynn, 1.74e14 FP64-equivalent flops), the
    largest single-permanent size of the benchmark configurations, in FP64 and in
    float-float (about three minutes together)."""
    import torch
    from perceval_gb300 import _native
    from perceval_gb300.utils.matrix import random_unitary
    _native.load()
    Ubig = random_unitary(1024, seed=0)
    rng = np.random.default_rng(40)
    n = 40
    a = np.ascontiguousarray(Ubig[np.ix_(rng.choice(1024, n, False), rng.choice(1024, n, False))])
    ad = torch.from_numpy(a).cuda()
    res = {}
    for prec in ("fp64", "float-float"):
        o = torch.empty(1, dtype=torch.complex128, device="cuda")
        s0, e0 = torch.cuda.Event(True), torch.cuda.Event(True)
        s0.record()
        _native.permanent_batch(ad, np.array([0]), np.array([n]), o, 0, precision=prec)
        e0.record()
        e0.synchronize()
        ms = s0.elapsed_time(e0)
        v = complex(o.cpu().item())
        res[prec] = {"glynn": [v.real, v.imag], "glynn_ms": ms,
                     "glynn_tflops_fp64_equiv": glynn_flops(n) / (ms * 1e-3) / 1e12}
    f, ff = complex(*res["fp64"]["glynn"]), complex(*res["float-float"]["glynn"])
    res["float_float_rel_diff_vs_fp64"] = abs(ff - f) / abs(f)
    print(json.dumps({"perm_single_n40": res}), flush=True)


def profile_case(name: str):
    """One untimed run of a single hot kernel on a small case, for ncu captures."""
    import torch
    from perceval_gb300 import _native, autotune
    from perceval_gb300.utils.matrix import random_unitary
    _native.load()
    autotune.load()  # the launch shapes the headline run tuned and cached, if any
    dev = torch.device("cuda")
    if name in ("perm24", "perm24dadd", "perm24ff"):
        # 64 matrices of the n = 24 bin (one perm_bin_fx<24>, perm_bin_f64<24> or
        # perm_bin_kernel<24> launch)
        mats, flat, offs, sizes = make_batch(seed=0)
        sel = [i for i in range(N_MATS) if sizes[i] == 24][:64]
        sub = torch.from_numpy(np.concatenate([mats[i].reshape(-1) for i in sel])).to(dev)
        out = torch.empty(len(sel), dtype=torch.complex128, device=dev)
        _native.permanent_batch(sub, np.arange(len(sel), dtype=np.int64) * 576, np.full(len(sel), 24, np.int32), out,
                                precision={"perm24": "fp64", "perm24dadd": "fp64-dadd"}.get(name, "float-float"))
    elif name in ("slos20", "slos20ff"):
        # SLOS m = 20, n = 10: last layer 20,030,010 states (320 MB, above L2)
        plan = _native.SlosPlan(20, [1] * 10 + [0] * 10, precision="fp64" if name == "slos20" else "float-float")
        plan.forward(torch.from_numpy(random_unitary(20, seed=0)).to(dev))
        plan.probabilities()
    elif name == "slos20p":
        # SLOS m = 20, n = 10, every probability with the last layer writing them directly
        plan = _native.SlosPlan(20, [1] * 10 + [0] * 10)
        plan.forward_probabilities(torch.from_numpy(random_unitary(20, seed=0)).to(dev))
    elif name == "slosmask22":
        # heralded SLOS m = 22, n = 11 (modes 18..21 detected as 1, 1, 0, 0): the largest kept
        # layer (k = 10) holds 7,330,675 states, 117 MB of amplitudes plus 0.3 GB of parent
        # tables (above L2); about 1 GB on the device
        from perceval_gb300.utils import FSMask
        plan = _native.SlosPlan(22, [1] * 11 + [0] * 11, mask=FSMask(22, 11, ["*" * 18 + "1100"]))
        plan.forward(torch.from_numpy(random_unitary(22, seed=0)).to(dev))
        plan.probabilities()
    elif name == "slap1024":
        # SLAP m = 1024, n = 3: 179,481,600 outputs (1.4 GB of probabilities), one slap_walk launch
        inp = [1] * 3 + [0] * 1021
        _native.slap_all(torch.from_numpy(random_unitary(1024, seed=0)).to(dev), inp)
    elif name == "slos16b256":
        from perceval_gb300.components.mesh import clements_mesh_unitary
        ph = torch.from_numpy(np.random.default_rng(0).uniform(0, 2 * math.pi, (256, 240)))
        plan = _native.SlosPlan(16, [1] * 8 + [0] * 8, batch=256, keep_layers=True)
        plan.forward(clements_mesh_unitary(ph, 16).contiguous().to(dev))
        plan.backward(torch.ones(plan.count * 256, dtype=torch.float64, device=dev))
    elif name == "gurvits20":
        U = random_unitary(1024, seed=0)
        rng = np.random.default_rng(11)
        gm = np.stack([U[np.ix_(rng.choice(1024, 20, False), rng.choice(1024, 20, False))] for _ in range(1000)])
        out = torch.empty(1000, dtype=torch.complex128, device=dev)
        err = torch.empty(1000, dtype=torch.float64, device=dev)
        _native.permanent_estimate_batch(torch.from_numpy(gm.reshape(-1)).to(dev), np.arange(1000) * 400,
                                         np.full(1000, 20), out, err, 10000, 1, 0)
    elif name == "gemm":
        M, N, K = 7680, 512, 512
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
        C = torch.empty(M, N, device="cuda", dtype=torch.float32)
        _native.gemm_bf16(A, B, M, N, K, K, K, C=C)
    elif name in ("cc2017", "cc2017fp64"):
        # n = 20 photons on m = 400, 608 samples (float-float, or the FP64 mode)
        U4 = torch.from_numpy(random_unitary(400, seed=0)).to(dev)
        _native.cc2017_sample(U4, [1] * 20 + [0] * 380, 608, seed=1, precision=2 if name == "cc2017fp64" else 0)
    else:
        raise SystemExit(f"unknown profile case {name}")
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-secondary", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--learned", action="store_true",
                    help="run the learned-proposal sampler workload (n=30, m=900 and n=8, m=64) and exit")
    ap.add_argument("--learned-train", type=int, default=2048, help="exact training samples at n=30")
    ap.add_argument("--large-perm", action="store_true",
                    help="one n = 40 permanent in FP64 and in float-float (about three minutes)")
    ap.add_argument("--profile-case", choices=["perm24", "perm24dadd", "perm24ff", "slos20", "slos20ff", "slos20p", "slosmask22", "slap1024", "slos16b256",
                                               "cc2017", "cc2017fp64", "gurvits20", "gemm"],
                    help="run one small untimed case of a single kernel (for ncu) and exit")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
    elif args.learned:
        run_learned(args)
    elif args.large_perm:
        run_large_perm(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
