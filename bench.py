#!/usr/bin/env python3
"""Benchmark of the trial-factoring hot path on GB300.

Workload (the metric's plain single-job configuration): Proth k=3,
S(n) = 3*2^n + 1 for n = 1..100000, trial-factored by every prime in
[2^32, 2^34) produced by the device sieve.  One step = one 2^30-wide prime
segment: device sieve -> primes in HBM -> residue kernel; the 12 segments of
[2^32, 2^34) are the steps (the default --steps 12 covers the range once).
Unit of work: one (n, p) residue update; value = updates / s.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line (rank 0).  `--impl reference` times the reference
algorithm on the host cores instead (the CPU oracle, a restatement of the
reference's CPU engine): each step is a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FAMILY, PARAM, N0, N1 = 1, 3, 1, 100001          # proth, k = 3, n in [1, 100001)
F0, F1 = 1 << 32, 1 << 34
SEG = 1 << 30
NSEG = (F1 - F0) // SEG
MAXF = 32
# algorithmic 32-bit integer operations per update of the doubling
# recurrence u <- 2u mod p on 64-bit words: 2 (2u - p, add with carry),
# 1 (sign test), 2 (conditional add of p), 1 (zero test of the residue)
OPS_PER_UPDATE = 6
# DRAM bytes per prime of residue_kernel<PROTH> from one ncu capture on
# [2^32, 2^32 + 2^27): 48,436,480 + 1,024 bytes for 6,047,768 primes; traffic
# grows with the prime count (each prime is read once), so a full launch's
# traffic is this figure times its primes
DRAM_BYTES_PER_PRIME = (48436480 + 1024) / 6047768
METRIC = "prime*term residue updates/s"
WORKLOAD = ("Proth k=3: 3*2^n+1 for n=1..100000 by residue doubling, all primes in [2^32, 2^34) from the "
            "device sieve; single job, plain kernel")


def mv_bound(y: int) -> int:
    """Montgomery-Vaughan bound on the primes in an interval of length y."""
    return int(2 * y / math.log(y)) + 64


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


def int_peak(device: int):
    """Integer ALU instructions/s from libctd_probe.so (measured on this GPU now)."""
    from cutrialdive_gb300._build import PROBE

    if not os.path.exists(PROBE):
        return None
    L = ctypes.CDLL(PROBE)
    L.ctd_probe_int_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    best = 0.0
    for _ in range(3):
        v, s = ctypes.c_double(), ctypes.c_double()
        if L.ctd_probe_int_peak(device, ctypes.byref(v), ctypes.byref(s)) == 0:
            best = max(best, v.value)
    return best or None


# ---------------------------------------------------------------- CPU legs
def cpu_updates_per_s(n_primes_target_s: float, threads: int, lo: int):
    """Times the CPU oracle's residue loop (the reference CPU engine's
    process_chunk, restated) on a prime sample starting at `lo` sized for
    about `n_primes_target_s` seconds.  Returns (updates/s, sample text)."""
    import oracle

    N = N1 - N0
    # calibrate on a small slice
    width = 1 << 18
    primes = oracle.sieve(lo, lo + width)
    t = time.perf_counter()
    oracle.residue_hits(FAMILY, PARAM, N0, N1, primes, MAXF, threads=threads)
    dt = max(time.perf_counter() - t, 1e-3)
    rate = primes.size * N / dt
    want = n_primes_target_s * rate / N  # primes
    width = max(width, int(width * want / max(primes.size, 1)))
    primes = oracle.sieve(lo, lo + width)
    t = time.perf_counter()
    oracle.residue_hits(FAMILY, PARAM, N0, N1, primes, MAXF, threads=threads)
    dt = time.perf_counter() - t
    return primes.size * N / dt, primes.size * N, dt, f"primes in [{lo}, {lo + width}) ({primes.size}), n in [1, 100001)"


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    import oracle  # noqa: F401  (fails loudly if missing)

    per_step_s = 2.0
    total_updates, total_t, samples = 0, 0.0, []
    for i in range(args.warmup + args.steps):
        lo = F0 + (i % NSEG) * SEG
        rate, updates, dt, sample = cpu_updates_per_s(per_step_s, threads, lo)
        if i >= args.warmup:
            total_updates += updates
            total_t += dt
            samples.append(sample)
    value = total_updates / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (deterministic: the configuration has no random input)",
        "config": {"workload": WORKLOAD, "step": "a bounded sample of one 2^30 prime segment (about 2 s of CPU)"},
        "cpu_baseline": {"value": value, "unit": "updates/s", "cores": threads, "kind": "port",
                         "sample": samples[0] if samples else ""},
        "e2e": {"value": value, "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference CPU engine (src/trial_factoring_impl.hpp:193-366) as restated by the oracle; "
                 "the reference's own build (oracle/_ref) is x86-only and does not travel to this host"),
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU leg
def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    import cutrialdive_gb300 as ctd
    from cutrialdive_gb300 import _native as NAT

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = NAT.load()
    eng = ctd.Engine(local)
    info = eng.device_info()
    stream = torch.cuda.Stream(device=local)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    N = N1 - N0
    cap = mv_bound(SEG)
    primes = torch.empty(cap, dtype=torch.int64, device="cuda")
    counts = torch.zeros(N, dtype=torch.int32, device="cuda")
    factors = torch.zeros(N * MAXF, dtype=torch.int64, device="cuda")
    job = NAT.CtdJob(FAMILY, MAXF, PARAM, N0, N1, F0, F1)
    count = ctypes.c_uint64()

    def seg_of(j):
        return (rank * args.steps + j) % NSEG

    def step(j, ev=None):
        fx = F0 + seg_of(j) * SEG
        with torch.cuda.stream(stream):
            if ev is not None:
                ev[0].record(stream)
            rc = L.ctd_sieve_device(eng.handle, fx, fx + SEG, ctypes.c_void_p(primes.data_ptr()), cap,
                                    ctypes.byref(count), sptr)
            if rc:
                raise NAT.CtdError(rc, L.ctd_last_error(eng.handle).decode())
            if ev is not None:
                ev[1].record(stream)
            rc = L.ctd_residues_device(eng.handle, ctypes.byref(job), ctypes.c_void_p(primes.data_ptr()), count.value,
                                       ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(factors.data_ptr()), sptr)
            if rc:
                raise NAT.CtdError(rc, L.ctd_last_error(eng.handle).decode())
            if ev is not None:
                ev[2].record(stream)
        return count.value

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for j in range(args.warmup):
        step(j)
    torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    launches0 = L.ctd_kernel_launches()
    barrier()
    torch.cuda.synchronize()
    nprimes = []
    with ClockSampler(local) as clocks:
        t_start.record(stream)
        for j in range(args.steps):
            nprimes.append(step(j, evs[j]))
        t_end.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = L.ctd_kernel_launches() - launches0
    elapsed = t_start.elapsed_time(t_end) * 1e-3
    sieve_ms = [e[0].elapsed_time(e[1]) for e in evs]
    resid_ms = [e[1].elapsed_time(e[2]) for e in evs]
    updates = sum(nprimes) * N
    if world > 1:
        t = torch.tensor([elapsed, float(updates)], dtype=torch.float64, device="cuda")
        tmax = t.clone()
        torch.distributed.all_reduce(tmax[:1], op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
        elapsed, total_updates = float(tmax[0]), float(t[1])
    else:
        total_updates = float(updates)
    value = total_updates / elapsed

    # ---- end to end: the C-ABI plain call with host buffers, copies inside
    e2e = None
    if not args.no_e2e:
        hc = torch.zeros(N, dtype=torch.int32).pin_memory()
        hf = torch.zeros(N * MAXF, dtype=torch.int64).pin_memory()
        buf = ctd.factors_buffer(N0, MAXF, hc.numpy().view(np.uint32), hf.numpy().view(np.uint64))
        e2e_updates = 0
        for j in range(min(args.warmup, 1)):
            fx = F0 + seg_of(j) * SEG
            eng.run_plain(NAT.CtdJob(FAMILY, MAXF, PARAM, N0, N1, fx, fx + SEG), buf, segment_length=SEG)
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in range(args.steps):
            fx = F0 + seg_of(j) * SEG
            eng.run_plain(NAT.CtdJob(FAMILY, MAXF, PARAM, N0, N1, fx, fx + SEG), buf, segment_length=SEG)
            e2e_updates += nprimes[j] * N
        torch.cuda.synchronize()
        e2e_t = time.perf_counter() - t0
        barrier()
        e2e_total = float(e2e_updates)
        if world > 1:
            t = torch.tensor([e2e_t, e2e_total], dtype=torch.float64, device="cuda")
            tmax = t.clone()
            torch.distributed.all_reduce(tmax[:1], op=torch.distributed.ReduceOp.MAX)
            torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
            e2e_t, e2e_total = float(tmax[0]), float(t[1])
        e2e = {"value": e2e_total / e2e_t, "unit": "updates/s", "h2d_bytes_per_step": N * 4 + N * MAXF * 8,
               "d2h_bytes_per_step": N * 4 + N * MAXF * 8,
               "api": "ctd_run_plain (include/ctd_gpu.h) with pinned host factors buffers, one segment per call"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    peak_int = int_peak(local)
    res_avg_s = statistics.mean(resid_ms) * 1e-3
    per_launch_updates = statistics.mean(nprimes) * N
    achieved = per_launch_updates * OPS_PER_UPDATE / res_avg_s
    roofline = {
        "bound": "int_alu", "kernel": "residue_kernel<PROTH>",
        "achieved": achieved / 1e9, "peak": (peak_int / 1e9) if peak_int else None, "unit": "Gop/s",
        "frac": (achieved / peak_int) if peak_int else None,
        "traffic": DRAM_BYTES_PER_PRIME * statistics.mean(nprimes),
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 2^27-segment launch, "
                          "scaled by primes per launch (profiles/residue_kernel_proth_k3_seg2p27_full.md)",
        "algorithmic_bytes": 8 * statistics.mean(nprimes),
        "ops_per_update": OPS_PER_UPDATE, "launch_ms": statistics.mean(resid_ms),
        "peak_source": "measured now: libctd_probe 32-bit add/xor chains (integer ALU issue rate) on this GPU",
    }
    sieve_s = statistics.mean(sieve_ms) * 1e-3
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    sieve_bytes = statistics.mean(nprimes) * 8
    sieve = {"kernel": "device sieve (sieve_windows + scan_counts + compact_windows, host count readback)",
             "ms_per_step": statistics.mean(sieve_ms), "primes_per_step": statistics.mean(nprimes),
             "achieved_gbs": sieve_bytes / sieve_s / 1e9, "peak_gbs": hbm,
             "frac": (sieve_bytes / sieve_s / 1e9 / hbm) if hbm else None,
             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm else "absent"}
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, _, dt, sample = cpu_updates_per_s(15.0, threads, F0)
        cpu = {"value": rate, "unit": "updates/s", "cores": threads, "kind": "port", "sample": sample,
               "seconds": dt}
    line = {
        "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (deterministic: the configuration has no random input)",
        "config": {"workload": WORKLOAD, "step": "one 2^30-wide prime segment: device sieve + residue kernel",
                   "segments": NSEG, "max_factors_per_number": MAXF,
                   "l2": "inputs larger than L2 (about 370 MB of primes per step)",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU", "device": info["name"]},
        "roofline": roofline, "sieve": sieve, "cpu_baseline": cpu, "e2e": e2e,
        "clocks": clocks.summary(), "gpu_launches": int(launches),
        "updates": total_updates, "seconds": elapsed,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ------------------------------------------------- batched / served workloads
BATCHED_WORKLOAD = ("Batched: 64 heterogeneous jobs drawn from seed 1234 (families uniform over smarandache b 2..16, "
                    "riesel k odd in [3, 10^6], proth_fixed_n n in [1000, 20000], mersenne; index ranges log-uniform "
                    "in [100, 20000] starting in [1, 50000]; TF range [2^a, 2^(a+2)), a in 30..38)")


def same_results(a, b) -> bool:
    """Equal counts, and equal sorted factor lists wherever no term overflowed
    its slots (which primes an overflowing term keeps depends on arrival order)."""
    import numpy as np

    if not np.array_equal(a.counts, b.counts):
        return False
    m = a.max_factors_per_number
    ra, rb = a.to_factoring_results(), b.to_factoring_results()
    return all(ra[i] == rb[i] for i in range(len(ra)) if a.counts[i] <= m)


def job_updates(eng, jobs) -> int:
    """Exact residue updates of a job list: primes in [f0, f1) x terms."""
    total = 0
    for j in jobs:
        total += eng.prime_count(j.f0, j.f1) * (j.n1 - j.n0)
    return total


def run_batched(args, world, rank, local):
    import torch

    import cutrialdive_gb300 as ctd
    from cutrialdive_gb300 import _native as NAT
    from cutrialdive_gb300 import jobs as J

    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    L = NAT.load()
    eng = ctd.Engine(local)
    mix = J.batched_mix()
    jobs = [j.ctd(MAXF, args.shrink) for j in mix]
    updates = job_updates(eng, jobs)

    def bufs():
        return [ctd.factors_buffer.empty(j.n0, j.n1 - j.n0, MAXF) for j in jobs]

    def batched_pass():
        b = bufs()
        eng.batch_run(jobs, b, segment_length=1 << 30, use_graph=True)
        return b

    def sequential_pass():
        b = bufs()
        for j, x in zip(jobs, b):
            eng.run_plain(j, x)
        return b

    for _ in range(args.warmup):
        out_b = batched_pass()
    l0 = L.ctd_kernel_launches()
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out_b = batched_pass()
        torch.cuda.synchronize()
        tb = (time.perf_counter() - t0) / args.steps
    launches = (L.ctd_kernel_launches() - l0) // args.steps
    out_s = sequential_pass()  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq_steps = max(1, min(args.steps, 2))
    for _ in range(seq_steps):
        out_s = sequential_pass()
    torch.cuda.synchronize()
    ts = (time.perf_counter() - t0) / seq_steps
    identical = all(same_results(a, b) for a, b in zip(out_b, out_s))
    h2d = sum((j.n1 - j.n0) * (4 + 8 * MAXF) for j in jobs)
    line = {
        "metric": METRIC, "value": updates / tb, "unit": "updates/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tb, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded job mix, seed 1234)",
        "config": {"workload": BATCHED_WORKLOAD,
                   "sample": f"each job's TF range cut to its first 1/{args.shrink}: [2^a, 2^a + 3*2^a/{args.shrink})",
                   "step": "one ctd_batch_run over all 64 jobs (aligned 2^30 segments, one CUDA graph)",
                   "l2": "prime lists of a segment (up to about 400 MB) exceed L2"},
        "updates_per_step": updates,
        "sequential": {"value": updates / ts, "ms_per_step": 1e3 * ts, "steps": seq_steps,
                       "api": "ctd_run_plain per job, default 2^26 segments, same host buffers"},
        "batched_over_sequential": ts / tb, "identical_outputs": identical,
        "e2e": {"value": updates / tb, "unit": "updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                "api": "ctd_batch_run with host factors buffers (copies inside the call)"},
        "clocks": clocks.summary(), "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)
    return 0 if identical else 1


def run_served(args, world, rank, local):
    import numpy as np
    import torch

    import cutrialdive_gb300 as ctd
    from cutrialdive_gb300 import _native as NAT
    from cutrialdive_gb300 import jobs as J

    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    L = NAT.load()
    eng = ctd.Engine(local)
    rates = [float(r) for r in args.rates.split(",")]
    sweep = []
    l0 = L.ctd_kernel_launches()
    with ClockSampler(local) as clocks:
        for rate in rates:
            mix, arrivals = J.served_mix(rate)
            count = min(len(mix), max(1, int(rate * args.window)))
            jobs = [j.ctd(MAXF, args.shrink) for j in mix[:count]]
            arrivals = arrivals[:count]
            updates = job_updates(eng, jobs)
            srv = ctd.Server(eng, memory_budget=160 << 30, max_active=256, segment_length=1 << 30)
            lat, ids, i = [], {}, 0
            t0 = time.perf_counter()
            while len(lat) < count:
                now = time.perf_counter() - t0
                while i < count and arrivals[i] <= now:
                    ids[srv.submit(jobs[i])] = i
                    i += 1
                st = srv.status()
                if st["active"] or st["queued"]:
                    for jid in srv.tick():
                        srv.fetch(jid)
                        lat.append(time.perf_counter() - t0 - arrivals[ids.pop(jid)])
                elif i < count:
                    time.sleep(max(0.0, min(arrivals[i] - now, 0.05)))
            span = time.perf_counter() - t0
            srv.close()
            sweep.append({"rate_jobs_s": rate, "jobs": count, "p50_s": float(np.percentile(lat, 50)),
                          "p99_s": float(np.percentile(lat, 99)), "updates": updates,
                          "updates_per_s": updates / span, "seconds": span})
    launches = L.ctd_kernel_launches() - l0
    best = max(sweep, key=lambda r: r["updates_per_s"])
    line = {
        "metric": METRIC + "; p50/p99 job latency", "value": best["updates_per_s"], "unit": "updates/s",
        "n_gpus": 1, "steps": len(rates), "warmup": 0, "ms_per_step": 1e3 * best["seconds"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (Poisson arrivals of the seeded job mix, seed 99)",
        "config": {"workload": "Serving: Poisson arrival stream from the batched distribution (seed 99), "
                               "admission by a 160 GB HBM budget",
                   "sample": f"each job's TF range cut to its first 1/{args.shrink}; at each rate the jobs "
                             f"arriving in the first {args.window:g} s (at most 2000)",
                   "server": "ctd_serve_* with max_active 256, 2^30 segments per tick"},
        "sweep": sweep, "clocks": clocks.summary(), "gpu_launches": int(launches),
        "e2e": {"value": best["updates_per_s"], "unit": "updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0, "api": "ctd_serve_submit/tick/fetch (host buffers)"},
    }
    print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    global SEG, NSEG
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=NSEG, help="steps (default: every 2^30 segment once)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--segment-bits", type=int, default=30,
                    help="log2 of the prime-segment width of one step (profiling uses smaller cases)")
    ap.add_argument("--workload", choices=["proth", "batched", "served"], default="proth",
                    help="proth: the plain single-job line (default); batched: the 64-job mix through "
                         "ctd_batch_run against the same jobs one by one; served: the Poisson serving sweep")
    ap.add_argument("--shrink", type=int, default=256, help="batched/served: keep the first 1/shrink of each TF range")
    ap.add_argument("--rates", default="1,5,10,25,50", help="served: arrival rates in jobs/s")
    ap.add_argument("--window", type=float, default=10.0, help="served: seconds of arrivals per rate")
    args = ap.parse_args()
    SEG = 1 << args.segment_bits
    NSEG = (F1 - F0) // SEG
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.workload == "batched":
        return run_batched(args, world, rank, local)
    if args.workload == "served":
        return run_served(args, world, rank, local)
    return run_ours(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
