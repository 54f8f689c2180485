#!/usr/bin/env python3
"""Benchmark of the trial-factoring hot path on GB300.

Default line (the metric's plain single-job configuration): Proth k=3,
S(n) = 3*2^n + 1 for n = 1..100000, trial-factored by every prime in
[2^32, 2^34) produced by the device sieve.  One step = one 2^30-wide prime
segment: device sieve -> primes in HBM -> residue launches; the default 12
steps cover the range once.  Unit of work: one (n, p) residue update;
value = updates / s.  The same line carries two more measurements of the
metric ("batched vs plain; p50/p99 job latency"):
  * "batched": the 64-job mix (seed 1234), each job's TF range cut to its
    first 1/64, through one ctd_batch_run against the same jobs one by one
    through ctd_run_plain, both on 2^30 segments; outputs checked against
    each other and against the reference engine's factor files;
  * "served": Poisson arrivals of the serving stream (seed 99) at two
    rates through ctd_serve_*, p50/p99 completion latency and updates/s.

Other workloads (--workload): `linear` (Fibonacci, Lucas and tribonacci,
n = 1..50000, primes in [2^34, 2^36)), `smarandache` (base 10, n = 10..1000,
all primes below 2^28), `batched` and `served` alone.

  python bench.py [--gpus N --steps K --warmup W] [--workload W] [--impl reference]

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

MAXF = 32
METRIC = "prime*term residue updates/s"


class Plain:
    """A plain-kernel workload: jobs (family, param, n0, n1) trial-factored
    by every prime of [f0, f1), walked in segments of 2^seg_bits; one step =
    one segment for every job (device sieve once, one residue launch per job)."""

    def __init__(self, name, jobs, f0, f1, seg_bits, text, steps):
        self.name, self.jobs, self.f0, self.f1, self.seg_bits = name, jobs, f0, f1, seg_bits
        self.text, self.default_steps = text, steps

    @property
    def seg(self) -> int:
        return 1 << self.seg_bits

    @property
    def nseg(self) -> int:
        return max(1, -(-(self.f1 - self.f0) // self.seg))

    def segment(self, j: int) -> tuple[int, int]:
        fx = self.f0 + (j % self.nseg) * self.seg
        return fx, min(fx + self.seg, self.f1)


PLAIN = {
    "proth": Plain("proth", [(1, 3, 1, 100001)], 1 << 32, 1 << 34, 30,
                   "Proth k=3: 3*2^n+1 for n=1..100000, all primes in [2^32, 2^34) from the device sieve; "
                   "single job, plain kernel", 12),
    "linear": Plain("linear", [(4, 0, 1, 50001), (5, 0, 1, 50001), (8, 0, 1, 50001)], 1 << 34, 1 << 36, 30,
                    "Linear recurrences: Fibonacci, Lucas and tribonacci for n=1..50000, primes in [2^34, 2^36); "
                    "three jobs back to back through the plain kernel", 3),
    "smarandache": Plain("smarandache", [(3, 10, 10, 1001)], 2, 1 << 28, 28,
                         "Plain Smarandache base 10, Sm(n) for n=10..1000, trial-factored by all primes in "
                         "[2, 2^28)", 12),
}
FAMILY_NAMES = {0: "MERSENNE", 1: "PROTH", 2: "RIESEL", 3: "SMARANDACHE", 4: "FIBONACCI", 5: "LUCAS",
                6: "PROTH_FIXED_N", 7: "RIESEL_FIXED_N", 8: "TRIBONACCI"}
# Roofline inputs per workload (what the dominant launch executes):
#  * proth -- the classified doubling launch (screen_kernel, classify_kernel
#    once per divisibility pattern, refine_kernel, nine_kernel,
#    regroup_kernel, class_walk_kernel): bound by integer issue slots.
#    Thread instructions and DRAM bytes per prime come from one ncu capture
#    of the same 13 launches on the 2^27-wide segment
#    [2^32, 2^32 + 2^27) of this workload
#    (6,047,768 primes; the capture's command is in the profile summary);
#    the live launch time comes from CUDA events in this run.
#  * smarandache -- the 32-bit Shoup step (p < 2^30): three 32-bit
#    multiplies per update (the quotient's high half, x M and q p), against
#    the integer multiply-add rate measured now;
#  * linear -- the dominant tribonacci launch: lazily reduced blocks of 18
#    steps, a three-input 64-bit add (2) and the compare (1) per step plus 3
#    shifts per block = 57/18 ALU operations per update, against the ALU
#    compare rate measured now.
PROTH_NCU = {"primes": 6047768,
             # warp instructions x active lanes per instruction, one entry per launch
             "thread_inst": {
                 "screen_kernel": 65171117 * 29.81,
                 "classify_kernel_p0": 132079999 * 29.59,
                 "classify_kernel_p1": 296012527 * 28.57,
                 "classify_kernel_p2": 50881891 * 29.24,
                 "classify_kernel_p3": 113313117 * 27.48,
                 "classify_kernel_p4": 32032031 * 29.39,
                 "classify_kernel_p5": 70274163 * 27.39,
                 "classify_kernel_p6": 12315032 * 28.47,
                 "classify_kernel_p7": 27235315 * 26.17,
                 "refine_kernel": 289309073 * 26.81,
                 "nine_kernel": 85534542 * 28.53,
                 "regroup_kernel": 56933014 * 15.98,
                 "class_walk_kernel": 1766393743 * 29.29},
             # dram__bytes_read.sum + dram__bytes_write.sum of the same launches, MB
             "dram_bytes": (62.006784 + 14.746624 + 55.477248 + 5.529600 + 64.505856 + 8.557056 + 31.603712 +
                            1.104896 + 47.789312 + 3.366144 + 21.782528 + 0.321280 + 36.367616 + 1.626624 + 8.100096
                            + 0.015616 + 15.639552 + 0.112640 + 83.481600 + 1.313792 + 68.398080 + 0.144128 +
                            73.165568 + 8.725248 + 53.848832 + 5.083648) * 1e6}
SMARANDACHE_MULS_PER_UPDATE = 3
TRIBONACCI_ALU_OPS_PER_UPDATE = 57 / 18


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


# ---------------------------------------------------------------- CPU legs
def cpu_updates_per_s(wl: Plain, target_s: float, threads: int, lo: int):
    """Times the CPU oracle's residue loop (the reference CPU engine's
    process_chunk, restated) over every job of the workload on a prime sample
    starting at `lo`, sized for about `target_s` seconds.
    Returns (updates/s, updates, seconds, sample text)."""
    import oracle

    lo = max(lo, 3)
    terms = sum(n1 - n0 for _, _, n0, n1 in wl.jobs)

    def run(primes):
        t = time.perf_counter()
        for fam, param, n0, n1 in wl.jobs:
            oracle.residue_hits(fam, param, n0, n1, primes, MAXF, threads=threads)
        return time.perf_counter() - t

    width = 1 << 16
    primes = oracle.sieve(lo, lo + width)
    dt = max(run(primes), 1e-3)
    want = target_s * (primes.size / dt)  # primes
    width = max(width, int(width * want / max(primes.size, 1)))
    primes = oracle.sieve(lo, lo + width)
    dt = run(primes)
    jobs = ", ".join(f"{FAMILY_NAMES[f].lower()} n in [{a}, {b})" for f, _, a, b in wl.jobs)
    return (primes.size * terms / dt, primes.size * terms, dt,
            f"primes in [{lo}, {lo + width}) ({primes.size}) x ({jobs})")


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    wl = PLAIN[args.workload] if args.workload in PLAIN else PLAIN["proth"]
    threads = os.cpu_count() or 1
    import oracle  # noqa: F401  (fails loudly if missing)

    per_step_s = args.cpu_seconds
    total_updates, total_t, samples = 0, 0.0, []
    for i in range(args.warmup + args.steps):
        lo, _ = wl.segment(i)
        rate, updates, dt, sample = cpu_updates_per_s(wl, per_step_s, threads, lo)
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
        "config": {"workload": wl.text,
                   "step": f"a bounded sample (about {per_step_s:g} s of CPU) of one 2^{wl.seg_bits} prime segment"},
        "cpu_baseline": {"value": value, "unit": "updates/s", "cores": threads, "kind": "port",
                         "sample": samples[0] if samples else ""},
        "e2e": {"value": value, "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference CPU engine (src/trial_factoring_impl.hpp:193-366) as restated by the oracle, all host "
                 "threads; the reference's own build (oracle/_ref) is x86-only and does not travel to this host"),
    }
    print(json.dumps(line), flush=True)
    return 0


def probe_peaks(device: int) -> dict:
    """Integer roofline denominators measured now by libctd_probe.so: the
    ALU-pipe compare rate, the mixed add/xor integer issue rate and the
    32-bit multiply-add rate."""
    from cutrialdive_gb300._build import PROBE

    out = {"alu": None, "int": None, "imad": None}
    if not os.path.exists(PROBE):
        return out
    L = ctypes.CDLL(PROBE)
    for key, fn in (("alu", "ctd_probe_alu_peak"), ("int", "ctd_probe_int_peak"), ("imad", "ctd_probe_imad_peak")):
        f = getattr(L, fn, None)
        if f is None:
            continue
        f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        best = 0.0
        for _ in range(3):
            v, s = ctypes.c_double(), ctypes.c_double()
            if f(device, ctypes.byref(v), ctypes.byref(s)) == 0:
                best = max(best, v.value)
        out[key] = best or None
    return out


# --------------------------------------------------------------- GPU leg
def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    import cutrialdive_gb300 as ctd
    from cutrialdive_gb300 import _native as NAT

    wl = PLAIN[args.workload]
    if args.segment_bits:
        wl.seg_bits = args.segment_bits
    steps = args.steps if args.steps else wl.default_steps
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = NAT.load()
    eng = ctd.Engine(local)
    info = eng.device_info()
    stream = torch.cuda.Stream(device=local)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    cap = mv_bound(wl.seg)
    primes = torch.empty(cap, dtype=torch.int64, device="cuda")
    bufs = []
    for fam, param, n0, n1 in wl.jobs:
        N = n1 - n0
        bufs.append((torch.zeros(N, dtype=torch.int32, device="cuda"),
                     torch.zeros(N * MAXF, dtype=torch.int64, device="cuda")))
    terms = [n1 - n0 for _, _, n0, n1 in wl.jobs]
    count = ctypes.c_uint64()

    def check(rc):
        if rc:
            raise NAT.CtdError(rc, L.ctd_last_error(eng.handle).decode())

    def seg_of(j):
        return wl.segment(rank * steps + j)

    def step(j, ev=None):
        """One segment for every job; returns the primes tested (the prime 2 included)."""
        fx, fy = seg_of(j)
        with torch.cuda.stream(stream):
            # each step is a fresh pass: the warm-up and whole-configuration
            # workloads run the same segment again, and hits pushed twice
            # would overflow the terms' slots
            for c, f in bufs:
                c.zero_()
                f.zero_()
            if ev is not None:
                ev[0].record(stream)
            extra = 0
            if fx <= 2 < fy:
                for (fam, param, n0, n1), (c, f) in zip(wl.jobs, bufs):
                    job = NAT.CtdJob(fam, MAXF, param, n0, n1, 2, fy)
                    check(L.ctd_mod2_device(eng.handle, ctypes.byref(job), ctypes.c_void_p(c.data_ptr()),
                                            ctypes.c_void_p(f.data_ptr()), sptr))
                extra, fx = 1, 3
            check(L.ctd_sieve_device(eng.handle, fx, fy, ctypes.c_void_p(primes.data_ptr()), cap,
                                     ctypes.byref(count), sptr))
            if ev is not None:
                ev[1].record(stream)
            for k, ((fam, param, n0, n1), (c, f)) in enumerate(zip(wl.jobs, bufs)):
                job = NAT.CtdJob(fam, MAXF, param, n0, n1, fx, fy)
                check(L.ctd_residues_device(eng.handle, ctypes.byref(job), ctypes.c_void_p(primes.data_ptr()),
                                            count.value, ctypes.c_void_p(c.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                                            sptr))
                if ev is not None:
                    ev[2 + k].record(stream)
        return count.value + extra, count.value

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for j in range(args.warmup):
        step(j)
    torch.cuda.synchronize()

    nj = len(wl.jobs)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2 + nj)] for _ in range(steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    launches0 = L.ctd_kernel_launches()
    barrier()
    torch.cuda.synchronize()
    nprimes, nodd = [], []
    with ClockSampler(local) as clocks:
        t_start.record(stream)
        for j in range(steps):
            a, b = step(j, evs[j])
            nprimes.append(a)
            nodd.append(b)
        t_end.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = L.ctd_kernel_launches() - launches0
    elapsed = t_start.elapsed_time(t_end) * 1e-3
    sieve_ms = [e[0].elapsed_time(e[1]) for e in evs]
    job_ms = [[evs[j][1 + k].elapsed_time(evs[j][2 + k]) for j in range(steps)] for k in range(nj)]
    updates = sum(nprimes) * sum(terms)
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
        # one fresh (zeroed, pinned) set of host factors buffers per step,
        # allocated before the timed region: each call starts a new pass
        def host_bufs():
            out = []
            for (fam, param, n0, n1) in wl.jobs:
                N = n1 - n0
                hc = torch.zeros(N, dtype=torch.int32).pin_memory()
                hf = torch.zeros(N * MAXF, dtype=torch.int64).pin_memory()
                out.append(ctd.factors_buffer(n0, MAXF, hc.numpy().view(np.uint32), hf.numpy().view(np.uint64)))
            return out

        hsets = [host_bufs() for _ in range(steps + 1)]

        def e2e_step(j, hbufs):
            fx, fy = seg_of(j)
            for (fam, param, n0, n1), buf in zip(wl.jobs, hbufs):
                eng.run_plain(NAT.CtdJob(fam, MAXF, param, n0, n1, fx, fy), buf, segment_length=wl.seg)

        e2e_step(0, hsets[steps])
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in range(steps):
            e2e_step(j, hsets[j])
        torch.cuda.synchronize()
        e2e_t = time.perf_counter() - t0
        barrier()
        e2e_total = float(updates)
        if world > 1:
            t = torch.tensor([e2e_t, e2e_total], dtype=torch.float64, device="cuda")
            tmax = t.clone()
            torch.distributed.all_reduce(tmax[:1], op=torch.distributed.ReduceOp.MAX)
            torch.distributed.all_reduce(t[1:], op=torch.distributed.ReduceOp.SUM)
            e2e_t, e2e_total = float(tmax[0]), float(t[1])
        # bytes across the link per step, as ctd_run_plain moves them: a fresh
        # (all-zero) resume state is cleared on the device, not uploaded; back
        # come the counts and one record {term, count, slots} per term with hits
        d2h = []
        for j in range(steps):
            b = 0
            for buf in hsets[j]:
                c = buf.counts.astype(np.int64)
                b += 4 * len(c) + 8 + 8 * int((np.minimum(c, MAXF) + 2)[c > 0].sum())
            d2h.append(b)
        e2e = {"value": e2e_total / e2e_t, "unit": "updates/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": int(statistics.mean(d2h)),
               "host_buffer_bytes_per_step": sum(N * (4 + 8 * MAXF) for N in terms),
               "api": "ctd_run_plain (include/ctd_gpu.h) per job with pinned host factors buffers, one segment per "
                      "call: the call reads the host resume state (all zeros: cleared on the device, nothing "
                      "uploaded) and writes back the counts and the occupied slots"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    peaks = probe_peaks(local)
    # the dominant launch of the step and its roofline
    k = max(range(nj), key=lambda i: sum(job_ms[i]))
    fam = wl.jobs[k][0]
    launch_s = statistics.mean(job_ms[k]) * 1e-3
    primes_launch = statistics.mean(nodd)
    per_launch_updates = primes_launch * terms[k]
    if wl.name == "proth":
        inst = sum(PROTH_NCU["thread_inst"].values()) / PROTH_NCU["primes"] * primes_launch
        achieved = inst / launch_s
        roofline = {
            "bound": "int_issue",
            "kernel": "screen_kernel<PROTH> + classify_kernel<PROTH, pattern> x 8 + refine_kernel<PROTH> + "
                      "nine_kernel<PROTH> + regroup_kernel + class_walk_kernel<PROTH>",
            "achieved": achieved / 1e9, "peak": (peaks["int"] / 1e9) if peaks["int"] else None, "unit": "Ginst/s",
            "frac": (achieved / peaks["int"]) if peaks["int"] else None,
            "thread_instructions_per_update": inst / per_launch_updates, "launch_ms": launch_s * 1e3,
            "achieved_source": "ncu thread instructions of the launch's 13 kernels on a 2^27-segment of this workload, "
                               "scaled by the primes per launch, over the CUDA-event launch time of this run",
            "peak_source": "measured now: libctd_probe add/xor chains (integer issue rate) on this GPU",
            "traffic": PROTH_NCU["dram_bytes"] / PROTH_NCU["primes"] * primes_launch,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the same capture, scaled by "
                              "the primes per launch",
            "algorithmic_bytes": 8 * primes_launch,
        }
    elif wl.name == "smarandache":
        achieved = per_launch_updates * SMARANDACHE_MULS_PER_UPDATE / launch_s
        roofline = {
            "bound": "int_multiply", "kernel": "residue_kernel<SMARANDACHE> (32-bit Shoup step)",
            "achieved": achieved / 1e9, "peak": (peaks["imad"] / 1e9) if peaks["imad"] else None,
            "unit": "Gmul/s", "frac": (achieved / peaks["imad"]) if peaks["imad"] else None,
            "muls_per_update": SMARANDACHE_MULS_PER_UPDATE, "launch_ms": launch_s * 1e3,
            "peak_source": "measured now: libctd_probe 32-bit multiply-add chains on this GPU",
            "traffic": None, "algorithmic_bytes": 8 * primes_launch,
        }
    else:
        achieved = per_launch_updates * TRIBONACCI_ALU_OPS_PER_UPDATE / launch_s
        roofline = {
            "bound": "int_alu", "kernel": f"residue_kernel<{FAMILY_NAMES[fam]}>",
            "achieved": achieved / 1e9, "peak": (peaks["alu"] / 1e9) if peaks["alu"] else None, "unit": "Gop/s",
            "frac": (achieved / peaks["alu"]) if peaks["alu"] else None,
            "ops_per_update": TRIBONACCI_ALU_OPS_PER_UPDATE, "launch_ms": launch_s * 1e3,
            "peak_source": "measured now: libctd_probe predicate-compare chains (integer ALU pipe) on this GPU",
            "traffic": None, "algorithmic_bytes": 8 * primes_launch,
        }
    roofline["kernel_share"] = sum(job_ms[k]) / max(sum(sum(x) for x in job_ms) + sum(sieve_ms), 1e-9)
    per_job = {f"{FAMILY_NAMES[f].lower()}": {"ms_per_launch": statistics.mean(job_ms[i]),
                                             "updates_per_s": statistics.mean(nodd) * terms[i] /
                                             (statistics.mean(job_ms[i]) * 1e-3)}
               for i, (f, _, _, _) in enumerate(wl.jobs)}
    sieve_s = statistics.mean(sieve_ms) * 1e-3
    hbm = measured_peaks().get("hbm_gbs")
    sieve_bytes = statistics.mean(nodd) * 8
    sieve = {"kernel": "device sieve (sieve_windows + scan_counts + compact_windows, host count readback)",
             "ms_per_step": statistics.mean(sieve_ms), "primes_per_step": statistics.mean(nodd),
             "achieved_gbs": sieve_bytes / sieve_s / 1e9, "peak_gbs": hbm,
             "frac": (sieve_bytes / sieve_s / 1e9 / hbm) if hbm else None,
             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm else "absent"}
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, _, dt, sample = cpu_updates_per_s(wl, 15.0, threads, wl.f0)
        cpu = {"value": rate, "unit": "updates/s", "cores": threads, "kind": "port", "sample": sample,
               "seconds": dt}
    line = {
        "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (deterministic: the configuration has no random input)",
        "config": {"workload": wl.text,
                   "step": f"one 2^{wl.seg_bits}-wide prime segment: device sieve + one residue launch per job",
                   "segments": wl.nseg, "max_factors_per_number": MAXF,
                   "l2": f"inputs larger than L2 (about {8 * statistics.mean(nodd) / 1e6:.0f} MB of primes per step)"
                         if 8 * statistics.mean(nodd) > 129e6 else
                         "the whole prime list of a step is read once per job launch",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU", "device": info["name"]},
        "roofline": roofline, "per_job": per_job, "sieve": sieve, "cpu_baseline": cpu, "e2e": e2e,
        "clocks": clocks.summary(), "gpu_launches": int(launches),
        "updates": total_updates, "seconds": elapsed,
    }
    ok = True
    if wl.name == "proth" and not args.no_batched:
        line["batched"] = measure_batched(args, eng, local)
        ok &= line["batched"]["identical_outputs"] and line["batched"]["identical_to_reference"]
    if wl.name == "proth" and not args.no_served:
        line["served"] = measure_served(args, eng, local)
        ok &= line["served"]["identical_to_reference"]
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0 if ok else 1


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


def reference_mix_files() -> dict:
    """The reference engine's factor files of the batched and serving mixes
    on their fixture samples (tests/golden/golden_job_mixes.json)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden_util import expand, parse_args

    with open(os.path.join(ROOT, "tests", "golden", "golden_job_mixes.json")) as fh:
        data = json.load(fh)
    out = {}
    for name, g in data.items():
        a = parse_args(g["args"])
        out[name] = (a["f1"], expand(a["n0"], a["n1"], g["nonempty"]))
    return out


def restricted_text(buf, bound: int) -> str:
    """A job's factor file keeping only the primes below `bound` (the factor
    file of the same job on the TF range cut at `bound`)."""
    res = buf.to_factoring_results()
    n0 = res.n0()
    lines = []
    for i in range(len(res)):
        ps = [p for p in res[i] if p < bound]
        lines.append(f"{n0 + i} - " + ", ".join(map(str, ps)))
    return "\n".join(lines) + "\n"


def measure_batched(args, eng, local) -> dict:
    """The batched mix through one ctd_batch_run against the same jobs one by
    one through ctd_run_plain (both on 2^30 segments, both with host buffers
    copied in and out inside the call)."""
    import torch

    from cutrialdive_gb300 import _native as NAT
    from cutrialdive_gb300 import jobs as J

    import cutrialdive_gb300 as ctd

    L = NAT.load()
    mix = J.batched_mix()
    jobs = [j.ctd(MAXF, args.batched_shrink) for j in mix]
    updates = job_updates(eng, jobs)
    seg = 1 << 30

    def bufs():
        return [ctd.factors_buffer.empty(j.n0, j.n1 - j.n0, MAXF) for j in jobs]

    def batched_pass():
        b = bufs()
        eng.batch_run(jobs, b, segment_length=seg, use_graph=True)
        return b

    def sequential_pass():
        b = bufs()
        for j, x in zip(jobs, b):
            eng.run_plain(j, x, segment_length=seg)
        return b

    out_b = batched_pass()  # warm-up: captures and instantiates the graph
    g0 = eng.batch_graph_stats()
    l0 = L.ctd_kernel_launches()
    steps = args.batched_steps
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            out_b = batched_pass()
        torch.cuda.synchronize()
        tb = (time.perf_counter() - t0) / steps
        launches_b = (L.ctd_kernel_launches() - l0) // steps
        l1 = L.ctd_kernel_launches()
        t0 = time.perf_counter()
        out_s = sequential_pass()
        torch.cuda.synchronize()
        ts = time.perf_counter() - t0
        launches_s = L.ctd_kernel_launches() - l1
    g1 = eng.batch_graph_stats()
    identical = all(same_results(a, b) for a, b in zip(out_b, out_s))
    ref = reference_mix_files()
    checked = 0
    ref_ok = True
    for i, (j, buf) in enumerate(zip(jobs, out_b)):
        name = f"batched{i:02d}"
        if name in ref:
            bound, text = ref[name]
            ref_ok &= restricted_text(buf, bound) == text
            checked += 1
    hbytes = sum((j.n1 - j.n0) * (4 + 8 * MAXF) for j in jobs)
    return {
        "workload": BATCHED_WORKLOAD,
        "sample": f"each job's TF range cut to its first 1/{args.batched_shrink}: "
                  f"[2^a, 2^a + 3*2^a/{args.batched_shrink})",
        "updates_per_step": updates,
        "value": updates / tb, "unit": "updates/s", "ms_per_step": 1e3 * tb, "steps": steps, "warmup": 1,
        "api": "one ctd_batch_run of all 64 jobs (2^30 segments, the schedule replayed as one CUDA graph), host "
               "factors buffers copied in and out inside the call",
        "sequential": {"value": updates / ts, "ms_per_step": 1e3 * ts, "steps": 1, "gpu_launches": int(launches_s),
                       "api": "ctd_run_plain per job, 2^30 segments, the same host buffers"},
        "batched_over_sequential": ts / tb,
        "identical_outputs": bool(identical),
        "identical_to_reference": bool(ref_ok and checked == len(jobs)),
        "reference_check": f"{checked} jobs: factor lines with p < 2^a + 2^24 equal the reference engine's files "
                           "(tests/golden/golden_job_mixes.json)",
        "graph": {k: g1[k] - g0[k] for k in g1},
        "gpu_launches": int(launches_b),
        "h2d_bytes_per_step": hbytes, "d2h_bytes_per_step": hbytes,
        "clocks": clocks.summary(),
    }


def measure_served(args, eng, local) -> dict:
    """Poisson arrivals of the serving stream through ctd_serve_*: per rate,
    the jobs arriving in the first `window` seconds, each job's TF range cut
    to its first 1/served_shrink; p50/p99 from arrival to fetched result."""
    import numpy as np

    import cutrialdive_gb300 as ctd
    from cutrialdive_gb300 import _native as NAT
    from cutrialdive_gb300 import jobs as J

    L = NAT.load()
    rates = [float(r) for r in args.rates.split(",")]
    ref = reference_mix_files()
    sweep = []
    ref_ok, checked = True, 0
    l0 = L.ctd_kernel_launches()
    with ClockSampler(local) as clocks:
        for rate in rates:
            mix, arrivals = J.served_mix(rate)
            count = min(len(mix), max(1, int(rate * args.window)))
            jobs = [j.ctd(MAXF, args.served_shrink) for j in mix[:count]]
            arrivals = arrivals[:count]
            updates = job_updates(eng, jobs)
            srv = ctd.Server(eng, memory_budget=160 << 30, max_active=256, segment_length=1 << 30)
            lat, ids, i, results = [], {}, 0, {}
            t0 = time.perf_counter()
            while len(lat) < count:
                now = time.perf_counter() - t0
                while i < count and arrivals[i] <= now:
                    ids[srv.submit(jobs[i])] = i
                    i += 1
                st = srv.status()
                if st["active"] or st["queued"]:
                    for jid in srv.tick():
                        k = ids.pop(jid)
                        results[k] = srv.fetch(jid)
                        lat.append(time.perf_counter() - t0 - arrivals[k])
                elif i < count:
                    time.sleep(max(0.0, min(arrivals[i] - now, 0.02)))
            span = time.perf_counter() - t0
            srv.close()
            for k, buf in results.items():
                name = f"served{k:03d}"
                if name in ref:
                    bound, text = ref[name]
                    ref_ok &= restricted_text(buf, bound) == text
                    checked += 1
            sweep.append({"rate_jobs_s": rate, "jobs": count, "p50_s": float(np.percentile(lat, 50)),
                          "p99_s": float(np.percentile(lat, 99)), "updates": updates,
                          "updates_per_s": updates / span, "seconds": span})
    return {
        "workload": "Serving: Poisson arrival stream from the batched distribution (seed 99), admission by a "
                    "160 GB device-memory budget",
        "sample": f"each job's TF range cut to its first 1/{args.served_shrink}; at each rate the jobs arriving in "
                  f"the first {args.window:g} s",
        "server": "ctd_serve_* with max_active 256, 2^30 segments per tick, ticks queued up to two ahead",
        "sweep": sweep,
        "identical_to_reference": bool(ref_ok and checked > 0),
        "reference_check": f"{checked} results of the stream's first 200 jobs, summed over the rates: factor lines "
                           "with p < 2^a + 2^22 equal the reference engine's files "
                           "(tests/golden/golden_job_mixes.json)",
        "gpu_launches": int(L.ctd_kernel_launches() - l0),
        "clocks": clocks.summary(),
    }


def run_batched(args, world, rank, local):
    import torch

    import cutrialdive_gb300 as ctd

    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    eng = ctd.Engine(local)
    b = measure_batched(args, eng, local)
    line = {
        "metric": METRIC, "value": b["value"], "unit": "updates/s", "n_gpus": 1, "steps": b["steps"],
        "warmup": b["warmup"], "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded job mix, seed 1234)",
        "config": {"workload": b["workload"], "sample": b["sample"]},
        "batched": b, "clocks": b["clocks"], "gpu_launches": b["gpu_launches"],
        "e2e": {"value": b["value"], "unit": "updates/s", "h2d_bytes_per_step": b["h2d_bytes_per_step"],
                "d2h_bytes_per_step": b["d2h_bytes_per_step"], "api": b["api"]},
    }
    print(json.dumps(line), flush=True)
    return 0 if b["identical_outputs"] and b["identical_to_reference"] else 1


def run_served(args, world, rank, local):
    import torch

    import cutrialdive_gb300 as ctd

    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    eng = ctd.Engine(local)
    sv = measure_served(args, eng, local)
    best = max(sv["sweep"], key=lambda r: r["updates_per_s"])
    line = {
        "metric": METRIC + "; p50/p99 job latency", "value": best["updates_per_s"], "unit": "updates/s",
        "n_gpus": 1, "steps": len(sv["sweep"]), "warmup": 0, "ms_per_step": 1e3 * best["seconds"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (Poisson arrivals of the seeded job mix, seed 99)",
        "config": {"workload": sv["workload"], "sample": sv["sample"], "server": sv["server"]},
        "served": sv, "clocks": sv["clocks"], "gpu_launches": sv["gpu_launches"],
        "e2e": {"value": best["updates_per_s"], "unit": "updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0, "api": "ctd_serve_submit/tick/fetch (host buffers)"},
    }
    print(json.dumps(line), flush=True)
    return 0 if sv["identical_to_reference"] else 1


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="timed steps (default: proth 12 = every 2^30 segment of [2^32, 2^34) once; linear 3; "
                         "smarandache 12; batched 3)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--segment-bits", type=int, default=0,
                    help="log2 of the prime-segment width of one step (profiling uses smaller cases)")
    ap.add_argument("--workload", choices=["proth", "linear", "smarandache", "batched", "served"], default="proth",
                    help="proth: the plain single-job line (default); linear: Fibonacci, Lucas and tribonacci back "
                         "to back; smarandache: the CPU-runnable plain configuration; batched: the 64-job mix "
                         "through ctd_batch_run against the same jobs one by one; served: the Poisson serving sweep")
    ap.add_argument("--batched-shrink", type=int, default=64,
                    help="batched: keep the first 1/shrink of each job's TF range")
    ap.add_argument("--batched-steps", type=int, default=2, help="batched: timed passes")
    ap.add_argument("--served-shrink", type=int, default=256,
                    help="served: keep the first 1/shrink of each job's TF range")
    ap.add_argument("--rates", default="10,50", help="served: arrival rates in jobs/s")
    ap.add_argument("--window", type=float, default=6.0, help="served: seconds of arrivals per rate")
    ap.add_argument("--no-batched", action="store_true", help="default line without the batched measurement")
    ap.add_argument("--no-served", action="store_true", help="default line without the served measurement")
    ap.add_argument("--cpu-seconds", type=float, default=2.0,
                    help="--impl reference: seconds of CPU work per step (a bounded sample of the step)")
    args = ap.parse_args()
    if not args.steps:
        args.steps = PLAIN[args.workload].default_steps if args.workload in PLAIN else 3
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
