"""Golden factor files at configuration scale, from the reference's own CPU engine.

Runs oracle/_ref/cutrialdive_ref (cutrialdive 1.2.0's CPU build, compiled from
its unmodified sources by oracle/build_ref.sh) and stores each factor file in
the sparse form of make_golden_factor_files.py (command line, sha256 of the
whole file, its non-empty lines):

* golden_scale_slices.json -- sixteen evenly spaced 2^24-wide prime slices
  across each plain configuration's whole TF range, the last one ending at
  the range's top:
    - Proth 3*2^n+1, n = 1..100000, slices of [2^32, 2^34);
    - Fibonacci, Lucas and tribonacci, n = 1..50000, slices of
      [2^34, 2^36); tribonacci from n = 2, because every prime divides
      T(1) = 0, so that term overflows its slots and which primes the
      reference's multi-threaded engine keeps there depends on timing.
* golden_job_mixes.json -- the batched mix (64 jobs, seed 1234) with each
  job's TF range cut to its first 2^24 integers, [2^a, 2^a + 2^24), and the
  first 200 jobs of the serving stream (seed 99) cut to [2^a, 2^a + 2^22).

Usage: python tests/golden/make_golden_scale.py [slices|mixes|all]
(runs only where the reference engine was built; about an hour on 8 cores).
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden_factor_files import REF, run_case, sparse  # noqa: E402

SLICE_BITS = 24
NSLICES = 16
MIX_SAMPLE_BITS = {"batched": 24, "served": 22}
SERVED_JOBS = 200


def slice_starts(f0: int, f1: int) -> list[int]:
    """NSLICES evenly spaced 2^SLICE_BITS-wide slices of [f0, f1), the first
    at f0 and the last ending at f1."""
    w = 1 << SLICE_BITS
    span = (f1 - w) - f0
    return [f0 + span * i // (NSLICES - 1) for i in range(NSLICES)]


def slice_cases() -> dict:
    cases = {}
    for lo in slice_starts(1 << 32, 1 << 34):
        cases[f"proth3_n1-100001_p{lo}"] = (f"--num-seq proth,3 -s 1 -e 100001 --tf-start {lo} "
                                            f"--tf-end {lo + (1 << SLICE_BITS)}")
    for fam, n0 in (("fibonacci", 1), ("lucas", 1), ("tribonacci", 2)):
        for lo in slice_starts(1 << 34, 1 << 36):
            cases[f"{fam}_n{n0}-50001_p{lo}"] = (f"--num-seq {fam} -s {n0} -e 50001 --tf-start {lo} "
                                                 f"--tf-end {lo + (1 << SLICE_BITS)}")
    return cases


def job_args(job, sample_bits: int) -> str:
    spec = job.family if job.family == "mersenne" else f"{job.family},{job.param}"
    f0 = 1 << job.a
    return f"--num-seq {spec} -s {job.n0} -e {job.n1} --tf-start {f0} --tf-end {f0 + (1 << sample_bits)}"


def mix_cases() -> dict:
    from cutrialdive_gb300 import jobs as J

    out = {}
    for i, j in enumerate(J.batched_mix()):
        out[f"batched{i:02d}"] = job_args(j, MIX_SAMPLE_BITS["batched"])
    served, _ = J.served_mix(1.0)
    for i, j in enumerate(served[:SERVED_JOBS]):
        out[f"served{i:03d}"] = job_args(j, MIX_SAMPLE_BITS["served"])
    return out


def generate(cases: dict, path: str) -> None:
    data = {}
    if os.path.exists(path):
        with open(path) as fh:
            data = json.load(fh)
    threads = max(os.cpu_count() or 2, 2)  # >= 2 threads: the siever's [start, end) contract
    for name, args in cases.items():
        if name in data and data[name]["args"] == args:
            continue
        t = time.time()
        text = run_case(args, threads)
        data[name] = {"args": args, **sparse(text)}
        print(f"{name}: {len(data[name]['nonempty'])} lines with factors, {time.time() - t:.1f}s", flush=True)
        with open(path + ".tmp", "w") as fh:  # keep what is done if interrupted
            json.dump(data, fh, indent=0)
        os.replace(path + ".tmp", path)
    data = {k: data[k] for k in cases}
    with open(path, "w") as fh:
        json.dump(data, fh, indent=0)


def main() -> None:
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/cutrialdive_ref is missing: run oracle/build_ref.sh where the reference is mounted")
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    if which in ("slices", "all"):
        generate(slice_cases(), os.path.join(HERE, "golden_scale_slices.json"))
    if which in ("mixes", "all"):
        generate(mix_cases(), os.path.join(HERE, "golden_job_mixes.json"))


if __name__ == "__main__":
    main()
