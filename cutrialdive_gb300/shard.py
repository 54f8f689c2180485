"""Prime-range sharding across GPUs or hosts.

Trial factoring shards by prime with no exchange step: every prime's residue
walk is independent, so each shard trial-factors the same terms by its own
contiguous slice of [f0, f1) and produces its own factors buffer.  The only
combining step is the per-term union of the shards' factor lists, which the
reference already performs when it sorts each term's slots
(src/factors_buffer.hpp:123-138).  No device collective is involved: ranks
exchange host factors buffers once, at the end.
"""
from __future__ import annotations

import numpy as np

from .api import factors_buffer


def split_prime_range(f0: int, f1: int, shards: int, align: int = 1 << 20) -> list[tuple[int, int]]:
    """Contiguous [a, b) slices covering [f0, f1), boundaries on multiples of
    `align` where possible, sized so the prime counts are close to equal
    (slices are sized by x/ln x, the prime-counting estimate)."""
    if shards < 1 or f1 <= f0:
        raise ValueError("need at least one shard and a non-empty range")
    import math

    def li(x: float) -> float:  # logarithmic-integral-like estimate of pi(x)
        x = max(x, 3.0)
        return x / math.log(x)

    target = [li(f0) + (li(f1) - li(f0)) * k / shards for k in range(1, shards)]
    cuts = [f0]
    lo, hi = f0, f1
    for t in target:
        a, b = cuts[-1], f1
        while b - a > 1:  # bisect x with li(x) ~ t
            m = (a + b) // 2
            if li(m) < t:
                a = m
            else:
                b = m
        c = (b // align) * align if align > 1 else b
        c = min(max(c, cuts[-1]), f1)
        cuts.append(c)
    cuts.append(f1)
    return [(cuts[i], cuts[i + 1]) for i in range(shards)]


def merge_buffers(parts: list[factors_buffer]) -> factors_buffer:
    """Per-term union of shard factors buffers over the same terms.

    Counts add up; stored factors are concatenated in shard order and kept up
    to the per-term capacity (when a term overflows, which factors are kept
    depends on arrival order in the reference as well)."""
    if not parts:
        raise ValueError("nothing to merge")
    n0, m, N = parts[0].n0, parts[0].max_factors_per_number, parts[0].numbers_count
    for p in parts:
        if (p.n0, p.max_factors_per_number, p.numbers_count) != (n0, m, N):
            raise ValueError("shards cover different terms")
    out = factors_buffer.empty(n0, N, m)
    fo = out.factors.reshape(N, m)
    fill = np.zeros(N, np.int64)
    for p in parts:
        fp = p.factors.reshape(N, m)
        stored = np.minimum(p.counts.astype(np.int64), m)
        for i in np.nonzero(stored)[0]:
            take = int(min(stored[i], m - fill[i]))
            if take > 0:
                fo[i, fill[i]:fill[i] + take] = fp[i, :take]
                fill[i] += take
        out.counts += p.counts
    return out


def run_sharded(spec, opts, compute, rank: int, world: int, group=None) -> factors_buffer | None:
    """Runs this rank's slice of the prime range with `compute(spec, opts,
    f0, f1) -> factors_buffer` and gathers every shard's buffer on rank 0,
    which returns the merged buffer (other ranks return None).

    `compute` is the GPU engine in production (one rank per GPU); the
    exchange uses torch.distributed object collectives (NCCL or gloo)."""
    import torch.distributed as dist

    lo, hi = split_prime_range(opts.f0, opts.f1, world)[rank]
    local = compute(spec, opts, lo, hi)
    gathered = [None] * world if rank == 0 else None
    dist.gather_object((lo, hi, local.counts, local.factors), gathered, dst=0, group=group)
    if rank != 0:
        return None
    parts = [factors_buffer(opts.n0, opts.max_factors_per_number, c, f) for (_, _, c, f) in gathered]
    return merge_buffers(parts)


def gpu_compute(spec, opts, f0: int, f1: int, device: int = 0) -> factors_buffer:
    """One shard on one GPU through the C ABI (ctd_run_plain)."""
    from .api import engine, make_job, trial_factoring_options

    sub = trial_factoring_options(opts.n0, opts.n1, f0, f1, None, opts.max_factors_per_number)
    buf = factors_buffer.empty(opts.n0, opts.n1 - opts.n0, opts.max_factors_per_number)
    if f1 > f0:
        engine(device).run_plain(make_job(spec, sub), buf)
    return buf


# --------------------------------------------------------------- factor files
def parse_factor_file(text: str) -> dict[int, list[int]]:
    """'<n> - p1, p2' lines (src/factoring_results.hpp:185-201) -> {n: [p...]}."""
    out: dict[int, list[int]] = {}
    for ln in text.splitlines():
        if not ln.strip():
            continue
        head, sep, tail = ln.partition(" - ")
        if not sep:
            head, tail = ln.rstrip().rstrip("-").strip(), ""
        n = int(head)
        ps = [int(x) for x in tail.replace(",", " ").split()]
        out.setdefault(n, []).extend(ps)
    return out


def merge_factor_files(texts: list[str]) -> str:
    """Per-term union of factor files over the same terms, each term's primes
    ascending, in the reference's line format (a term with no factor keeps
    its trailing space)."""
    merged: dict[int, set[int]] = {}
    for t in texts:
        for n, ps in parse_factor_file(t).items():
            merged.setdefault(n, set()).update(ps)
    return "".join(f"{n} - {', '.join(map(str, sorted(merged[n])))}\n" for n in sorted(merged))


def _main(argv=None) -> int:
    import argparse
    import sys

    ap = argparse.ArgumentParser(prog="python -m cutrialdive_gb300.shard",
                                 description="Split a TF range into prime-balanced shards, or merge shard factor files.")
    sub = ap.add_subparsers(dest="cmd", required=True)
    sp = sub.add_parser("split", help="print one '--tf-start A --tf-end B' line per shard")
    sp.add_argument("f0", type=int)
    sp.add_argument("f1", type=int)
    sp.add_argument("shards", type=int)
    sp.add_argument("--align", type=int, default=1 << 20)
    mp = sub.add_parser("merge", help="merge factor files of the same terms into one")
    mp.add_argument("files", nargs="+")
    mp.add_argument("-o", "--output")
    a = ap.parse_args(argv)
    if a.cmd == "split":
        for lo, hi in split_prime_range(a.f0, a.f1, a.shards, a.align):
            print(f"--tf-start {lo} --tf-end {hi}")
        return 0
    texts = []
    for f in a.files:
        with open(f) as fh:
            texts.append(fh.read())
    out = merge_factor_files(texts)
    if a.output:
        with open(a.output, "w") as fh:
            fh.write(out)
    else:
        sys.stdout.write(out)
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
