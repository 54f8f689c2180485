"""Multi-GPU story on CPU: prime-range shards, gathered and merged on rank 0
over torch.distributed (gloo, world_size 2).  The per-shard compute here is
the CPU oracle (the GPU engine in production); what is under test is the
split / gather / merge logic, checked against an unsharded oracle run."""
import os
import socket

import numpy as np
import pytest

import cutrialdive_gb300 as ctd
from cutrialdive_gb300 import shard

import oracle as O

CASES = [(O.PROTH, 3, 1, 3001, 0, 1 << 20), (O.SMARANDACHE, 10, 10, 400, 2, 1 << 20),
         (O.TRIBONACCI, 0, 2, 2002, 1 << 18, 1 << 21)]


def oracle_compute(spec, opts, f0, f1):
    fam, param = ctd.dispatch(spec)
    buf = ctd.factors_buffer.empty(opts.n0, opts.n1 - opts.n0, opts.max_factors_per_number)
    if f1 > f0:
        b = O.trial_factor(fam, param, opts.n0, opts.n1, f0, f1, opts.max_factors_per_number, threads=2)
        buf.counts[:], buf.factors[:] = b.counts, b.factors
    return buf


def spec_of(fam, param):
    names = {O.PROTH: "proth", O.SMARANDACHE: "smarandache", O.TRIBONACCI: "tribonacci"}
    return ctd.num_seq_spec(ctd.num_seq_id[names[fam]], str(param) if fam != O.TRIBONACCI else "")


@pytest.mark.parametrize("shards", [1, 2, 3, 7])
def test_split_covers_range(shards):
    f0, f1 = 12345, (1 << 34) + 99
    parts = shard.split_prime_range(f0, f1, shards)
    assert parts[0][0] == f0 and parts[-1][1] == f1 and len(parts) == shards
    assert all(a <= b for a, b in parts)
    assert all(parts[i][1] == parts[i + 1][0] for i in range(shards - 1))


@pytest.mark.parametrize("case", CASES)
def test_merge_equals_unsharded(case):
    fam, param, n0, n1, f0, f1 = case
    spec = spec_of(fam, param)
    opts = ctd.trial_factoring_options(n0, n1, f0, f1, None, 64)
    parts = [oracle_compute(spec, opts, a, b) for a, b in shard.split_prime_range(f0, f1, 3, align=1 << 10)]
    merged = shard.merge_buffers(parts)
    full = O.trial_factor(fam, param, n0, n1, f0, f1, 64, threads=2)
    assert str(merged.to_factoring_results()) == full.format()
    assert np.array_equal(merged.counts, full.counts)


def _worker(rank, world, port, queue):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = []
        for fam, param, n0, n1, f0, f1 in CASES:
            spec = spec_of(fam, param)
            opts = ctd.trial_factoring_options(n0, n1, f0, f1, None, 64)
            merged = shard.run_sharded(spec, opts, oracle_compute, rank, world)
            if rank == 0:
                out.append(str(merged.to_factoring_results()))
            else:
                assert merged is None
        if rank == 0:
            queue.put(out)
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_gather_and_merge():
    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    got = queue.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for (fam, param, n0, n1, f0, f1), text in zip(CASES, got):
        assert text == O.trial_factor(fam, param, n0, n1, f0, f1, 64, threads=2).format()


def test_factor_file_split_and_merge_cli(tmp_path):
    """The multi-box story as files: one factor file per shard, merged."""
    fam, param, n0, n1, f0, f1 = CASES[0]
    parts = shard.split_prime_range(f0, f1, 3, align=1 << 10)
    paths = []
    for k, (a, b) in enumerate(parts):
        p = tmp_path / f"shard{k}.txt"
        p.write_text(O.trial_factor(fam, param, n0, n1, a, b, 64, threads=2).format())
        paths.append(str(p))
    out = tmp_path / "merged.txt"
    assert shard._main(["merge", *paths, "-o", str(out)]) == 0
    assert out.read_text() == O.trial_factor(fam, param, n0, n1, f0, f1, 64, threads=2).format()


def test_split_cli_prints_ranges(capsys):
    assert shard._main(["split", "4294967296", "17179869184", "4"]) == 0
    lines = capsys.readouterr().out.splitlines()
    assert len(lines) == 4 and lines[0].startswith("--tf-start 4294967296 ") and lines[-1].endswith(" 17179869184")
