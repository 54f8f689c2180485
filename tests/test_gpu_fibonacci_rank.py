"""Fibonacci and Lucas through the rank of apparition: for long index ranges
the residue kernel finds every hit of a prime from a(p) | p - (5/p) instead
of walking the recurrence.  The factors must equal the oracle's walk and the
kernel's own walk (CTD_VARIANT_WALK) on the same inputs, on both sides of
the cost model's choice and for tiled ranges."""
import pytest

import cutrialdive_gb300 as ctd
import oracle as O

pytestmark = pytest.mark.gpu


def run(eng, job):
    buf = ctd.factors_buffer.empty(job.n0, job.n1 - job.n0, job.max_factors)
    eng.run_plain(job, buf)
    return str(buf.to_factoring_results())


CASES = [
    # small primes: a(p) <= p + 1, so many hits and many capped lists
    (1, 3001, 3, 1 << 16),
    # primes around 2^30 and 2^36: hits only where a(p) is small
    (5, 20005, 1 << 30, (1 << 30) + (1 << 16)),
    (1000, 41000, 1 << 36, (1 << 36) + (1 << 16)),
    # the range ends at the trial table's limit (largest index 2^20 - 1)
    (2, 1 << 20, 1 << 33, (1 << 33) + (1 << 11)),
    # short range: the walk is cheaper and is taken
    (40000, 40300, 1 << 32, (1 << 32) + (1 << 20)),
]


@pytest.mark.parametrize("fam", [O.FIBONACCI, O.LUCAS])
@pytest.mark.parametrize("case", CASES)
def test_rank_path_matches_oracle_and_walk(eng, fam, case):
    n0, n1, f0, f1 = case
    job = ctd.CtdJob(fam, 32, 0, n0, n1, f0, f1)
    want = O.trial_factor(fam, 0, n0, n1, f0, f1, 32, threads=1).format()
    assert run(eng, job) == want
    try:
        eng.set_tuning(fam, {"block_size": 256, "ctas_per_sm": 0, "items_per_thread": 8, "min_tile": 4096,
                             "segment_log2": 0, "variant": 1})
        assert run(eng, job) == want
        # tiles of 1024 indices: each tile chooses between rank and walk
        eng.set_tuning(fam, {"block_size": 64, "ctas_per_sm": 1, "items_per_thread": 32, "min_tile": 1024,
                             "segment_log2": 22, "variant": 0})
        assert run(eng, job) == want
    finally:
        eng.set_tuning(fam, None)


@pytest.mark.parametrize("fam", [O.FIBONACCI, O.LUCAS])
def test_rank_path_in_batches(eng, fam):
    """The batched engine runs the same device code per (prime, range) item."""
    jobs = [ctd.CtdJob(fam, 32, 0, 1, 30001, 1 << 31, (1 << 31) + (1 << 20)),
            ctd.CtdJob(fam, 32, 0, 7, 5007, 3, 1 << 18)]
    bufs = [ctd.factors_buffer.empty(j.n0, j.n1 - j.n0, j.max_factors) for j in jobs]
    eng.batch_run(jobs, bufs)
    for j, b in zip(jobs, bufs):
        assert str(b.to_factoring_results()) == O.trial_factor(fam, 0, j.n0, j.n1, j.f0, j.f1, 32,
                                                                threads=1).format()
