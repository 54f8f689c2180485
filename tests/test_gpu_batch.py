"""Batched and served forms: every job's factors buffer in the mix equals
the oracle's for that job alone (exact where no term overflowed its slots;
equal counts and valid stored primes where one did)."""
import functools
import random

import pytest

import cutrialdive_gb300 as ctd
import oracle as O

pytestmark = pytest.mark.gpu

M = 32
W = 1 << 22
# heterogeneous jobs whose prime ranges overlap and straddle 2^22-aligned
# segments; some include the prime 2, some start below 2^16
MIX = [
    (O.PROTH, 3, 1, 4001, 1 << 30, (1 << 30) + W),
    (O.RIESEL, 999_999, 10, 2010, (1 << 30) + (W >> 1), (1 << 30) + W + (W >> 1)),
    (O.MERSENNE, 0, 2000, 6000, (1 << 30) - (W >> 1), (1 << 30) + (W >> 1)),
    (O.PROTH_FIXED_N, 12345, 1, 3001, (1 << 30) + 3 * W, (1 << 30) + 4 * W),
    (O.SMARANDACHE, 10, 10, 1001, 2, W),
    (O.SMARANDACHE, 7, 500, 900, 1 << 30, (1 << 30) + W),
    (O.FIBONACCI, 0, 1, 3001, 2, W >> 1),
    (O.TRIBONACCI, 0, 2, 2002, (1 << 30) - (W >> 2), (1 << 30) + (W >> 2)),
    (O.LUCAS, 0, 5, 905, 1 << 20, W),
]


@functools.lru_cache(maxsize=None)
def alone(case):
    f, p, n0, n1, f0, f1 = case
    return O.trial_factor(f, p, n0, n1, f0, f1, M)


def assert_same(buf, case):
    want = alone(case)
    assert buf.counts.tolist() == want.counts.tolist(), case
    gl, wl = buf.to_factoring_results(), want.factor_lists()
    f0, f1 = case[4], case[5]
    for i, c in enumerate(buf.counts.tolist()):
        if c <= M:
            assert gl[i] == wl[i], (case, i)
        else:  # overflow: which primes are kept depends on arrival order
            assert len(set(gl[i])) == M and all(f0 <= q < f1 for q in gl[i]), (case, i)


def new_buffers(mix):
    jobs = [ctd.CtdJob(f, M, p, n0, n1, f0, f1) for f, p, n0, n1, f0, f1 in mix]
    bufs = [ctd.factors_buffer.empty(n0, n1 - n0, M) for f, p, n0, n1, f0, f1 in mix]
    return jobs, bufs


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_equals_alone(eng, use_graph):
    jobs, bufs = new_buffers(MIX)
    eng.batch_run(jobs, bufs, segment_length=W, use_graph=use_graph)
    for case, buf in zip(MIX, bufs):
        assert_same(buf, case)


def test_batch_single_job_matches_plain(eng):
    case = MIX[0]
    jobs, bufs = new_buffers([case])
    eng.batch_run(jobs, bufs, segment_length=0, use_graph=True)
    plain = ctd.factors_buffer.empty(case[2], case[3] - case[2], M)
    eng.run_plain(jobs[0], plain)
    assert str(bufs[0].to_factoring_results()) == str(plain.to_factoring_results())


def test_served_equals_alone(eng):
    """Jobs arrive while others run (two per tick, at most four active) and
    finish in any order."""
    srv = ctd.Server(eng, memory_budget=1 << 30, max_active=4, segment_length=W)
    pending = list(range(len(MIX)))
    random.Random(7).shuffle(pending)
    ids, results = {}, {}
    ticks = 0
    while pending or len(results) < len(MIX):
        for _ in range(2):
            if pending:
                k = pending.pop()
                f, p, n0, n1, f0, f1 = MIX[k]
                ids[srv.submit(ctd.CtdJob(f, M, p, n0, n1, f0, f1))] = k
        st = srv.status()
        assert st["active"] <= 4
        for jid in srv.tick():
            results[ids[jid]] = srv.fetch(jid)
        ticks += 1
        assert ticks < 10_000
    assert srv.status() == {"active": 0, "queued": 0, "memory_used": 0}
    srv.close()
    for k, case in enumerate(MIX):
        assert_same(results[k], case)


def test_server_admission_by_memory_budget(eng):
    """A budget smaller than any job's buffers admits one job at a time (a
    job that does not fit is still admitted when nothing else runs), and
    every result equals the oracle's."""
    srv = ctd.Server(eng, memory_budget=1, max_active=8, segment_length=W)
    ids = {srv.submit(ctd.CtdJob(f, M, p, n0, n1, f0, f1)): k for k, (f, p, n0, n1, f0, f1) in enumerate(MIX[:4])}
    results = {}
    for _ in range(10_000):
        if len(results) == len(ids):
            break
        st = srv.status()
        assert st["active"] <= 1
        for jid in srv.tick():
            results[ids[jid]] = srv.fetch(jid)
    srv.close()
    assert len(results) == len(ids)
    for k in results:
        assert_same(results[k], MIX[k])


def test_batch_rejects_invalid_jobs(eng):
    jobs, bufs = new_buffers(MIX[:2])
    jobs[1] = ctd.CtdJob(O.PROTH, M, 0, 1, 10, 3, 100)  # k = 0 is rejected, as by the reference
    with pytest.raises(ctd.CtdError):
        eng.batch_run(jobs, bufs)


def test_batch_graph_replayed_and_updated(eng):
    """A second call with the same schedule replays the captured graph; one
    with the same shape but other jobs updates it in place; both give the
    oracle's results."""
    before = eng.batch_graph_stats()
    for _ in range(2):
        jobs, bufs = new_buffers(MIX)
        eng.batch_run(jobs, bufs, segment_length=W, use_graph=True)
        for case, buf in zip(MIX, bufs):
            assert_same(buf, case)
    mid = eng.batch_graph_stats()
    assert mid["replays"] >= before["replays"] + 1
    # same shape (segments, active lists, launches), other launch arguments:
    # the Smarandache job that includes the prime 2 ends one term earlier
    other = [(f, p, n0, n1 - 1 if (f, p) == (O.SMARANDACHE, 10) else n1, f0, f1) for f, p, n0, n1, f0, f1 in MIX]
    jobs, bufs = new_buffers(other)
    eng.batch_run(jobs, bufs, segment_length=W, use_graph=True)
    for case, buf in zip(other, bufs):
        assert_same(buf, case)
    after = eng.batch_graph_stats()
    assert after["updates"] == mid["updates"] + 1 and after["instantiations"] == mid["instantiations"]
