"""GPU parity at configuration scale.

* Sixteen 2^24-wide prime slices spread over each plain configuration's whole
  TF range (Proth k=3 over [2^32, 2^34); Fibonacci, Lucas and tribonacci over
  [2^34, 2^36)), byte-identical to the factor files of the reference's own
  CPU engine (tests/golden/golden_scale_slices.json).
* The batched mix (64 jobs, seed 1234) and the first 200 jobs of the serving
  stream (seed 99) on stated samples of their TF ranges, each job's factor
  file byte-identical to the reference engine's for that job alone
  (tests/golden/golden_job_mixes.json) -- through ctd_run_plain one by one,
  through ctd_batch_run all at once, and through the server with jobs
  arriving while others run.
* Whole configuration ranges, where no CPU can produce the file in time: the
  default step forms against the term-by-term walk (CTD_VARIANT_WALK), two
  different algorithms that must report the same factor lists.
"""
import json
import os

import pytest

import cutrialdive_gb300 as ctd
import oracle as O
from golden_util import expand, parse_args, sha256

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):  # reported by test_fixtures_present
        return {}
    with open(path) as fh:
        return json.load(fh)


SLICES = load("golden_scale_slices.json")
MIXES = load("golden_job_mixes.json")


def test_fixtures_present():
    assert len(SLICES) == 64, "tests/golden/golden_scale_slices.json: run tests/golden/make_golden_scale.py"
    assert len(MIXES) == 264, "tests/golden/golden_job_mixes.json: run tests/golden/make_golden_scale.py"


def job_of(a):
    return ctd.CtdJob(a["family"], a["max_factors"], a["param"], a["n0"], a["n1"], a["f0"], a["f1"])


def want_text(g):
    a = parse_args(g["args"])
    text = expand(a["n0"], a["n1"], g["nonempty"])
    assert sha256(text) == g["sha256"], "fixture does not rebuild"
    return text


def first_diff(got, want):
    return [(x, y) for x, y in zip(got.splitlines(), want.splitlines()) if x != y][:5]


def run_plain(eng, a, seg=0):
    buf = ctd.factors_buffer.empty(a["n0"], a["n1"] - a["n0"], a["max_factors"])
    eng.run_plain(job_of(a), buf, segment_length=seg)
    return str(buf.to_factoring_results())


@pytest.mark.parametrize("name", sorted(SLICES))
def test_configuration_slices(eng, name):
    g = SLICES[name]
    got = run_plain(eng, parse_args(g["args"]))
    want = want_text(g)
    assert got == want, f"{name}: {first_diff(got, want)}"


def mix(prefix):
    return {k: v for k, v in MIXES.items() if k.startswith(prefix)}


def test_batched_mix_plain_one_by_one(eng):
    for name, g in mix("batched").items():
        got = run_plain(eng, parse_args(g["args"]))
        want = want_text(g)
        assert got == want, f"{name}: {first_diff(got, want)}"


@pytest.mark.parametrize("use_graph", [True, False])
def test_batched_mix_all_at_once(eng, use_graph):
    cases = mix("batched")
    args = [parse_args(g["args"]) for g in cases.values()]
    jobs = [job_of(a) for a in args]
    bufs = [ctd.factors_buffer.empty(a["n0"], a["n1"] - a["n0"], a["max_factors"]) for a in args]
    eng.batch_run(jobs, bufs, use_graph=use_graph)
    for (name, g), buf in zip(cases.items(), bufs):
        got, want = str(buf.to_factoring_results()), want_text(g)
        assert got == want, f"{name}: {first_diff(got, want)}"


def test_served_stream(eng):
    """The serving stream's first 200 jobs, submitted four per tick in
    arrival order while earlier ones run (at most 64 active)."""
    cases = mix("served")
    names = sorted(cases)
    srv = ctd.Server(eng, memory_budget=8 << 30, max_active=64)
    ids, results = {}, {}
    pending = list(names)
    for _ in range(100_000):
        for _ in range(4):
            if pending:
                name = pending.pop(0)
                ids[srv.submit(job_of(parse_args(cases[name]["args"])))] = name
        for jid in srv.tick():
            results[ids[jid]] = srv.fetch(jid)
        if not pending and len(results) == len(names):
            break
    srv.close()
    assert len(results) == len(names)
    for name in names:
        got, want = str(results[name].to_factoring_results()), want_text(cases[name])
        assert got == want, f"{name}: {first_diff(got, want)}"


def run_variant(eng, family, variant, n0, n1, f0, f1):
    eng.set_tuning(family, None)
    t = eng.get_tuning(family)
    t["variant"] = variant
    eng.set_tuning(family, t)
    try:
        buf = ctd.factors_buffer.empty(n0, n1 - n0, 32)
        eng.run_plain(ctd.CtdJob(family, 32, 0 if family != O.PROTH else 3, n0, n1, f0, f1), buf,
                      segment_length=1 << 30)
        return buf
    finally:
        eng.set_tuning(family, None)


@pytest.mark.parametrize("family,n1,f0,f1", [(O.PROTH, 100001, 1 << 32, 1 << 34),
                                             (O.FIBONACCI, 50001, 1 << 34, 1 << 36),
                                             (O.LUCAS, 50001, 1 << 34, 1 << 36)])
def test_whole_configuration_against_the_walk(eng, family, n1, f0, f1):
    """The whole plain configuration range through the default step forms
    (filtered baby-step blocks for Proth, the rank of apparition for
    Fibonacci and Lucas) and through the term-by-term walk: equal factor
    lists, thousands of hits each."""
    fast = run_variant(eng, family, 0, 1, n1, f0, f1)
    walk = run_variant(eng, family, 1, 1, n1, f0, f1)
    assert fast.counts.tolist() == walk.counts.tolist()
    got, want = str(fast.to_factoring_results()), str(walk.to_factoring_results())
    assert got == want, first_diff(got, want)
    assert int(fast.counts.sum()) > 1000
    # soundness of a sample of the hits, with Python integers
    res = fast.to_factoring_results()
    checked = 0
    for i in range(0, len(res), 97):
        for p in res[i]:
            n = 1 + i
            if family == O.PROTH:
                assert (3 * pow(2, n, p) + 1) % p == 0
            checked += 1
    assert checked > 0


@pytest.mark.parametrize("family,param,n0,n1,f0,sub", [
    (O.PROTH, 3, 1, 100001, 1 << 32, 1 << 21),
    (O.FIBONACCI, 0, 1, 50001, 1 << 35, 1 << 20),
    (O.LUCAS, 0, 1, 50001, 1 << 35, 1 << 20),
    (O.TRIBONACCI, 0, 2, 50001, 1 << 35, 1 << 20),
])
def test_hits_at_scale_complete_on_a_subslice(eng, family, param, n0, n1, f0, sub):
    """A 2^28-wide range at configuration widths: every (n, p) the GPU
    reports on its first `sub` integers equals the oracle's list there (no
    missed hit, no extra hit), and every reported p lies in the range."""
    f1 = f0 + (1 << 28)
    buf = ctd.factors_buffer.empty(n0, n1 - n0, 32)
    eng.run_plain(ctd.CtdJob(family, 32, param, n0, n1, f0, f1), buf)
    res = buf.to_factoring_results()
    got = [[p for p in res[i] if p < f0 + sub] for i in range(len(res))]
    want = O.trial_factor(family, param, n0, n1, f0, f0 + sub, max_factors=32).factor_lists()
    assert got == want
    assert all(f0 <= p < f1 for i in range(len(res)) for p in res[i])
