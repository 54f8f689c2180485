"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
golden factor files produced by the reference's own engine.  Integer work:
every comparison is exact (byte-identical factor files, equal prime lists).
"""
import numpy as np
import pytest

import cutrialdive_gb300 as ctd
import oracle as O
from golden_util import expand, parse_args, sha256

pytestmark = pytest.mark.gpu


def run_gpu(eng, family, param, n0, n1, f0, f1, max_factors=32, resume=0, seg=0, buf=None, cb=None):
    job = ctd.CtdJob(family, max_factors, param, n0, n1, f0, f1)
    if buf is None:
        buf = ctd.factors_buffer.empty(n0, n1 - n0, max_factors)
    eng.run_plain(job, buf, resume_after_prime=resume, segment_length=seg, callback=cb)
    return buf


def text(buf):
    return str(buf.to_factoring_results())


# ----------------------------------------------------------------- sieve
def test_sieve_known_answers(eng, kats):
    # src/autotests.cpp:136-351, including the window near 2^61
    for c in kats["sieve"]:
        got = eng.sieve(c["lo"], c["hi"]).tolist()
        if "expected" in c:
            assert got == c["expected"], c["src"]
        if "count" in c:
            assert len(got) == c["count"], c["src"]


@pytest.mark.parametrize("lo,hi", [(0, 3), (0, 100), (2, 3), (3, 4), (1, 2), (9, 10), (0, 1 << 20),
                                   ((1 << 20) - 7, (1 << 21) + 9), (1 << 32, (1 << 32) + (1 << 21)),
                                   ((1 << 34) - 12345, (1 << 34) + 54321), ((1 << 40) + 3, (1 << 40) + (1 << 20)),
                                   (999_999_937, 1_000_000_000 + (1 << 20) + 11)])
def test_sieve_matches_oracle(eng, lo, hi):
    assert np.array_equal(eng.sieve(lo, hi), O.sieve(lo, hi))


def test_sieve_window_edges(eng):
    # ranges that start and end on window and word boundaries of the device sieve
    W = 1 << 20
    for k in (1, 2, 3, 7):
        lo = (1 << 33) + k * W
        for d in (-65, -64, -1, 0, 1, 63, 64, 65):
            a, b = lo + d, lo + 3 * W + d
            assert np.array_equal(eng.sieve(a, b), O.sieve(a, b)), (a, b)


def test_sieve_prime_counts(eng):
    # pi(2^28) (the plain Smarandache configuration) and pi(2^30)
    assert eng.sieve(0, 1 << 28).size == 14_630_843
    assert eng.sieve(0, 1 << 30).size == 54_400_028


# --------------------------------------------------------- golden files
def test_golden_factor_files(eng, golden_files):
    """Every factor file the reference engine produced, byte for byte."""
    for name, g in golden_files.items():
        a = parse_args(g["args"])
        buf = run_gpu(eng, a["family"], a["param"], a["n0"], a["n1"], a["f0"], a["f1"], a["max_factors"])
        got = text(buf)
        want = expand(a["n0"], a["n1"], g["nonempty"])
        assert sha256(want) == g["sha256"], f"{name}: fixture does not rebuild"
        if got != want:
            gl, wl = got.splitlines(), want.splitlines()
            diff = [(x, y) for x, y in zip(gl, wl) if x != y][:5]
            pytest.fail(f"{name}: GPU factor file differs from the reference engine's: {diff}")


# ------------------------------------------------------ oracle parity
FAMILIES = [(O.PROTH, 3), (O.PROTH, 2718281828459), (O.RIESEL, 999_999), (O.MERSENNE, 0),
            (O.FIBONACCI, 0), (O.LUCAS, 0), (O.TRIBONACCI, 0), (O.PROTH_FIXED_N, 1234),
            (O.RIESEL_FIXED_N, 20000), (O.SMARANDACHE, 2), (O.SMARANDACHE, 10), (O.SMARANDACHE, 13),
            (O.SMARANDACHE, 16), (O.SMARANDACHE, 64), (O.PEANO, 0)]


@pytest.mark.parametrize("family,param", FAMILIES)
def test_small_primes_vs_oracle(eng, family, param):
    n0, n1 = (3, 2003) if family != O.PEANO else (2956708207, 2956708707)
    got = run_gpu(eng, family, param, n0, n1, 0, 1 << 18, max_factors=64)
    want = O.trial_factor(family, param, n0, n1, 0, 1 << 18, max_factors=64)
    assert text(got) == want.format()
    assert int(got.counts.max()) <= 64


@pytest.mark.parametrize("family,param", FAMILIES[:-1])
@pytest.mark.parametrize("f0,f1", [((1 << 31) - (1 << 18), (1 << 31) + (1 << 18)),
                                   ((1 << 36), (1 << 36) + (1 << 20)),
                                   ((1 << 62) + (1 << 61), (1 << 62) + (1 << 61) + (1 << 13))])
def test_large_primes_vs_oracle(eng, family, param, f0, f1):
    n0, n1 = 1000, 9000
    got = run_gpu(eng, family, param, n0, n1, f0, f1)
    want = O.trial_factor(family, param, n0, n1, f0, f1)
    assert text(got) == want.format()


@pytest.mark.parametrize("family,param", [(O.PROTH, 3), (O.FIBONACCI, 0), (O.TRIBONACCI, 0), (O.SMARANDACHE, 10),
                                          (O.RIESEL_FIXED_N, 777)])
def test_index_tiles_vs_oracle(eng, family, param):
    """Few primes and a long index range: the engine splits each prime's
    range into tiles that jump to their first index."""
    n0, n1 = 7, 120_007
    f0, f1 = 1 << 30, (1 << 30) + 4000
    got = run_gpu(eng, family, param, n0, n1, f0, f1)
    want = O.trial_factor(family, param, n0, n1, f0, f1)
    assert text(got) == want.format()


def test_fibonacci_lucas_n0_zero_quirk(eng):
    # make_state(0) leaves a zero state in the reference: every prime divides every term
    for fam in (O.FIBONACCI, O.LUCAS):
        got = run_gpu(eng, fam, 0, 0, 9000, 1 << 20, (1 << 20) + 200, max_factors=64)
        want = O.trial_factor(fam, 0, 0, 9000, 1 << 20, (1 << 20) + 200, max_factors=64)
        assert text(got) == want.format()


def test_resume_matches_uninterrupted(eng):
    """Resume from a snapshot taken after a middle segment: same result as one pass."""
    fam, param, n0, n1, f0, f1 = O.PROTH, 3, 1, 20001, 1 << 24, 1 << 26
    full = run_gpu(eng, fam, param, n0, n1, f0, f1, seg=1 << 23)
    snaps = []

    def cb(prog, snapshot):
        if snapshot:
            snaps.append((prog.last_prime, buf.counts.copy(), buf.factors.copy()))
            return ctd._native.CTD_CB_ABORT
        return ctd._native.CTD_CB_SNAPSHOT if prog.segment_end >= f0 + 3 * (1 << 23) else 0

    buf = ctd.factors_buffer.empty(n0, n1 - n0, 32)
    with pytest.raises(ctd.CtdError):
        run_gpu(eng, fam, param, n0, n1, f0, f1, seg=1 << 23, buf=buf, cb=cb)
    last, counts, factors = snaps[0]
    resumed = ctd.factors_buffer(n0, 32, counts, factors)
    run_gpu(eng, fam, param, n0, n1, f0, f1, seg=1 << 23, resume=last, buf=resumed)
    assert text(resumed) == text(full)


def test_overflowing_term_keeps_count(eng):
    # more factors than slots: counts keep growing (src/factors_buffer.hpp:110-121)
    got = run_gpu(eng, O.FIBONACCI, 0, 0, 4, 0, 1 << 12, max_factors=8)
    want = O.trial_factor(O.FIBONACCI, 0, 0, 4, 0, 1 << 12, max_factors=8)
    assert got.counts.tolist() == want.counts.tolist()


def test_overflow_semantics_tribonacci_n1(eng):
    """T(1) = 0: every prime divides it and the term overflows its slots.
    Which primes are kept depends on arrival order (in the reference too), so
    parity is: equal counts everywhere, identical lines where nothing
    overflowed, and stored factors that are distinct primes of the range."""
    n0, n1, f0, f1, m = 1, 5001, 1 << 20, (1 << 20) + (1 << 16), 32
    got = run_gpu(eng, O.TRIBONACCI, 0, n0, n1, f0, f1, max_factors=m)
    want = O.trial_factor(O.TRIBONACCI, 0, n0, n1, f0, f1, max_factors=m)
    assert got.counts.tolist() == want.counts.tolist()
    primes = set(O.sieve(f0, f1).tolist())
    gl, wl = got.to_factoring_results(), want.factor_lists()
    for i, c in enumerate(got.counts.tolist()):
        if c <= m:
            assert gl[i] == wl[i]
        else:
            assert len(set(gl[i])) == m and set(gl[i]) <= primes


@pytest.mark.parametrize("family,n0,n1", [(O.FIBONACCI, 1, 2501), (O.LUCAS, 3, 1003), (O.TRIBONACCI, 2, 1502),
                                          (O.FIBONACCI, 7, 40)])
def test_linear_recurrences_across_the_lazy_block_limit(eng, family, n0, n1):
    """Primes on both sides of 2^40, where the lazily reduced blocks give way to
    the modular-add walk; index ranges with and without a partial last block."""
    f0, f1 = (1 << 40) - (1 << 17), (1 << 40) + (1 << 17)
    got = run_gpu(eng, family, 0, n0, n1, f0, f1)
    want = O.trial_factor(family, 0, n0, n1, f0, f1, max_factors=32)
    assert got.counts.tolist() == want.counts.tolist()
    assert text(got) == want.format()


@pytest.mark.parametrize("family,param", [(O.PROTH, 1279), (O.RIESEL, 3), (O.MERSENNE, 0), (O.PROTH_FIXED_N, 77),
                                          (O.RIESEL_FIXED_N, 5)])
def test_baby_step_blocks_tail_and_short_ranges(eng, family, param):
    """Index ranges of 1..200 terms (below, at and above two 32-term blocks) so
    the block walk, its tail and the term-by-term walk all run."""
    f0, f1 = (1 << 33), (1 << 33) + (1 << 18)
    for n0, n1 in [(5, 6), (5, 68), (5, 69), (5, 70), (1000, 1063), (1000, 1200)]:
        got = run_gpu(eng, family, param, n0, n1, f0, f1)
        want = O.trial_factor(family, param, n0, n1, f0, f1, max_factors=32)
        assert text(got) == want.format(), (n0, n1)


def test_two_contexts_sieve_and_run(eng):
    """A second context on the same device (a device switch in between) sieves
    and runs like the first: per-device kernel attributes are set per call."""
    import torch

    other = ctd.Engine(0)
    try:
        lo, hi = (1 << 33) + 12345, (1 << 33) + (1 << 22)
        torch.cuda.set_device(0)
        assert np.array_equal(other.sieve(lo, hi), eng.sieve(lo, hi))
        a = run_gpu(other, O.PROTH, 3, 1, 5001, lo, hi)
        b = run_gpu(eng, O.PROTH, 3, 1, 5001, lo, hi)
        assert text(a) == text(b)
    finally:
        other.close()


# ------------------------------------------- power-residue classes, fixed-n solve
DOUBLING = [(O.PROTH, 3), (O.PROTH, 2718281828459), (O.RIESEL, 999_999), (O.RIESEL, 1), (O.MERSENNE, 0),
            (O.PROTH, 1 << 20), (O.RIESEL, 3 * 5 * 7 * 11 * 13)]


@pytest.mark.parametrize("family,param", DOUBLING)
@pytest.mark.parametrize("f0,f1", [(0, 1 << 16), ((1 << 31) - (1 << 17), (1 << 31) + (1 << 17)),
                                   ((1 << 40) + (1 << 30), (1 << 40) + (1 << 30) + (1 << 16))])
def test_doubling_classes_vs_oracle(eng, family, param, f0, f1):
    """Index ranges long enough for the power-residue classes (12000 terms):
    small primes with dense hits, primes around 2^31 and above 2^40."""
    n0, n1 = 5, 12005
    got = run_gpu(eng, family, param, n0, n1, f0, f1, max_factors=64)
    want = O.trial_factor(family, param, n0, n1, f0, f1, max_factors=64)
    assert text(got) == want.format()


@pytest.mark.parametrize("family,param", DOUBLING[:5])
def test_doubling_classes_on_short_ranges(eng, family, param):
    """The classified walk forced onto ranges of 1..300 terms (classes with
    fewer terms than two blocks, partial blocks, the tail)."""
    t = eng.get_tuning(family)
    t["classify_min"] = 1
    eng.set_tuning(family, t)
    try:
        f0, f1 = (1 << 33), (1 << 33) + (1 << 18)
        for n0, n1 in [(5, 6), (5, 40), (5, 69), (1000, 1063), (1000, 1300), (7, 2100)]:
            got = run_gpu(eng, family, param, n0, n1, f0, f1)
            want = O.trial_factor(family, param, n0, n1, f0, f1, max_factors=32)
            assert text(got) == want.format(), (n0, n1)
        got = run_gpu(eng, family, param, 3, 2503, 0, 1 << 14, max_factors=64)
        want = O.trial_factor(family, param, 3, 2503, 0, 1 << 14, max_factors=64)
        assert text(got) == want.format()
    finally:
        eng.set_tuning(family, None)


@pytest.mark.parametrize("family,param,n0,n1,f0,f1", [
    (O.RIESEL, 999_999, 1, 30001, 1 << 33, (1 << 33) + (1 << 27)),
    (O.MERSENNE, 0, 10000, 60000, 1 << 35, (1 << 35) + (1 << 27)),
    (O.PROTH, 1279, 20000, 40000, 1 << 38, (1 << 38) + (1 << 27)),
    (O.PROTH_FIXED_N, 20000, 1, 50001, 1 << 31, (1 << 31) + (1 << 27)),
    (O.RIESEL_FIXED_N, 1234, 1, 70001, 1 << 36, (1 << 36) + (1 << 27)),
    (O.PROTH_FIXED_N, 7, 0, 30000, 0, 1 << 20),
])
def test_default_forms_against_the_walk(eng, family, param, n0, n1, f0, f1):
    """Power-residue classes (doubling) and the closed-form solve (fixed n)
    against the term-by-term walk on ranges too large for the CPU oracle."""
    def run(variant):
        eng.set_tuning(family, None)
        t = eng.get_tuning(family)
        t["variant"] = variant
        eng.set_tuning(family, t)
        try:
            return text(run_gpu(eng, family, param, n0, n1, f0, f1, max_factors=64))
        finally:
            eng.set_tuning(family, None)

    fast, walk = run(0), run(1)
    assert fast == walk
