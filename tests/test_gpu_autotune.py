"""Autotuner (ctd_autotune / ctd_set_tuning): the chosen launch shape and
tiling change only the speed; results stay equal to the oracle's."""
import pytest

import cutrialdive_gb300 as ctd
import oracle as O

pytestmark = pytest.mark.gpu


def run(eng, job):
    buf = ctd.factors_buffer.empty(job.n0, job.n1 - job.n0, job.max_factors)
    eng.run_plain(job, buf)
    return str(buf.to_factoring_results())


@pytest.mark.parametrize("case", [
    (O.PROTH, 3, 1, 20001, 1 << 32, (1 << 32) + (1 << 22)),
    (O.SMARANDACHE, 10, 500, 2500, 1 << 30, (1 << 30) + (1 << 22)),
    (O.TRIBONACCI, 0, 2, 6002, 1 << 20, 1 << 22),
    (O.RIESEL_FIXED_N, 777, 3, 9003, 1 << 31, (1 << 31) + (1 << 22)),
    (O.SMARANDACHE, 7, 1, 3001, 3, 1 << 20),
])
def test_autotune_keeps_results(eng, case):
    fam, param, n0, n1, f0, f1 = case
    job = ctd.CtdJob(fam, 32, param, n0, n1, f0, f1)
    want = O.trial_factor(fam, param, n0, n1, f0, f1, 32).format()
    bits = max(3, f0).bit_length()
    try:
        best = eng.autotune(job, budget_s=1.0)
        assert 32 <= best["block_size"] <= 256 and best["block_size"] % 32 == 0
        assert best["ctas_per_sm"] >= 0 and best["items_per_thread"] > 0 and best["min_tile"] > 0
        assert best["segment_log2"] in (26, 28, 30)
        # kept for the family at the width of the job's first prime only
        assert eng.get_tuning_for(fam, bits) == best
        assert eng.get_tuning_for(fam, bits + 1) == eng.get_tuning(fam)
        assert run(eng, job) == want
        eng.set_tuning_for(fam, bits, None)
        # an extreme but valid shape, and every step form: still the same factors
        for variant in (0, 1, 2):
            eng.set_tuning(fam, {"block_size": 64, "ctas_per_sm": 1, "items_per_thread": 32, "min_tile": 1024,
                                 "segment_log2": 22, "variant": variant})
            assert run(eng, job) == want, variant
    finally:
        eng.set_tuning(fam, None)
        eng.set_tuning_for(fam, bits, None)
    assert eng.get_tuning(fam)["segment_log2"] == 26


@pytest.mark.parametrize("family,param", [(O.PROTH, 3), (O.MERSENNE, 0), (O.RIESEL, 999_999)])
def test_classes_on_and_off_same_factors(eng, family, param):
    """classify_min (the autotuner's power-residue switch) and refine_q (the
    rare primes of the classes' refinement: none, up to 31, all) change only
    the speed."""
    n0, n1, f0, f1 = 1, 9001, (1 << 33) - (1 << 21), (1 << 33) + (1 << 21)
    job = ctd.CtdJob(family, 32, param, n0, n1, f0, f1)
    outs = []
    try:
        for cm, rq in ((1, 0), (1, 1), (1, 31), (0xFFFFFFFF, 0)):
            t = eng.get_tuning(family)
            t["classify_min"] = cm
            t["refine_q"] = rq
            eng.set_tuning_for(family, f0.bit_length(), t)
            eng.set_tuning_for(family, f1.bit_length(), t)
            outs.append(run(eng, job))
    finally:
        eng.set_tuning_for(family, f0.bit_length(), None)
        eng.set_tuning_for(family, f1.bit_length(), None)
    want = O.trial_factor(family, param, n0, n1, f0, f1, 32).format()
    assert all(o == want for o in outs)


def test_set_tuning_rejects_bad_values(eng):
    for bad in ({"block_size": 48}, {"block_size": 512}, {"items_per_thread": 0}, {"segment_log2": 50}, {"variant": 3}):
        t = {"block_size": 256, "ctas_per_sm": 0, "items_per_thread": 8, "min_tile": 4096, "segment_log2": 0}
        t.update(bad)
        with pytest.raises(ctd.CtdError):
            eng.set_tuning(O.PROTH, t)
    assert eng.get_tuning(O.PROTH)["block_size"] == 256
