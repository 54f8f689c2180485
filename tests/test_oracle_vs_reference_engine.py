"""The oracle against the factor files written by the reference's own CPU
engine (tests/golden/golden_factor_files.json, made by
tests/golden/make_golden_factor_files.py from oracle/_ref).  Byte-exact."""
import os

import pytest

import oracle as O
from golden_util import expand, parse_args, sha256

# cases whose CPU run takes more than a few seconds; covered on the GPU and
# by the full run in tests/golden/make_golden_factor_files.py
HEAVY = {"smarandache10_n10-1001_tf28", "proth3_n1-100001_p2^32+2^24", "smarandache10_n990-5000_p2^29-2^30",
         "tribonacci_n2-50001_p2^34+2^22", "mersenne_n1000-21000_p2^24+2^22"}


def cases():
    import json

    path = os.path.join(os.path.dirname(__file__), "golden", "golden_factor_files.json")
    with open(path) as fh:
        data = json.load(fh)
    return [(k, v) for k, v in data.items()]


@pytest.mark.parametrize("name,g", cases(), ids=[c[0] for c in cases()])
def test_oracle_reproduces_reference_engine(name, g):
    if name in HEAVY and not os.environ.get("CTD_SLOW_TESTS"):
        pytest.skip("heavy CPU case (set CTD_SLOW_TESTS=1)")
    a = parse_args(g["args"])
    want = expand(a["n0"], a["n1"], g["nonempty"])
    assert sha256(want) == g["sha256"]
    got = O.trial_factor(a["family"], a["param"], a["n0"], a["n1"], a["f0"], a["f1"], a["max_factors"])
    assert got.format() == want, name


def scale_fixtures():
    import json

    out = []
    for name in ("golden_scale_slices.json", "golden_job_mixes.json"):
        with open(os.path.join(os.path.dirname(__file__), "golden", name)) as fh:
            out.extend(json.load(fh).items())
    return out


def test_scale_fixtures_rebuild():
    """Every configuration-scale fixture rebuilds to the sha256 of the
    reference engine's file."""
    fx = scale_fixtures()
    assert len(fx) == 64 + 264
    for name, g in fx:
        a = parse_args(g["args"])
        assert sha256(expand(a["n0"], a["n1"], g["nonempty"])) == g["sha256"], name


def cheap_mix_jobs(count=12):
    fx = [(n, g) for n, g in scale_fixtures() if n.startswith(("batched", "served"))]

    def cost(item):
        a = parse_args(item[1]["args"])
        return (a["n1"] - a["n0"]) * (a["f1"] - a["f0"]) / a["f0"].bit_length() * (8 if a["family"] == 3 else 1)

    fx.sort(key=cost)
    return fx[:count]


@pytest.mark.parametrize("name,g", cheap_mix_jobs(), ids=[c[0] for c in cheap_mix_jobs()])
def test_oracle_reproduces_mix_jobs(name, g):
    """The oracle against the reference engine on the cheapest sampled jobs of
    the batched and serving mixes (all families of the mixes occur)."""
    a = parse_args(g["args"])
    want = expand(a["n0"], a["n1"], g["nonempty"])
    got = O.trial_factor(a["family"], a["param"], a["n0"], a["n1"], a["f0"], a["f1"], a["max_factors"])
    assert got.format() == want, name
