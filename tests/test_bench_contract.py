"""bench.py's reference arm (the CPU restatement of the reference engine,
timed on the host cores) prints one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload", ["proth", "linear", "smarandache"])
def test_reference_arm_json_line(workload):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--workload", workload, "--cpu-seconds", "0.2"],
                         capture_output=True, text=True, timeout=300, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "updates/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"]


def test_restricted_factor_files_match_reference_fixtures():
    """bench.py checks batched and served results against the reference
    engine's files of a smaller TF range by dropping the primes above it:
    the oracle's result on a wider range, cut that way, reproduces the
    reference file of the narrower one."""
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    from cutrialdive_gb300 import factors_buffer

    ref = bench.reference_mix_files()
    assert len(ref) == 264
    bound, text = ref["served159"]
    import golden_util

    with open(os.path.join(ROOT, "tests", "golden", "golden_job_mixes.json")) as fh:
        a = golden_util.parse_args(json.load(fh)["served159"]["args"])
    wide = oracle.trial_factor(a["family"], a["param"], a["n0"], a["n1"], a["f0"], a["f1"] + (1 << 20), 32)
    buf = factors_buffer(a["n0"], 32, wide.counts, wide.factors)
    assert bench.restricted_text(buf, bound) == text
