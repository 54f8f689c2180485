"""The cutrialdive command-line drop-in: flags, messages, exit codes, values
(CPU), and end-to-end factor files / checkpoint resume (GPU)."""
import os
import subprocess

import numpy as np
import pytest

import cutrialdive_gb300 as ctd
from cutrialdive_gb300._build import CLI
from golden_util import expand, parse_args

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cli(*args, cwd=None, timeout=600):
    if not os.path.exists(CLI):
        from cutrialdive_gb300 import _build

        _build.build_all()
    return subprocess.run([CLI, *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=timeout)


# -------------------------------------------------------------- CPU side
def test_usage_help_version():
    r = cli()
    assert r.returncode == 1 and "cutrialdive ( --version" in r.stderr
    r = cli("--help")
    assert r.returncode == 0 and "--max-factors-per-number" in r.stdout
    r = cli("--version")
    assert r.returncode == 0 and r.stdout.startswith("cutrialdive version 1.2.0")


@pytest.mark.parametrize("args,message", [
    ("-s 1", "Invalid command line, option --num-seq must come first"),
    ("--num-seq foo -s 1", "Invalid number sequence id `foo'"),
    ("--num-seq proth, -s 1", "Invalid value for option --num-seq"),
    ("--num-seq proth,3 -s 1", "Missing mandatory option"),
    ("--num-seq proth,3 -s 1 --tf-bits 65", "The value of option --tf-bits must be an integer between 0 and 64"),
    ("--num-seq proth,3 -s 1 --tf-bits 10 --segment-bits 64",
     "value of option --segment-bits must be an integer in range [0, 63]"),
    ("--num-seq proth,3 -s 1 --tf-bits 10 --segment-bits 20 --segment-length 5",
     "Invalid command line, --segment-length is not allowed when --segment-bits is present"),
    # the check sits after the range flags in the parse loop (src/command_line.cpp:337-340),
    # so it fires on the next flag that reaches it
    ("--num-seq proth,3 -s 1 --tf-bits 10 --tf-start 3 --no-progress", "Mixing --tf-bits with --tf-start and --tf-end"),
    ("--num-seq proth,3 -s 1 --tf-bits 10 --output", "Missing value for option --output"),
    ("--num-seq proth,3 -s 1 --tf-bits 10 --verbosity 5", "Invalid value for option --verbosity"),
    ("--checkpoint-period 5 --num-seq proth,3", "Invalid command line, option --checkpoint-period is unexpected"),
    ("--num-seq proth,x -s 1 -e 5 --tf-bits 10", "Missing or invalid k value `x' in Proth number spec"),
    ("--num-seq smarandache,65 -s 1 -e 5 --tf-bits 10", "Base `65' is not supported for Smarandache numbers"),
    ("--num-seq riesel_fixed_n -s 1 -e 5 --tf-bits 10", "Missing or invalid n value `' in Riesel sequence spec"),
])
def test_parse_errors(args, message):
    # src/command_line.cpp:23-373 and src/num_seq_dispatch.hpp:120-170
    r = cli(*args.split())
    assert r.returncode == 1
    assert message in r.stderr


def test_empty_ranges_are_reported_not_run():
    # src/trial_factoring_impl.hpp:380-387
    r = cli("--num-seq", "mersenne", "-s", "5", "-e", "5", "--tf-bits", "10")
    assert r.returncode == 0 and "Range [5, 5[ is empty, no number to process..." in r.stdout
    r = cli("--num-seq", "mersenne", "-s", "5", "--tf-start", "9", "--tf-end", "9")
    assert r.returncode == 0 and "Range [9, 9[ is empty, no prime numbers to divide by..." in r.stdout


def test_unwritable_output_directory_fails_before_any_work(tmp_path):
    """An output file that cannot be created stops the run with exit code 1
    before the device is touched.  (The reference opens the file without
    checking it and, exiting 0, writes the results nowhere; a drop-in should
    not lose a run's results silently.)"""
    out = tmp_path / "no_such_dir" / "factors.txt"
    r = cli("--num-seq", "proth,3", "-s", "1", "-e", "100", "--tf-bits", "20", "--output", out)
    assert r.returncode == 1
    assert f"cannot open file {out}" in r.stderr + r.stdout
    assert not out.parent.exists()


def test_print_expression():
    # tests/smarandache_tests.cpp:311-324 and the per-family printers
    out = lambda *a: cli(*a).stdout.strip()  # noqa: E731
    assert out("--num-seq", "smarandache,10", "--print-expression", "2") == "(10*10^2 - (10 - 1)*2 - 10)/(10 - 1)^2"
    assert out("--num-seq", "smarandache", "--print-expression", "29") == (
        "(((10*10^9 - (10 - 1)^2 - 10)/(10 - 1)^2*(10^2 - 1)^2 + 10^3 - 10 + 1)*10^40 - (10^2 - 1)*29 - 10^2)"
        "/(10^2 - 1)^2")
    assert out("--num-seq", "mersenne", "--print-expression", "7") == "2^7-1"
    assert out("--num-seq", "proth,1279", "--print-expression", "79") == "1279*2^79 + 1"
    assert out("--num-seq", "riesel_fixed_n,5", "--print-expression", "9") == "9*2^5-1"
    assert out("--num-seq", "fibonacci", "--print-expression", "9") == "Expression not available"


def test_print_value():
    out = lambda *a: cli(*a).stdout.strip()  # noqa: E731
    assert out("--num-seq", "smarandache,10", "--print", "12") == "123456789101112"
    assert out("--num-seq", "smarandache,2", "--print", "8") == str(0b110111001011101111000)
    assert out("--num-seq", "proth,3", "--print", "70") == str(3 * 2**70 + 1)
    assert out("--num-seq", "riesel_fixed_n,5", "--print", "0") == "-1"
    assert out("--num-seq", "lucas", "--print", "69") == "263115950957276"
    assert out("--num-seq", "tribonacci", "--print", "201") == "28610320653810477165032088685001500201865067503083660"
    assert out("--num-seq", "fibonacci", "--print", "83") == "99194853094755497"


# -------------------------------------------------------------- GPU side
@pytest.mark.gpu
@pytest.mark.parametrize("name", ["smarandache10_n10-1001_tf28", "proth1279_n0-80_tf16", "lucas_n2-1002_tf16",
                                  "riesel_fixed_n5000_k0-800_tf16"])
def test_cli_factor_file_matches_reference_engine(tmp_path, golden_files, name):
    g = golden_files[name]
    a = parse_args(g["args"])
    out = tmp_path / "factors.txt"
    r = cli(*g["args"].split(), "--no-progress", "--output", out, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert out.read_text() == expand(a["n0"], a["n1"], g["nonempty"])
    assert not (tmp_path / "factors.txt.chkpnt").exists()  # removed after the results are written


@pytest.mark.gpu
def test_cli_resume_from_checkpoint(tmp_path):
    """A checkpoint taken part-way (written by the Python mirror in the
    reference layout) resumes through the CLI to the uninterrupted result."""
    args = ["--num-seq", "riesel,999999", "-s", "1", "-e", "20001", "--tf-start", str(1 << 24), "--tf-end",
            str(1 << 27), "--segment-bits", "24", "--no-progress"]
    full = tmp_path / "full.txt"
    assert cli(*args, "--output", full, cwd=tmp_path).returncode == 0
    part = tmp_path / "part.txt"
    spec = ctd.num_seq_spec(ctd.num_seq_id.riesel, "999999")
    opts = ctd.trial_factoring_options(1, 20001, 1 << 24, 1 << 27, str(part), 32)
    buf = ctd.factors_buffer.empty(1, 20000, 32)
    # the first three segments only
    split = (1 << 24) + (3 << 24)
    ctd.engine(0).run_plain(ctd.make_job(spec, ctd.trial_factoring_options(1, 20001, 1 << 24, split)),
                            buf, segment_length=1 << 24)
    import oracle

    last = int(oracle.sieve(split - 4096, split)[-1])
    ctd.write_checkpoint(str(part) + ".chkpnt", spec, opts, last, buf)
    r = cli("--resume", str(part) + ".chkpnt", "--no-progress", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Resuming at the smallest prime > %d." % last in r.stdout
    assert part.read_text() == full.read_text()
    assert not os.path.exists(str(part) + ".chkpnt")


@pytest.mark.gpu
def test_cli_writes_periodic_checkpoints(tmp_path):
    out = tmp_path / "o.txt"
    r = cli("--num-seq", "proth,3", "-s", "1", "-e", "30001", "--tf-start", str(1 << 30), "--tf-end",
            str((1 << 30) + (1 << 27)), "--segment-bits", "22", "--checkpoint-period", "0", "--output", out,
            "--no-progress", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Checkpoint file will be written to `%s.chkpnt' (period is 0s)." % out in r.stdout
    assert out.exists() and not (tmp_path / "o.txt.chkpnt").exists()
    assert len(out.read_text().splitlines()) == 30000


@pytest.mark.gpu
def test_cli_autotest():
    r = cli("--autotest")
    assert r.returncode == 0 and "Done" in r.stdout and "Failure" not in r.stderr
