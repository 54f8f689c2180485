"""Generates the golden factor files from the reference's own CPU engine.

Runs oracle/_ref/cutrialdive_ref -- cutrialdive 1.2.0's CPU build compiled
from its unmodified sources by oracle/build_ref.sh -- on each case below with
--output, and stores the result in golden_factor_files.json:

* the exact command line,
* sha256 of the complete factor file,
* its non-empty lines (terms with at least one factor; every other line is
  "<n> - ").

The full file is reconstructed from that and checked against the sha256, so
the comparison stays byte-exact while the fixture stays small.
Runs only where the reference sources were available to build the engine.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "cutrialdive_ref")

# name -> arguments after the binary (each case lists its --num-seq first)
CASES = {
    # the plain Smarandache configuration in full: Sm(10..1000), primes below 2^28
    "smarandache10_n10-1001_tf28": "--num-seq smarandache,10 -s 10 -e 1001 --tf-bits 28",
    # Proth 3*2^n+1, n = 1..100000, on the first 2^24 of [2^32, 2^34)
    "proth3_n1-100001_p2^32+2^24": "--num-seq proth,3 -s 1 -e 100001 --tf-start 4294967296 --tf-end 4311744512",
    # Fibonacci / Lucas / tribonacci, n = 1..50000: a slice of [2^34, 2^36) and a denser range
    "fibonacci_n1-50001_p2^34+2^22": "--num-seq fibonacci -s 1 -e 50001 --tf-start 17179869184 --tf-end 17184063488",
    "lucas_n1-50001_p2^34+2^22": "--num-seq lucas -s 1 -e 50001 --tf-start 17179869184 --tf-end 17184063488",
    "tribonacci_n2-50001_p2^34+2^22": "--num-seq tribonacci -s 2 -e 50001 --tf-start 17179869184 --tf-end 17184063488",
    "fibonacci_n1-50001_p2^20+2^18": "--num-seq fibonacci -s 1 -e 50001 --tf-start 1048576 --tf-end 1310720",
    "lucas_n1-50001_p2^20+2^18": "--num-seq lucas -s 1 -e 50001 --tf-start 1048576 --tf-end 1310720",
    "tribonacci_n2-50001_p2^20+2^18": "--num-seq tribonacci -s 2 -e 50001 --tf-start 1048576 --tf-end 1310720",
    # the reference's own end-to-end cases (tests/tf_tests.cpp:70-109) and neighbours
    "mersenne_n1-101_tf16": "--num-seq mersenne -s 1 -e 101 --tf-bits 16 --max-factors-per-number 1024",
    "proth1279_n0-80_tf16": "--num-seq proth,1279 -s 0 -e 80 --tf-bits 16 --max-factors-per-number 128",
    "riesel1279_n0-80_tf16": "--num-seq riesel,1279 -s 0 -e 80 --tf-bits 16 --max-factors-per-number 128",
    "riesel271129_n6700224-6700324_tf18": "--num-seq riesel,271129 -s 6700224 -e 6700324 --tf-bits 18",
    "proth_fixed_n1000_k1-801_tf16": "--num-seq proth_fixed_n,1000 -s 1 -e 801 --tf-bits 16",
    "riesel_fixed_n5000_k0-800_tf16": "--num-seq riesel_fixed_n,5000 -s 0 -e 800 --tf-bits 16",
    "proth_fixed_n20000_k1-20001_p2^30+2^20": "--num-seq proth_fixed_n,20000 -s 1 -e 20001 --tf-start 1073741824 --tf-end 1074790400",
    "mersenne_n1000-21000_p2^24+2^22": "--num-seq mersenne -s 1000 -e 21000 --tf-start 16777216 --tf-end 20971520",
    "riesel999999_n1-20001_p2^31-2^31+2^22": "--num-seq riesel,999999 -s 1 -e 20001 --tf-start 2147483648 --tf-end 2151677952",
    # reference quirk: make_state(0) zeroes the state, so every prime is recorded
    "fibonacci_n0-40_tf8": "--num-seq fibonacci -s 0 -e 40 --tf-bits 8 --max-factors-per-number 64",
    "lucas_n0-40_tf8": "--num-seq lucas -s 0 -e 40 --tf-bits 8 --max-factors-per-number 64",
    "fibonacci_n1-1001_tf16": "--num-seq fibonacci -s 1 -e 1001 --tf-bits 16",
    "lucas_n2-1002_tf16": "--num-seq lucas -s 2 -e 1002 --tf-bits 16",
    "tribonacci_n2-1002_tf16": "--num-seq tribonacci -s 2 -e 1002 --tf-bits 16",
    "smarandache2_n1-1001_tf16": "--num-seq smarandache,2 -s 1 -e 1001 --tf-bits 16",
    "smarandache3_n1-1001_tf16": "--num-seq smarandache,3 -s 1 -e 1001 --tf-bits 16",
    "smarandache7_n500-1300_tf17": "--num-seq smarandache,7 -s 500 -e 1300 --tf-bits 17",
    "smarandache16_n1-1001_tf16": "--num-seq smarandache,16 -s 1 -e 1001 --tf-bits 16",
    "smarandache64_n1-1001_tf16": "--num-seq smarandache,64 -s 1 -e 1001 --tf-bits 16",
    "smarandache10_n990-5000_p2^29-2^30": "--num-seq smarandache,10 -s 990 -e 5000 --tf-start 536870912 --tf-end 1073741824",
    "smarandache13_n100-2100_p2^31-2^31+2^24": "--num-seq smarandache,13 -s 100 -e 2100 --tf-start 2147483648 --tf-end 2164260864",
    "smarandache11_n100-400_p2^40+2^16": "--num-seq smarandache,11 -s 100 -e 400 --tf-start 1099511627776 --tf-end 1099511693312",
    # primes above 2^63: the wide (carry-keeping) arithmetic.  The reference's
    # segment loop computes fy + segment_length without overflow protection
    # (src/trial_factoring_impl.hpp:338-341), so ranges within 2^26 of 2^64
    # never terminate there; these stay below 2^64 - 2^27.
    "proth3_n1-3001_p2^63+2^12": "--num-seq proth,3 -s 1 -e 3001 --tf-start 9223372036854775808 --tf-end 9223372036854779904",
    "tribonacci_n2-3001_p2^64-2^27+2^12": "--num-seq tribonacci -s 2 -e 3001 --tf-start 18446744073575333888 --tf-end 18446744073575337984",
    "smarandache10_n1-2001_p2^64-2^27+2^12": "--num-seq smarandache,10 -s 1 -e 2001 --tf-start 18446744073575333888 --tf-end 18446744073575337984",
    "fibonacci_n1-3001_p2^64-2^27+2^12": "--num-seq fibonacci -s 1 -e 3001 --tf-start 18446744073575333888 --tf-end 18446744073575337984",
}


def run_case(args: str, threads: int) -> str:
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "factors.txt")
        cmd = [REF] + args.split() + ["--no-progress", "--threads", str(threads), "--output", out]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, cwd=d, timeout=900)
        return open(out).read()


def sparse(text: str) -> dict:
    lines = [ln for ln in text.splitlines() if not ln.endswith(" - ")]
    return {"sha256": hashlib.sha256(text.encode()).hexdigest(), "lines": len(text.splitlines()),
            "nonempty": lines}


def expand(n0: int, n1: int, nonempty: list) -> str:
    """Rebuild the full factor file from its non-empty lines."""
    by_n = {int(ln.split(" - ", 1)[0]): ln for ln in nonempty}
    return "".join((by_n.get(n, f"{n} - ")) + "\n" for n in range(n0, n1))


def main() -> None:
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/cutrialdive_ref is missing: run oracle/build_ref.sh where the reference is mounted")
    threads = os.cpu_count() or 2
    data = {}
    for name, args in CASES.items():
        t = time.time()
        text = run_case(args, max(threads, 2))  # >= 2 threads: the siever's [start, end) contract
        data[name] = {"args": args, **sparse(text)}
        print(f"{name}: {len(text.splitlines())} lines, {len(data[name]['nonempty'])} with factors, "
              f"{time.time() - t:.1f}s", flush=True)
    with open(os.path.join(HERE, "golden_factor_files.json"), "w") as fh:
        json.dump(data, fh, indent=0)


if __name__ == "__main__":
    main()
