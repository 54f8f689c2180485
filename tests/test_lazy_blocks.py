"""The lazily reduced blocks of the Fibonacci/Lucas and tribonacci walks
(run_fibonacci / run_tribonacci in cutrialdive_gb300/csrc/ctd_residue.cu).
A block runs on unreduced 64-bit values from states below 3p; after step j
every value is below K_j p, and the step's zero test is "x_lo p^-1 mod 2^32 <
K_j", exact for multiples k p with k < K_j.  The bounds K_j are immediates in
the kernel's PTX; this test reads them from the source and checks that they
follow the recurrence, that the values stay inside 64 bits and inside
Lazy::reduce's range for p < 2^40, and that the test flags every zero of
random blocks (false candidates are allowed, false negatives are not)."""
import os
import random
import re

import pytest

SRC = os.path.join(os.path.dirname(__file__), "..", "cutrialdive_gb300", "csrc", "ctd_residue.cu")


def ptx_bounds(macro):
    text = open(SRC).read()
    return [int(k) for k in re.findall(macro + r'\("%\d", "%\d"(?:, "%\d")?, (\d+)\)', text)]


def expected(order, steps):
    k = [3] * order  # states below 3p
    for _ in range(steps):
        k.append(sum(k[-order:]))
    return k[order:]


@pytest.mark.parametrize("macro, order", [("CTD_LZ_STEP", 2), ("CTD_LZ3_STEP", 3)])
def test_bounds_follow_the_recurrence(macro, order):
    ks = ptx_bounds(macro)
    assert ks, macro
    assert ks == expected(order, len(ks))
    assert ks[-1] * (1 << 40) < 1 << 64  # values stay in 64 bits for p < 2^40
    assert ks[-1] < 1 << 31  # Lazy::reduce takes x < 2^(floor(log2 p) + 32)


@pytest.mark.parametrize("macro, order", [("CTD_LZ_STEP", 2), ("CTD_LZ3_STEP", 3)])
def test_blocks_stay_in_bounds_and_flag_every_zero(macro, order):
    ks = ptx_bounds(macro)
    rng = random.Random(order)
    for _ in range(300):
        p = rng.randrange(1 << 33, 1 << 40) | 1
        pinv = pow(p, -1, 1 << 32)
        # values of a block from random states below 3p stay below K_j p
        vals = [rng.randrange(3 * p) for _ in range(order)]
        for kj in ks:
            x = sum(vals[-order:])
            assert x < kj * p
            vals.append(x)
        # every multiple k p with k < K_j passes step j's test
        for kj in ks:
            for k in (0, 1, kj - 1, rng.randrange(kj)):
                x = k * p
                assert (x & 0xFFFFFFFF) * pinv % (1 << 32) < kj
