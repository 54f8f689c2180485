"""The per-prime target filter of the baby-step blocks (TargetFilter in
cutrialdive_gb300/csrc/ctd_residue.cu), restated in Python.  Per thread, 32
slots of two 32-bit words: a target's low word t with hash h = t * FILTER_A
mod 2^32 sets bit t mod 32 of slot h >> 27's first word and bit
(h >> 22) mod 32 of its second; a state passes when both bits of its slot
are set (two funnel-shift rotations, which take their amount mod 32).

The kernel's exactness rests on the filter having no false negatives (a
block whose state equals a target must reach the exact compares), and its
speed on the false-pass rate (about E[X^2]/32^2 = 2/1024 for the X ~
Poisson(1) targets of a slot).  Both are checked here on target sets shaped
like the kernel's (target * 2^j mod p for the doubling families, target -
j c for the fixed-n ones)."""
import random

import pytest

A = 0x9E3779B1
M32 = 0xFFFFFFFF


def rot_right(w, by):
    by &= 31
    return ((w >> by) | (w << (32 - by))) & M32


def build(targets):
    slots = [[0, 0] for _ in range(32)]
    for t in targets:
        h = (t * A) & M32
        s = slots[h >> 27]
        s[0] |= 1 << (t & 31)
        s[1] |= 1 << ((h >> 22) & 31)
    return slots


def passes(slots, lo):
    h = (lo * A) & M32
    s = slots[h >> 27]
    return (rot_right(s[0], lo) & rot_right(s[1], h >> 22)) & 1


def doubling_targets(p, wt):
    out, t = [], wt
    for _ in range(32):
        out.append(t & M32)
        t = 2 * t % p
    return out


def fixed_n_targets(p, target, c):
    return [((target - j * c) % p) & M32 for j in range(32)]


@pytest.mark.parametrize("bits", [20, 31, 33, 35, 40, 62])
def test_no_false_negatives_and_rate(bits):
    rng = random.Random(bits)
    passed = tried = 0
    for _ in range(200):
        p = rng.randrange(1 << (bits - 1), 1 << bits) | 1
        for targets in (doubling_targets(p, rng.randrange(p)),
                        fixed_n_targets(p, p - 1, rng.randrange(1, p))):
            slots = build(targets)
            assert all(passes(slots, t) for t in targets)
            for _ in range(500):
                passed += passes(slots, rng.randrange(p) & M32)
                tried += 1
    rate = passed / tried
    # E[X^2] / 1024 for Poisson(1) occupancy; narrow primes (p < 2^32) have
    # fewer distinct low words to collide, so the rate only goes down
    assert rate < 3.0e-3, rate
