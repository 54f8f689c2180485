"""The rank-of-apparition path of the Fibonacci/Lucas residue kernel
(run_fibonacci_rank in cutrialdive_gb300/csrc/ctd_residue.cu), restated step
by step in Python and checked against direct walks of the recurrences
(fibonacci.hpp:245-285, lucas.hpp:394-418): for a prime p other than 2 and 5,
p | F(n) iff a(p) | n with a(p) | p - (5/p), and p | L(n) iff a(p) is even and
n is an odd multiple of a(p)/2.  The restatement follows the kernel's order
of work -- powers of 2 first, trial division by odd primes up to e - 1 with
the early stop once q^2 exceeds the cofactor, F(S) = 0 as the gate, the order
reduction from the largest prime down with the early rejection -- so a slip
in any of those steps shows here, without a GPU."""
import random

import pytest


def fib_pair(k, p):
    """(F(k), F(k+1)) mod p by the doubling identities."""
    a, b = 0, 1
    for bit in bin(k)[2:] if k else "":
        c = a * ((2 * b - a) % p) % p
        d = (a * a + b * b) % p
        a, b = (d, (c + d) % p) if bit == "1" else (c, d)
    return a, b


def odd_primes(limit):
    sieve = bytearray([1]) * limit
    sieve[0:2] = b"\0\0"
    for i in range(2, int(limit ** 0.5) + 1):
        if sieve[i]:
            sieve[i * i::i] = bytearray(len(sieve[i * i::i]))
    return [i for i in range(3, limit, 2) if sieve[i]]


TABLE = odd_primes(1 << 16)


def rank_hits(fibonacci, p, s, e):
    """Indices n in [s, e) with p | F(n) (or L(n)), the kernel's way."""
    D = p - 1 if p % 5 in (1, 4) else p + 1
    bmax = e - 1
    v2 = (D & -D).bit_length() - 1
    R, S, fac = D >> v2, 1 << v2, []
    qs = [q for q in TABLE if q <= bmax]
    i = 0
    while i < len(qs):
        for q in qs[i:i + 64]:
            if R % q == 0:
                v = 0
                while R % q == 0:
                    R //= q
                    S *= q
                    v += 1
                fac.append((q, v))
        i += 64
        if i < len(qs) and qs[i] ** 2 > R:
            break
    if 1 < R <= bmax:
        fac.append((R, 1))
        S *= R
    if fib_pair(S, p)[0]:
        return []
    amax = bmax if fibonacci else 2 * bmax
    a, fixed = S, 1
    for q, v in list(reversed(fac)) + [(2, v2)]:
        t = 0
        while t < v and fib_pair(a // q, p)[0] == 0:
            a //= q
            t += 1
        for _ in range(t, v):
            if fixed > amax:
                break
            fixed *= q
        if fixed > amax:
            return []
    if fibonacci:
        first = (s + a - 1) // a * a
    else:
        if a & 1:
            return []
        h, r = a >> 1, s % a
        first = s + (h - r if h >= r else a - r + h)
    return list(range(first, e, a))


def walk_hits(fibonacci, p, s, e):
    x, y = (0, 1) if fibonacci else (2, 1)
    out = []
    for n in range(e):
        if n >= s and x % p == 0:
            out.append(n)
        x, y = y, (x + y) % p
    return out


def is_prime(n):
    return n > 1 and all(n % q for q in range(2, int(n ** 0.5) + 1))


SMALL = [p for p in range(3, 1200) if is_prime(p) and p != 5]
rng = random.Random(11)
LARGE = [p for p in (rng.randrange(10 ** 5, 10 ** 7) for _ in range(800)) if is_prime(p) and p != 5][:60]


@pytest.mark.parametrize("fibonacci", [True, False])
@pytest.mark.parametrize("rng_", [(1, 1500), (7, 900), (200, 2500), (1, 60)])
def test_rank_hits_equal_walk(fibonacci, rng_):
    s, e = rng_
    for p in SMALL + LARGE:
        assert rank_hits(fibonacci, p, s, e) == walk_hits(fibonacci, p, s, e), (fibonacci, p, s, e)
