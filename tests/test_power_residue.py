"""The doubling families' power-residue classes (ctd_powres.cuh), run on the
host from the kernel's own source and checked with Python integers: every
n with 2^-n = wt (mod p) -- a zero of k*2^n-+1 or 2^n-1 -- lies in the class
n = r (mod M) the kernel walks, both the class of the 2^3-, 3rd-, 5th- and
7th-power characters and its refinement by the smallest rare prime 11..127
dividing p - 1 and by the 9th-power character, and a prime classed as dividing no term (M = 0) really divides none
(wt is outside the subgroup generated by 2)."""
import os
import random
import shutil
import subprocess

import pytest

sympy = pytest.importorskip("sympy")

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("powres") / "powres_host_check")
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "powres_host_check.cu")])
    return exe


def classes(checker, cases):
    inp = "".join(f"{p} {w}\n" for p, w in cases)
    out = subprocess.run([checker], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    return [tuple(map(int, line.split())) for line in out[:len(cases)]]


def both(got):
    """(M, r) of the base class and of the refined one, for each case"""
    assert all(g[6] == 1 for g in got), "narrow Montgomery or pattern classes differ"
    return [((M, r), (M2, r2)) for M, r, M2, r2, _, _, _ in got]


def test_quadratic_screen_and_jacobi(checker):
    """The Jacobi symbol of the screen equals sympy's, and every prime the
    quadratic screen excludes is one the classes find dividing no term."""
    rnd = random.Random(7)
    cases = []
    for p in primes_for_test():
        for w in {1, 2, p - 1, p - 2, p - 3 % p if p > 3 else 1, rnd.randrange(1, p), rnd.randrange(1, p)}:
            if 0 < w < p:
                cases.append((p, w))
    cases += [(p, w) for p in map(int, sympy.primerange(3, 200)) for w in range(1, p)]
    got = classes(checker, cases)
    screened = 0
    assert all(g[6] == 1 for g in got), "narrow Montgomery or pattern classes differ"
    for (p, w), (M, _, M2, _, x, jac, _) in zip(cases, got):
        assert jac == sympy.jacobi_symbol(w, p), (p, w, jac)
        if x:
            screened += 1
            assert M == 0 and M2 == 0, (p, w)
            assert p % 8 in (1, 7) and jac == -1, (p, w)
        else:
            assert not (p % 8 in (1, 7) and jac == -1), (p, w)
    assert screened > len(cases) // 8


def primes_for_test():
    rnd = random.Random(11)
    ps = [3, 5, 7, 11, 13, 17, 31, 41, 43, 97, 113, 193, 211, 257, 421, 631, 641, 1009, 2017, 65537, 3 * 2**30 + 1,
          15 * 2**27 + 1, 7 * 2**26 + 1, 2**31 - 1, 1000000007, 2**32 + 15]
    # primes with p - 1 divisible by large powers of 2 and by 3 * 5 * 7
    for m in (2**10 * 105, 2**8 * 105, 105, 64 * 3, 64 * 35, 11 * 13 * 105, 8 * 17 * 19, 23 * 29 * 31, 37 * 41,
              43 * 47 * 8, 53 * 59 * 61, 61 * 11, 67 * 71 * 2, 73 * 79, 83 * 89 * 4, 97 * 101, 103 * 107 * 8,
              109 * 113, 127 * 6, 2**6 * 9, 2 * 27 * 5, 4 * 81 * 7, 9 * 11 * 35):
        k = rnd.randrange(1, 2**22)
        while len([q for q in ps if q % m == 1]) < 8:
            if sympy.isprime(k * m + 1):
                ps.append(k * m + 1)
            k += 1
    while len(ps) < 260:
        bits = rnd.choice((12, 17, 24, 31, 33, 34))
        q = sympy.nextprime(rnd.getrandbits(bits) | (1 << (bits - 1)))
        ps.append(int(q))
    return ps


def test_every_zero_lies_in_the_class(checker):
    rnd = random.Random(3)
    cases = []
    for p in primes_for_test():
        for w in {1, p - 1, p - 3 % p if p > 3 else 1, rnd.randrange(1, p), rnd.randrange(1, p)}:
            if 0 < w < p:
                cases.append((p, w))
    got = both(classes(checker, cases))
    skipped = refined = 0
    for (p, w), cls in zip(cases, got):
        h = pow(2, -1, p)
        order = int(sympy.n_order(2, p))
        member = pow(w, order, p) == 1  # w in <2^-1> = <2>
        (M0, r0), (M2, r2) = cls
        # the classes of 2^3, 3, 5, 7 divide 420 (where 8 | p - 1, 2 is a
        # quadratic residue: the 2-part is at most 4), so the refinement's
        # M q stays below 420 * 127 < 2^16 with no check
        assert M0 == 0 or 420 % M0 == 0, (p, w, M0)
        if M0 and M2:
            assert M2 % M0 == 0 and r2 % M0 == r0, (p, w, cls)  # a sub-class
            refined += M2 > M0
        elif M0:
            refined += 1
        else:
            assert M2 == 0, (p, w, cls)
        for M, r in cls:
            if M == 0:
                assert not member, (p, w)
                skipped += 1
                continue
            assert 0 <= r < M <= 65535 and order % M == 0, (p, w, M, r)
            if member:
                n = int(sympy.discrete_log(p, w, h))
                assert pow(h, n, p) == w
                assert n % M == r, (p, w, M, r, n)
    assert skipped > 0 and refined > 20, (skipped, refined)


def test_largest_classes_fit_16_bits(checker):
    """Primes p = 1 (mod 840 * 127), where the classes of 2^3, 3, 5, 7 reach
    M = 420 and the refinement by q = 127 M = 53340: the walks' item code
    keeps M and r in 16 bits each, and every zero still lies in the class."""
    rnd = random.Random(17)
    ps, k = [], 1
    while len(ps) < 40:
        if sympy.isprime(k * 840 * 127 + 1):
            ps.append(k * 840 * 127 + 1)
        k += 1
    cases = [(p, w) for p in ps for w in (p - 3, rnd.randrange(1, p), rnd.randrange(1, p))]
    got = both(classes(checker, cases))
    assert max(M0 for (M0, _), _ in got) == 420
    assert max(M2 for _, (M2, _) in got) == 420 * 127
    for (p, w), cls in zip(cases, got):
        h = pow(2, -1, p)
        member = pow(w, int(sympy.n_order(2, p)), p) == 1
        n = int(sympy.discrete_log(p, w, h)) if member else None
        for M, r in cls:
            assert 0 <= r < max(M, 1) and M <= 65535, (p, w, M, r)
            if M:
                assert n is None or n % M == r, (p, w, M, r, n)
            else:
                assert not member, (p, w)


def test_small_primes_exhaustively(checker):
    """Every prime below 600 and every target: the class holds all zeros of
    one full period, and M = 0 exactly when there are none."""
    cases = [(p, w) for p in map(int, sympy.primerange(3, 600)) for w in range(1, p)]
    got = both(classes(checker, cases))
    for (p, w), cls in zip(cases, got):
        h = pow(2, -1, p)
        order = int(sympy.n_order(2, p))
        zeros = [n for n in range(order) if pow(h, n, p) == w]
        for M, r in cls:
            if M == 0:
                assert zeros == [], (p, w)
            else:
                assert all(n % M == r for n in zeros), (p, w, M, r, zeros)


def test_class_keeps_a_small_fraction_of_terms(checker):
    """Proth k = 3 (wt = -3) over primes near 2^33: the walked fraction,
    sum of 1/M over primes with a class, is near 0.15 of the terms."""
    rnd = random.Random(1)
    ps = []
    x = 2**33 + rnd.getrandbits(30)
    while len(ps) < 3000:
        x = int(sympy.nextprime(x))
        ps.append(x)
    raw = classes(checker, [(p, p - 3) for p in ps])
    # the quadratic screen takes out about a quarter of the primes (of the
    # 43 % that divide no term)
    assert 0.20 < sum(g[4] for g in raw) / len(ps) < 0.30
    got = both(raw)
    frac = sum(1 / M for (M, _), _ in got if M) / len(ps)
    assert 0.10 < frac < 0.22, frac
    # the rare primes 11..127 take it down by about prod(1 - 1/q) = 0.50
    # (the smallest one of each prime), the 9th-power character by another
    # 11 %: 0.45
    frac2 = sum(1 / M for _, (M, _) in got if M) / len(ps)
    assert 0.38 < frac2 / frac < 0.52, (frac, frac2)
