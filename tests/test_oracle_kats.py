"""The CPU oracle against the reference's own known-answer tests.

Tables come from tests/golden/reference_kats.json (extracted from the
reference sources by tests/golden/extract_reference_kats.py); the
REQUIRE-style cases below are transcribed from the cited reference lines.
"""
import hashlib

import numpy as np
import pytest

import oracle as O


# ------------------------------------------------ tests/test_modular.cpp
def test_mu64_table(kats):
    for c in kats["mu64"]:
        assert O.mu64(c["p"]) == c["mu"], c["src"]


def test_mu128_table(kats):
    for c in kats["mu128"]:
        assert O.mu128(c["p"]) == int(c["mu"]), c["src"]


def test_mul128hi_table(kats):
    for c in kats["mul128hi"]:
        assert O.mul128hi(int(c["a"]), int(c["b"])) == int(c["hi"]), c["src"]


def test_modular_propagation_sanity():
    # tests/test_modular.cpp:41-53
    r = 1
    for _ in range(1000):
        r = O.mulmod(r, 10, 101)
    assert r == pow(10, 1000, 101)


# ------------------------------------------------ src/autotests.cpp (sieve)
def test_sieve_known_answers(kats):
    for c in kats["sieve"]:
        primes = O.sieve(c["lo"], c["hi"]).tolist()
        if "expected" in c:
            assert primes == c["expected"], c["src"]
        if "count" in c:
            assert len(primes) == c["count"], c["src"]


def test_sieve_prime_counts():
    # pi(x) values used by the configurations (pinned by sympy and by
    # README.md:138-141 of the reference for the larger ones)
    assert O.sieve(0, 1 << 28).size == 14_630_843
    assert O.sieve(0, 1 << 20).size == 82_025


# ----------------------------------------- 2-by-1 division, src/autotests.cpp:41-132
def test_reciprocal_and_mod2by1():
    rng = np.random.default_rng(7)
    for _ in range(2000):
        d = int(rng.integers(1, 2**63, dtype=np.uint64)) | (1 << 63)
        rnd = O.reciprocal(d)
        assert rnd == ((2**128 - 1) // d) - 2**64
        u1 = int(rng.integers(0, 2**63, dtype=np.uint64)) % d
        u0 = int(rng.integers(0, 2**63, dtype=np.uint64)) * 2 + 1
        assert O.mod2by1(u1, u0, d, rnd) == ((u1 << 64) | u0) % d


def test_modnby1_random():
    rng = np.random.default_rng(11)
    for _ in range(300):
        limbs = rng.integers(0, 2**63, size=int(rng.integers(1, 40)), dtype=np.uint64)
        v = sum(int(x) << (64 * i) for i, x in enumerate(limbs.tolist()))
        d = int(rng.integers(3, 2**63, dtype=np.uint64)) | 1
        assert O.modnby1(limbs, d) == v % d


# --------------------------------------- tests/smarandache_tests.cpp values
def test_smarandache_values(kats):
    for c in kats["smarandache_values"]:
        limbs = O.smarandache_limbs(c["base"], c["n"])
        v = sum(int(x) << (64 * i) for i, x in enumerate(limbs.tolist()))
        nbytes = max(1, (v.bit_length() + 7) // 8)
        assert v.bit_length() == c["bits"], c["src"]
        assert hashlib.sha256(v.to_bytes(nbytes, "little")).hexdigest() == c["sha256_le"], c["src"]


# ------------------------------------------- per-family KATs (REQUIREs)
def r(family, param, n, p):
    return O.init_state(family, param, n, p).r


def test_mersenne_kats():
    # tests/mersenne_tests.cpp:32-68
    assert [O.value_mod_2(O.MERSENNE, 0, n) for n in range(5)] == [0, 1, 1, 1, 1]
    assert all(O.next_value_mod_2(O.MERSENNE, 0, 1, n) == 1 for n in range(6))
    cases = [(21, 7, 0), (21, 127, 0), (35, 31, 0), (37, 3, 1), (257, 3, 1), (257, 5, 1), (257, 7, 3),
             (67, 193707721, 0), (521, 5, 1), (991, 5, 2), (1279, 59, 7),
             (131071, 2**64 - 1, (1 << 63) - 1), (131071, 2**32 - 1, (1 << 31) - 1),
             (61 * 524287, (1 << 61) - 1, 0)]
    for n, d, v in cases:
        assert r(O.MERSENNE, 0, n, d) == v, (n, d)


def test_proth_kats():
    # tests/proth_tests.cpp:99-147
    assert O.value_mod_2(O.PROTH, 78557, 0) == 0
    assert [O.value_mod_2(O.PROTH, 78557, n) for n in (1, 2, 1276481311)] == [1, 1, 1]
    for n, v in [(0, 78558 % 3), (1, 2), (2, 0), (3, 2), (797827, 2), (877532, 0)]:
        assert r(O.PROTH, 78557, n, 3) == v
    for n, v in [(0, 271130 % 5), (1, 4), (2, 2), (3, 3), (4, 0), (6700224, 0), (4924567891, 3)]:
        assert r(O.PROTH, 271129, n, 5) == v
    res = O.residues(O.PROTH, 271129, 6700224, 6700224 + 9, 5)
    assert res[1:] == [4, 2, 3, 0, 4, 2, 3, 0]


def test_riesel_kats():
    # tests/riesel_tests.cpp:176-224
    assert O.value_mod_2(O.RIESEL, 78557, 0) == 0
    for n, v in [(0, 78556 % 3), (1, 0), (2, 1), (3, 0), (797827, 0), (877532, 1)]:
        assert r(O.RIESEL, 78557, n, 3) == v
    for n, v in [(0, 271128 % 5), (1, 2), (2, 0), (3, 1), (4, 3), (6700224, 3), (4924567891, 1)]:
        assert r(O.RIESEL, 271129, n, 5) == v
    res = O.residues(O.RIESEL, 271129, 6700224, 6700224 + 9, 5)
    assert res[1:] == [2, 0, 1, 3, 2, 0, 1, 3]


def test_fibonacci_kats():
    # tests/fibonacci_tests.cpp:41-125
    assert [O.value_mod_2(O.FIBONACCI, 0, n) for n in range(8)] == [0, 1, 1, 0, 1, 1, 0, 1]
    assert [O.value_mod_2(O.FIBONACCI, 0, n) for n in range(29, 34)] == [1, 0, 1, 1, 0]
    assert [O.next_value_mod_2(O.FIBONACCI, 0, rr, n) for rr, n in [(1, 28), (1, 29), (0, 30), (1, 70), (1, 71)]] \
        == [1, 0, 1, 1, 0]
    st = O.init_state(O.FIBONACCI, 0, 1, 11)
    assert (st.s[0], st.s[1]) == (0, 1)
    st = O.init_state(O.FIBONACCI, 0, 11, 11)
    assert (st.s[0], st.s[1]) == (0, 1)
    st = O.init_state(O.FIBONACCI, 0, 64, 13)
    assert (st.s[0], st.s[1]) == (0, 8)
    st = O.init_state(O.FIBONACCI, 0, 40, 89)
    assert (st.s[0], st.s[1], st.r) == (5, 86, 86)
    out = []
    for n in range(40, 45):
        O.step(O.FIBONACCI, 0, n, 89, st)
        out.append(st.r)
    assert out == [2, 88, 1, 0, 1]


def test_lucas_kats():
    # tests/lucas_tests.cpp:167-224
    assert [O.value_mod_2(O.LUCAS, 0, n) for n in range(8)] == [0, 1, 1, 0, 1, 1, 0, 1]
    for n, p, prev, cur in [(1, 11, 2, 1), (11, 11, 2, 1), (64, 13, 3, 8), (104, 97, 86, 79)]:
        st = O.init_state(O.LUCAS, 0, n, p)
        assert (st.s[0], st.s[1]) == (prev, cur), (n, p)
    st = O.init_state(O.LUCAS, 0, 104, 97)
    O.step(O.LUCAS, 0, 104, 97, st)
    assert st.r == 68


def test_tribonacci_kats():
    # tests/tribonacci_tests.cpp:276-341
    assert [O.value_mod_2(O.TRIBONACCI, 0, n) for n in range(8)] == [0, 0, 1, 1, 0, 0, 1, 1]
    assert [O.value_mod_2(O.TRIBONACCI, 0, n) for n in (199, 200, 201, 1000, 1001, 1002, 1003, 1004, 1005, 1006,
                                                         1007)] == [1, 0, 0, 0, 0, 1, 1, 0, 0, 1, 1]
    assert [O.next_value_mod_2(O.TRIBONACCI, 0, rr, n) for rr, n in [(1, 199), (0, 200), (0, 201)]] == [0, 0, 1]
    st = O.init_state(O.TRIBONACCI, 0, 1, 11)
    assert tuple(st.s) == (0, 1, 1)
    st = O.init_state(O.TRIBONACCI, 0, 7, 11)
    assert tuple(st.s) == (2, 2, 0)
    d = (1 << 31) - 1
    st = O.init_state(O.TRIBONACCI, 0, 64, d)
    assert tuple(st.s) == (15832480722303616 % d, 29120472094716576 % d, 53560898629395777 % d)


def test_smarandache_kats():
    # tests/smarandache_tests.cpp:326-422
    assert [O.value_mod_2(O.SMARANDACHE, 10, n) for n in (0, 1, 2, 3, 257, 258)] == [0, 1, 0, 1, 1, 0]
    assert [O.value_mod_2(O.SMARANDACHE, 3, n) for n in (0, 1, 2, 3)] == [0, 1, 1, 0]
    for base in (10, 3):
        rr = O.value_mod_2(O.SMARANDACHE, base, 0)
        for n in range(10000):
            assert rr == O.value_mod_2(O.SMARANDACHE, base, n)
            rr = O.next_value_mod_2(O.SMARANDACHE, base, rr, n)

    def step(base, v, n, p):
        st = O.init_state(O.PEANO, 0, 0, p)  # any state holder
        st.r = v
        O.step(O.SMARANDACHE, base, n, p, st)
        return st.r

    assert [step(3, v, n, 3) for v, n in [(0, 3), (1, 4), (2, 5), (0, 6), (1, 7), (2, 8), (0, 531441)]] \
        == [1, 2, 0, 1, 2, 0, 1]
    assert [step(10, v, n, 5) for v, n in [(0, 10), (1, 11), (2, 12), (3, 13), (4, 14), (4, 99), (0, 100)]] \
        == [1, 2, 3, 4, 0, 0, 1]
    assert step(10, 13, 42, 17) == 0
    assert step(10, 3, 42, 7) == 0
    assert step(10, 115, 42, 7 * 17) == 0
    assert step(10, 31, 42, 449) == 0
    assert step(10, 2, 99, 7) == 0
    assert step(10, 817, 99, 8171) == 0
    assert step(10, 0, 100, 8171) == 101
    assert step(10, 101, 101, 8171) == (1000 * 101 + 102) % 8171
    m31 = (1 << 31) - 1
    assert step(10, 1855760753, 999, m31) == 1201337273
    d = ((1 << 32) - 17) * ((1 << 32) - 5)
    assert step(10, 94664850192674748, 999, d) == 5864558986513650361


# ------------------------------------------- tests/tf_tests.cpp end to end
def test_tf_peano(oracle_lib):
    # tests/tf_tests.cpp:18-67 -- S(n) = n for n in [2956708207, 2956708707), primes < 2^24
    b = O.trial_factor(O.PEANO, 0, 2956708207, 2956708707, 0, 1 << 24, max_factors=1024, threads=4)
    f = b.factor_lists()
    assert len(f) == 500
    assert f[0] == []
    assert f[1] == [2, 43, 4297541]
    assert f[2] == [3, 7, 13, 107, 127, 797]
    assert f[-1] == [2, 7, 4310071]


def test_tf_mersenne(oracle_lib):
    # tests/tf_tests.cpp:70-85
    b = O.trial_factor(O.MERSENNE, 0, 1, 101, 0, 1 << 16, max_factors=1024, threads=4)
    assert b.factor_lists()[97 - 1] == [11447]


def test_tf_proth_1279(oracle_lib):
    # tests/tf_tests.cpp:88-109
    b = O.trial_factor(O.PROTH, 1279, 0, 80, 0, 1 << 16, max_factors=128, threads=4)
    assert b.factor_lists()[79] == [3, 2063]


@pytest.mark.parametrize("family,param", [(O.PROTH, 3), (O.RIESEL, 5), (O.MERSENNE, 0), (O.FIBONACCI, 0),
                                          (O.LUCAS, 0), (O.TRIBONACCI, 0), (O.PROTH_FIXED_N, 300),
                                          (O.RIESEL_FIXED_N, 77), (O.SMARANDACHE, 10), (O.SMARANDACHE, 8)])
def test_residues_match_bigint_definition(family, param):
    """Residues from the restated recurrences equal S(n) mod p computed from
    each family's definition with Python integers (n0 >= 1)."""
    def S(n):
        if family == O.PROTH:
            return param * 2**n + 1
        if family == O.RIESEL:
            return param * 2**n - 1
        if family == O.MERSENNE:
            return 2**n - 1
        if family == O.PROTH_FIXED_N:
            return n * 2**param + 1
        if family == O.RIESEL_FIXED_N:
            return n * 2**param - 1
        if family in (O.FIBONACCI, O.LUCAS, O.TRIBONACCI):
            a, b, c = {O.FIBONACCI: (0, 1, 1), O.LUCAS: (2, 1, 3), O.TRIBONACCI: (0, 0, 1)}[family]
            for _ in range(n):
                if family == O.TRIBONACCI:
                    a, b, c = b, c, a + b + c
                else:
                    a, b = b, a + b
            return a
        v = 0
        for i in range(1, n + 1):
            d, m = 1, i
            while m >= param:
                m //= param
                d += 1
            v = v * param**d + i
        return v

    for p in (3, 5, 101, 65537, 1000003, 4294967311, (1 << 61) - 1):
        n0 = 1 + (p % 7)
        got = O.residues(family, param, n0, n0 + 60, p)
        assert got == [S(n) % p for n in range(n0, n0 + 60)], p
