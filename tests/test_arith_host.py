"""The residue kernels' modular arithmetic (ctd_arith.cuh), run on the host
from the same source and checked against Python integers: Montgomery set-up
(R mod p, R^2 mod p), 2^e by squaring and doubling, the mixed
Montgomery-times-plain product that yields k*2^e mod p, and the
division-free floor(2^64/p) and Shoup quotients floor(w 2^64/p); and the
Smarandache jump to Sm_b(s) mod p (ctd_smarandache.cuh)."""
import os
import random
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("arith") / "arith_host_check")
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "arith_host_check.cu")])
    return exe


def cases():
    rnd = random.Random(5)
    out = [(3, 0, 1), (3, 1, 2), (5, 64, 7), (2**61 - 1, 100000, 3), (2**64 - 59, 12345, 2**64 - 1),
           (2**63 + 29, 1, 999999), ((1 << 32) + 15, 99999, 3)]
    for bits in (8, 20, 31, 32, 33, 34, 35, 36, 38, 39, 40, 50, 62, 63, 64):
        for _ in range(25):
            p = rnd.getrandbits(bits) | 1 | (1 << (bits - 1))
            if p < 3:
                continue
            out.append((p, rnd.randrange(0, 1 << rnd.choice((1, 8, 17, 40, 64))), rnd.getrandbits(64)))
    return out


def test_montgomery_setup_and_pow2(checker):
    cs = cases()
    inp = "".join(f"{p} {e} {k}\n" for p, e, k in cs)
    res = subprocess.run([checker], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    R = 1 << 64
    for (p, e, k), line in zip(cs, res):
        one, r2, pw, kpw, tok, mu, sh, npw, nmul, sh_any, small, sh_small = map(int, line.split())
        assert one == R % p, (p, e)
        assert r2 == R * R % p, (p, e)
        assert pw == pow(2, e, p), (p, e)
        assert kpw == k * pow(2, e, p) % p, (p, e, k)
        assert tok == k % p, (p, k)
        assert mu == R // p, p
        assert sh == (k % p) * R // p, (p, k)
        assert sh_any == sh, (p, k)  # the quotient without r2
        assert sh_small == small * R // p, (p, small)
        if p < 1 << 40:  # the narrow Montgomery product
            assert npw == pow(2, e, p), (p, e)
            assert nmul == (k % p) * ((k >> 7) % p) * pow(R, -1, p) % p, (p, k)


def smarandache_mod(b: int, s: int, p: int) -> int:
    """Sm_b(s) mod p by the definition: concatenate 1 .. s in base b."""
    x, pw = 0, b
    for m in range(1, s + 1):
        while pw <= m:
            pw *= b
        x = (x * pw + m) % p
    return x


@pytest.fixture(scope="module")
def sm_checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("smjump") / "smarandache_host_check")
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "smarandache_host_check.cu")])
    return exe


def test_smarandache_jump_closed_form_and_doubling(sm_checker):
    """The kernel's jump to Sm_b(s) mod p: closed-form class jumps with one
    simultaneous inversion, and the doubling jumps, both against Python."""
    from sympy import prevprime, randprime

    rnd = random.Random(9)
    cases = [(3, 10, 1), (5, 2, 0), (7, 10, 9), (11, 10, 10), (13, 10, 100), (101, 2, 1000),
             # p | b^d - 1 (a class multiplier = 1 mod p): 3 | 10 - 1, 7 | 2^3 - 1, 11 | 10^2 - 1
             (3, 10, 50), (7, 2, 300), (11, 10, 1200), (9901, 10, 5000),
             (prevprime(1 << 62), 16, 3000), (prevprime(1 << 64), 10, 2000), (prevprime(1 << 30), 2, 40000)]
    for _ in range(40):
        p = randprime(3, 1 << rnd.choice([8, 20, 28, 30, 31, 34, 40, 48]))
        cases.append((p, rnd.randrange(2, 65), rnd.randrange(0, 3000)))
    inp = "".join(f"{p} {b} {s}\n" for p, b, s in cases)
    out = subprocess.run([sm_checker], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    for (p, b, s), line in zip(cases, out):
        closed, dbl, chosen, small = map(int, line.split())
        want = smarandache_mod(b, s, p)
        assert closed == want, (p, b, s)
        assert dbl == want, (p, b, s)
        assert chosen == want, (p, b, s)
        assert small == want, (p, b, s)  # the 32-bit Montgomery form (p < 2^31)
