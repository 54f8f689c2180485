"""ctypes binding of the C oracle (``libctd_oracle.so``).

TEST INFRASTRUCTURE ONLY: the checker the CUDA path is compared with, and the
timed CPU baseline.  The product never imports this module.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from .build import LIB, build_oracle

MERSENNE, PROTH, RIESEL, SMARANDACHE = 0, 1, 2, 3
FIBONACCI, LUCAS, PROTH_FIXED_N, RIESEL_FIXED_N, TRIBONACCI = 4, 5, 6, 7, 8
PEANO = 256

_u64 = ctypes.c_uint64
_u32 = ctypes.c_uint32
_p64 = ctypes.POINTER(ctypes.c_uint64)
_p32 = ctypes.POINTER(ctypes.c_uint32)


class _Job(ctypes.Structure):
    _fields_ = [("family", _u32), ("max_factors", _u32), ("param", _u64),
                ("n0", _u64), ("n1", _u64), ("f0", _u64), ("f1", _u64)]


class _State(ctypes.Structure):
    _fields_ = [("r", _u64), ("s", _u64 * 3)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = LIB if os.path.exists(LIB) else build_oracle()
        L = ctypes.CDLL(path)
        L.ctdo_mu64.restype = _u64
        L.ctdo_mu64.argtypes = [_u64]
        L.ctdo_mu128.argtypes = [_u64, _p64]
        L.ctdo_mul128hi.argtypes = [_p64, _p64, _p64]
        for name in ("ctdo_mulmod", "ctdo_modpow"):
            getattr(L, name).restype = _u64
            getattr(L, name).argtypes = [_u64, _u64, _u64]
        L.ctdo_reciprocal.restype = _u64
        L.ctdo_reciprocal.argtypes = [_u64]
        L.ctdo_mod2by1.restype = _u64
        L.ctdo_mod2by1.argtypes = [_u64, _u64, _u64, _u64]
        L.ctdo_modnby1.restype = _u64
        L.ctdo_modnby1.argtypes = [_p64, _u64, _u64]
        L.ctdo_sieve.restype = _u64
        L.ctdo_sieve.argtypes = [_u64, _u64, _p64, _u64]
        L.ctdo_check_seq.restype = ctypes.c_int
        L.ctdo_check_seq.argtypes = [_u32, _u64]
        L.ctdo_value_mod_2.restype = _u64
        L.ctdo_value_mod_2.argtypes = [_u32, _u64, _u64]
        L.ctdo_next_value_mod_2.restype = _u64
        L.ctdo_next_value_mod_2.argtypes = [_u32, _u64, _u64, _u64]
        L.ctdo_init.argtypes = [_u32, _u64, _u64, _u64, _p64, _u64, ctypes.POINTER(_State)]
        L.ctdo_step.argtypes = [_u32, _u64, _u64, _u64, ctypes.POINTER(_State)]
        L.ctdo_smarandache_limbs.restype = _u64
        L.ctdo_smarandache_limbs.argtypes = [_u64, _u64, _p64, _u64]
        L.ctdo_trial_factor.restype = ctypes.c_int
        L.ctdo_trial_factor.argtypes = [ctypes.POINTER(_Job), _p32, _p64, _u64, _u64, ctypes.c_int]
        L.ctdo_residues.restype = ctypes.c_int
        L.ctdo_residues.argtypes = [ctypes.POINTER(_Job), _p64, _u64, _p32, _p64, ctypes.c_int]
        _lib = L
    return _lib


def _ptr64(a: np.ndarray):
    return a.ctypes.data_as(_p64)


def _ptr32(a: np.ndarray):
    return a.ctypes.data_as(_p32)


# ---------------------------------------------------------------- arithmetic
def mu64(p: int) -> int:
    return lib().ctdo_mu64(p)


def mu128(p: int) -> int:
    out = (_u64 * 2)()
    lib().ctdo_mu128(p, out)
    return (out[0] << 64) | out[1]


def mul128hi(a: int, b: int) -> int:
    A = (_u64 * 2)(a >> 64, a & (2**64 - 1))
    B = (_u64 * 2)(b >> 64, b & (2**64 - 1))
    out = (_u64 * 2)()
    lib().ctdo_mul128hi(A, B, out)
    return (out[0] << 64) | out[1]


def mulmod(a: int, b: int, d: int) -> int:
    return lib().ctdo_mulmod(a, b, d)


def modpow(a: int, e: int, d: int) -> int:
    return lib().ctdo_modpow(a, e, d)


def reciprocal(d: int) -> int:
    return lib().ctdo_reciprocal(d)


def mod2by1(u1: int, u0: int, d: int, rnd: int) -> int:
    return lib().ctdo_mod2by1(u1, u0, d, rnd)


def modnby1(limbs, d: int) -> int:
    a = np.ascontiguousarray(np.asarray(limbs, dtype=np.uint64))
    return lib().ctdo_modnby1(_ptr64(a), a.size, d)


# ------------------------------------------------------------------- primes
def sieve(lo: int, hi: int) -> np.ndarray:
    """Primes in [lo, hi), ascending."""
    L = lib()
    n = L.ctdo_sieve(lo, hi, None, 0)
    out = np.empty(max(n, 1), dtype=np.uint64)
    L.ctdo_sieve(lo, hi, _ptr64(out), n)
    return out[:n]


# ------------------------------------------------------------------ plugins
def check_seq(family: int, param: int) -> bool:
    return lib().ctdo_check_seq(family, param) == 0


def value_mod_2(family: int, param: int, n: int) -> int:
    return lib().ctdo_value_mod_2(family, param, n)


def next_value_mod_2(family: int, param: int, r: int, n: int) -> int:
    return lib().ctdo_next_value_mod_2(family, param, r, n)


def smarandache_limbs(base: int, n: int) -> np.ndarray:
    L = lib()
    k = L.ctdo_smarandache_limbs(base, n, None, 0)
    out = np.zeros(max(k, 1), dtype=np.uint64)
    L.ctdo_smarandache_limbs(base, n, _ptr64(out), k)
    return out[:k]


def init_state(family: int, param: int, n0: int, p: int):
    """(residue, state tuple) of S(n0) mod p."""
    limbs = smarandache_limbs(param, n0) if family == SMARANDACHE else np.zeros(1, np.uint64)
    st = _State()
    lib().ctdo_init(family, param, n0, p, _ptr64(limbs), limbs.size if family == SMARANDACHE else 0,
                    ctypes.byref(st))
    return st


def step(family: int, param: int, n: int, p: int, st) -> None:
    lib().ctdo_step(family, param, n, p, ctypes.byref(st))


def residues(family: int, param: int, n0: int, n1: int, p: int) -> list[int]:
    """[S(n) mod p for n in [n0, n1)] propagated like the engine."""
    st = init_state(family, param, n0, p)
    out = [st.r]
    for n in range(n0, n1 - 1):
        step(family, param, n, p, st)
        out.append(st.r)
    return out


# ------------------------------------------------------------------- engine
@dataclass
class FactorsBuffer:
    """Host factors buffer in the reference layout (src/factors_buffer.hpp:77-86)."""
    n0: int
    max_factors: int
    counts: np.ndarray   # uint32[N]
    factors: np.ndarray  # uint64[N * max_factors]

    @classmethod
    def empty(cls, n0: int, n1: int, max_factors: int) -> "FactorsBuffer":
        N = n1 - n0
        return cls(n0, max_factors, np.zeros(N, np.uint32), np.zeros(N * max_factors, np.uint64))

    def factor_lists(self) -> list[list[int]]:
        """Stored factors per index, sorted ascending (src/factors_buffer.hpp:123-138)."""
        m = self.max_factors
        f = self.factors.reshape(-1, m) if m else self.factors.reshape(len(self.counts), 0)
        out = []
        for i, c in enumerate(self.counts.tolist()):
            out.append(sorted(int(x) for x in f[i, : min(c, m)]))
        return out

    def format(self) -> str:
        """'<n> - p1, p2' lines (src/factoring_results.hpp:507-525)."""
        return "".join(f"{self.n0 + i} - {', '.join(map(str, fl))}\n"
                       for i, fl in enumerate(self.factor_lists()))


def _job(family, param, n0, n1, f0, f1, max_factors):
    return _Job(family, max_factors, param, n0, n1, f0, f1)


def trial_factor(family: int, param: int, n0: int, n1: int, f0: int, f1: int,
                 max_factors: int = 32, threads: int = 0, segment_length: int = 1 << 26,
                 resume_after_prime: int = 0, buf: FactorsBuffer | None = None) -> FactorsBuffer:
    """Whole job on the CPU: the restatement of host_trial_factor."""
    if buf is None:
        buf = FactorsBuffer.empty(n0, n1, max_factors)
    threads = threads or (os.cpu_count() or 1)
    rc = lib().ctdo_trial_factor(ctypes.byref(_job(family, param, n0, n1, f0, f1, max_factors)),
                                 _ptr32(buf.counts), _ptr64(buf.factors), resume_after_prime,
                                 segment_length, threads)
    if rc:
        raise ValueError("oracle rejected the job")
    return buf


def residue_hits(family: int, param: int, n0: int, n1: int, primes: np.ndarray,
                 max_factors: int = 32, threads: int = 0, buf: FactorsBuffer | None = None) -> FactorsBuffer:
    """The residue loop over an explicit odd-prime list (the GPU kernel's unit)."""
    primes = np.ascontiguousarray(primes, dtype=np.uint64)
    if buf is None:
        buf = FactorsBuffer.empty(n0, n1, max_factors)
    threads = threads or (os.cpu_count() or 1)
    rc = lib().ctdo_residues(ctypes.byref(_job(family, param, n0, n1, 0, 0, max_factors)),
                             _ptr64(primes), primes.size, _ptr32(buf.counts), _ptr64(buf.factors),
                             threads)
    if rc:
        raise ValueError("oracle rejected the job")
    return buf
