"""ctd_sieve_device_noalloc: the device sieve for callers that may not
allocate device memory (a process that reserves its whole memory budget at
start-up, or a host whose pool allocator owns all GPU memory).  Its scratch
is a fixed array compiled into the library instead of cudaMalloc'ed buffers.

Checked here through the C ABI against the allocating entry point
ctd_sieve_device on two calls in a row -- the second one smaller than the
first, so anything the first call left in the shared array would show up.
Prime lists are integers: the comparison is exact.  This file is collected
last so that a failure here never hides the other tests' results."""
import ctypes

import numpy as np
import pytest

import cutrialdive_gb300 as ctd
from cutrialdive_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _sieve(fn, eng, lo, hi, out):
    count = ctypes.c_uint64()
    rc = fn(eng.handle, lo, hi, ctypes.c_void_p(out.data_ptr()), out.numel(), ctypes.byref(count), None)
    assert rc == 0, N.load().ctd_last_error(eng.handle).decode()
    return out[: count.value].cpu().numpy().view(np.uint64).copy()


def test_noalloc_sieve_matches_allocating_sieve():
    torch = pytest.importorskip("torch")
    L = N.load()
    eng = ctd.Engine(0)
    cap = 1 << 22
    out_new = torch.zeros(cap, dtype=torch.int64, device="cuda")
    out_old = torch.zeros(cap, dtype=torch.int64, device="cuda")
    # two calls in a row: a full-width range high up, then a small one from 0
    # (fewer windows, smaller base primes, the prime 2)
    for lo, hi in [((1 << 40) + 12345, (1 << 40) + 12345 + (1 << 26)), (0, (1 << 20) + 777)]:
        new = _sieve(L.ctd_sieve_device_noalloc, eng, lo, hi, out_new)
        old = _sieve(L.ctd_sieve_device, eng, lo, hi, out_old)
        assert new.size == old.size > 0
        assert np.array_equal(new, old), (lo, hi)
    eng.close()


def test_noalloc_sieve_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    L = N.load()
    eng = ctd.Engine(0)
    out = torch.zeros(16, dtype=torch.int64, device="cuda")
    count = ctypes.c_uint64()
    too_wide = L.ctd_sieve_device_noalloc(eng.handle, 1 << 32, (1 << 32) + (1 << 26) + 1,
                                          ctypes.c_void_p(out.data_ptr()), 16, ctypes.byref(count), None)
    assert too_wide == N.CTD_ERR_INVALID_ARGUMENT
    assert b"CTD_NOALLOC_SIEVE_MAX_RANGE" in L.ctd_last_error(eng.handle)
    too_high = L.ctd_sieve_device_noalloc(eng.handle, 1 << 49, (1 << 49) + 100,
                                          ctypes.c_void_p(out.data_ptr()), 16, ctypes.byref(count), None)
    assert too_high == N.CTD_ERR_INVALID_ARGUMENT
    assert b"CTD_NOALLOC_SIEVE_MAX_HI" in L.ctd_last_error(eng.handle)
    eng.close()
