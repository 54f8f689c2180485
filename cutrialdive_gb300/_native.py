"""ctypes binding of libctd_gpu.so (the C ABI declared in include/ctd_gpu.h).

The library is in-tree (``cutrialdive_gb300/libctd_gpu.so``); loading fails
loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB

CTD_OK = 0
CTD_ERR_INVALID_ARGUMENT = -1
CTD_ERR_CUDA = -2
CTD_ERR_OUT_OF_MEMORY = -3
CTD_ERR_ABORTED = -4
CTD_ERR_TIMEOUT = -5
CTD_ERR_CAPACITY = -6
CTD_ERR_NOT_FOUND = -7

CTD_CB_CONTINUE, CTD_CB_SNAPSHOT, CTD_CB_ABORT = 0, 1, 2

u32, u64, i32 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
p64 = ctypes.POINTER(ctypes.c_uint64)
p32 = ctypes.POINTER(ctypes.c_uint32)
vp = ctypes.c_void_p


class CtdJob(ctypes.Structure):
    _fields_ = [("family", u32), ("max_factors", u32), ("param", u64),
                ("n0", u64), ("n1", u64), ("f0", u64), ("f1", u64)]


class CtdProgress(ctypes.Structure):
    _fields_ = [("segment_end", u64), ("last_prime", u64), ("primes_done", u64), ("elapsed_s", ctypes.c_double)]


class CtdTuning(ctypes.Structure):
    _fields_ = [("block_size", i32), ("ctas_per_sm", i32), ("items_per_thread", u32), ("min_tile", u32),
                ("segment_log2", u32), ("variant", u32), ("classify_min", u32), ("refine_q", u32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


PROGRESS_CB = ctypes.CFUNCTYPE(i32, vp, ctypes.POINTER(CtdProgress), i32)

# every symbol include/ctd_gpu.h declares, with its ctypes signature
SIGNATURES = {
    "ctd_abi_version": (i32, []),
    "ctd_strerror": (ctypes.c_char_p, [i32]),
    "ctd_kernel_launches": (u64, []),
    "ctd_open": (i32, [i32, ctypes.POINTER(vp)]),
    "ctd_close": (None, [vp]),
    "ctd_last_error": (ctypes.c_char_p, [vp]),
    "ctd_device_info": (i32, [vp, ctypes.c_char_p, ctypes.c_size_t, p64, ctypes.POINTER(i32)]),
    "ctd_set_launch": (i32, [vp, i32, i32]),
    "ctd_check_job": (i32, [ctypes.POINTER(CtdJob)]),
    "ctd_run_plain": (i32, [vp, ctypes.POINTER(CtdJob), p32, p64, u64, u64, PROGRESS_CB, vp]),
    "ctd_sieve": (i32, [vp, u64, u64, p64, u64, p64]),
    "ctd_sieve_device": (i32, [vp, u64, u64, vp, u64, p64, vp]),
    "ctd_residues_device": (i32, [vp, ctypes.POINTER(CtdJob), vp, u64, vp, vp, vp]),
    "ctd_mod2_device": (i32, [vp, ctypes.POINTER(CtdJob), vp, vp, vp]),
    "ctd_sieve_device_noalloc": (i32, [vp, u64, u64, vp, u64, p64, vp]),
    "ctd_batch_run": (i32, [vp, ctypes.POINTER(CtdJob), u32, ctypes.POINTER(p32), ctypes.POINTER(p64), u64, i32]),
    "ctd_batch_graph_stats": (i32, [vp, p64, p64, p64]),
    "ctd_serve_open": (i32, [vp, u64, u32, u64, ctypes.POINTER(vp)]),
    "ctd_serve_close": (None, [vp]),
    "ctd_serve_submit": (i32, [vp, ctypes.POINTER(CtdJob), p64]),
    "ctd_serve_tick": (i32, [vp, p64, u32, ctypes.POINTER(u32)]),
    "ctd_serve_fetch": (i32, [vp, u64, p32, p64]),
    "ctd_serve_status": (i32, [vp, ctypes.POINTER(u32), ctypes.POINTER(u32), p64]),
    "ctd_get_tuning": (i32, [vp, u32, ctypes.POINTER(CtdTuning)]),
    "ctd_set_tuning": (i32, [vp, u32, ctypes.POINTER(CtdTuning)]),
    "ctd_get_tuning_for": (i32, [vp, u32, u32, ctypes.POINTER(CtdTuning)]),
    "ctd_set_tuning_for": (i32, [vp, u32, u32, ctypes.POINTER(CtdTuning)]),
    "ctd_autotune": (i32, [vp, ctypes.POINTER(CtdJob), ctypes.c_double, ctypes.POINTER(CtdTuning)]),
}

_lib = None


def lib_path() -> str:
    return LIB


def load() -> ctypes.CDLL:
    """Load libctd_gpu.so (built by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise ImportError(
            f"libctd_gpu.so not found at {LIB}: build it first (python -c 'import __graft_entry__ as g; g.build()'); "
            "there is no CPU fallback")
    L = ctypes.CDLL(LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class CtdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status
