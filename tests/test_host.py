"""Host-side logic that needs no GPU: the C ABI library loads and exports
every symbol include/ctd_gpu.h declares; sequence-spec dispatch; factors
buffer formatting; checkpoint v1 codec (tests/checkpointing_tests.cpp)."""
import ctypes
import os
import re

import numpy as np
import pytest

import cutrialdive_gb300 as ctd
from cutrialdive_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "ctd_gpu.h")).read()
    return sorted(set(re.findall(r"\b(ctd_[a-z0-9_]+)\s*\(", text)) - {"ctd_progress_cb"})


def test_library_exports_header_symbols():
    L = _native.load()
    for name in header_symbols():
        assert hasattr(L, name), f"libctd_gpu.so does not export {name}"
    assert set(header_symbols()) <= set(_native.SIGNATURES), "binding misses a declared symbol"


def test_abi_calls_without_gpu():
    L = _native.load()
    assert L.ctd_abi_version() == 1
    assert L.ctd_strerror(_native.CTD_ERR_CAPACITY) == b"output buffer too small"
    ok = ctd.CtdJob(1, 32, 3, 1, 100, 3, 1000)
    assert L.ctd_check_job(ctypes.byref(ok)) == 0
    for bad in (ctd.CtdJob(1, 32, 0, 1, 100, 3, 1000),      # Proth k = 0
                ctd.CtdJob(3, 32, 65, 1, 100, 3, 1000),     # Smarandache base 65
                ctd.CtdJob(4, 32, 0, 10, 10, 3, 1000),      # empty index range
                ctd.CtdJob(4, 0, 0, 1, 10, 3, 1000),        # no factor slots
                ctd.CtdJob(99, 32, 0, 1, 10, 3, 1000)):     # unknown family
        assert L.ctd_check_job(ctypes.byref(bad)) == _native.CTD_ERR_INVALID_ARGUMENT


def test_no_fallback_without_library(monkeypatch, tmp_path):
    monkeypatch.setattr(_native, "LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_native, "_lib", None)
    with pytest.raises(ImportError, match="no CPU fallback"):
        _native.load()


# ------------------------------------------------------------ dispatch
def test_num_seq_id_from_string():
    assert ctd.num_seq_id_from_string("proth_fixed_n") == ctd.num_seq_id.proth_fixed_n == 6
    with pytest.raises(RuntimeError, match="Invalid number sequence id `fermat'"):
        ctd.num_seq_id_from_string("fermat")


def test_dispatch_like_reference():
    D = ctd.dispatch
    S = ctd.num_seq_spec
    assert D(S(ctd.num_seq_id.smarandache)) == (3, 10)
    assert D(S(ctd.num_seq_id.smarandache, "2")) == (3, 2)
    assert D(S(ctd.num_seq_id.proth, "1279")) == (1, 1279)
    assert D(S(ctd.num_seq_id.riesel, "12x")) == (2, 12)  # from_chars stops at the first non-digit
    with pytest.raises(RuntimeError, match="Missing or invalid k value `' in Proth number spec"):
        D(S(ctd.num_seq_id.proth))
    with pytest.raises(RuntimeError, match="Base `65' is not supported"):
        D(S(ctd.num_seq_id.smarandache, "65"))
    with pytest.raises(RuntimeError, match="Invalid base `x'"):
        D(S(ctd.num_seq_id.smarandache, "x"))
    with pytest.raises(ValueError, match="Proth parameter k must be non-zero"):
        D(S(ctd.num_seq_id.proth, "0"))
    with pytest.raises(ValueError, match="Invalid n value zero"):
        D(S(ctd.num_seq_id.riesel_fixed_n, "0"))


# ------------------------------------------------------------- results
def test_results_format_and_sort():
    buf = ctd.factors_buffer.empty(101, 4, 3)
    buf.counts[:] = [0, 2, 0, 4]
    buf.factors[3:5] = [103, 7]
    buf.factors[9:12] = [53, 3, 17]
    res = buf.to_factoring_results()
    # ascending per term, no brackets, trailing space when empty
    # (src/factoring_results.hpp:507-525); the 4th factor did not fit
    assert str(res) == "101 - \n102 - 7, 103\n103 - \n104 - 3, 17, 53\n"
    assert res.max_factors_count() == 4 and res.factors_count() == 6


# ----------------------------------------------------------- checkpoint
def test_checkpoint_round_trip(tmp_path):
    # tests/checkpointing_tests.cpp:23-73
    spec = ctd.num_seq_spec(ctd.num_seq_id.mersenne)
    opts = ctd.trial_factoring_options(101, 105, 0, 1 << 16, None, 32)
    buf = ctd.factors_buffer.empty(101, 4, 32)
    for idx, p in [(1, 3), (1, 7), (1, 103), (3, 3), (3, 5), (3, 17), (3, 53)]:
        buf.factors[idx * 32 + buf.counts[idx]] = p
        buf.counts[idx] += 1
    path = str(tmp_path / "x.chkpnt")
    ctd.write_checkpoint(path, spec, opts, 127, buf)
    spec2, opts2, last, buf2 = ctd.load_checkpoint(path)
    assert (spec2, opts2, last) == (spec, opts, 127)
    assert buf2.n0 == 101 and buf2.numbers_count == 4 and buf2.max_factors_per_number == 32
    assert np.array_equal(buf2.counts, buf.counts) and np.array_equal(buf2.factors, buf.factors)
    res = buf2.to_factoring_results()
    assert res.size() == 4 and res[0] == [] and res[1] == [3, 7, 103]


def test_checkpoint_layout_bytes(tmp_path):
    """Field order and widths of src/checkpoint.cpp:172-198 (native endian, LP64)."""
    import struct

    spec = ctd.num_seq_spec(ctd.num_seq_id.proth, "3")
    opts = ctd.trial_factoring_options(1, 3, 5, 99, "out.txt", 2)
    buf = ctd.factors_buffer.empty(1, 2, 2)
    buf.counts[:] = [3, 1]
    buf.factors[:] = [11, 13, 17, 0]
    path = str(tmp_path / "c")
    ctd.write_checkpoint(path, spec, opts, 97, buf)
    data = open(path, "rb").read()
    expect = (struct.pack("=II", 1, 1) + struct.pack("=Q", 1) + b"3" + struct.pack("=QQQQ", 1, 3, 5, 99)
              + struct.pack("=Q", 7) + b"out.txt" + struct.pack("=IQ", 2, 97) + struct.pack("=QIQ", 2, 2, 1)
              + struct.pack("=I", 3) + struct.pack("=QQ", 11, 13) + struct.pack("=I", 1) + struct.pack("=Q", 17))
    assert data == expect


def test_checkpoint_wrong_version_and_truncation(tmp_path):
    path = str(tmp_path / "bad")
    open(path, "wb").write((2).to_bytes(4, "little") + b"\0" * 20)
    with pytest.raises(RuntimeError, match="Unexpected version number `2'"):
        ctd.load_checkpoint(path)
    open(path, "wb").write((1).to_bytes(4, "little") + b"\0" * 5)
    with pytest.raises(RuntimeError, match="Truncated"):
        ctd.load_checkpoint(path)
    assert ctd.load_checkpoint(str(tmp_path / "absent")) is None


def test_checkpoint_into_missing_directory(tmp_path):
    """A checkpoint that cannot be created fails with the reference's message
    (src/checkpoint.cpp:181-184) instead of losing the state silently."""
    spec = ctd.num_seq_spec(ctd.num_seq_id.mersenne)
    opts = ctd.trial_factoring_options(1, 3, 0, 100, None, 2)
    buf = ctd.factors_buffer.empty(1, 2, 2)
    path = str(tmp_path / "no_such_dir" / "x.chkpnt")
    with pytest.raises(RuntimeError, match=r"Could not create temporary file `.*no_such_dir/x\.chkpnt\.tmp_\d+'"):
        ctd.write_checkpoint(path, spec, opts, 7, buf)
    assert not os.path.exists(os.path.dirname(path))
