"""Python mirror of cutrialdive's library API over the GB300 engine.

Same names, argument meaning and error behaviour as the reference's public
interface (src/trial_factoring.hpp:21-37, src/num_seq_spec.hpp:16-22,
src/num_seq_id.cpp:25-43, src/num_seq_dispatch.hpp:120-170,
src/trial_factoring_options.hpp:15-59, src/factoring_results.hpp:346-525,
src/checkpoint.cpp:172-225), so tests read like the reference's own.  All
trial factoring runs on the GPU through libctd_gpu.so.
"""
from __future__ import annotations

import ctypes
import enum
import io
import os
import struct
import sys
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native as N


# ------------------------------------------------------------ sequences
class num_seq_id(enum.IntEnum):
    """src/num_seq_id.hpp:16-26 (the numbering is stored in checkpoints)."""
    mersenne = 0
    proth = 1
    riesel = 2
    smarandache = 3
    fibonacci = 4
    lucas = 5
    proth_fixed_n = 6
    riesel_fixed_n = 7
    tribonacci = 8


PEANO = 256  # the reference's test-only S(n) = n (tests/peano.hpp), no --num-seq name


def num_seq_id_from_string(name: str) -> num_seq_id:
    """src/num_seq_id.cpp:25-43."""
    try:
        return num_seq_id[name]
    except KeyError:
        raise RuntimeError(f"Invalid number sequence id `{name}'") from None


@dataclass(frozen=True)
class num_seq_spec:
    seq_id: int
    seq_params: str = ""


def _parse_u64(s: str) -> Optional[int]:
    # std::from_chars on uint64_t: leading decimal digits, no sign, no spaces
    i = 0
    while i < len(s) and s[i].isdigit():
        i += 1
    if i == 0:
        return None
    v = int(s[:i])
    return v if v < 2**64 else None


def dispatch(spec: num_seq_spec) -> tuple[int, int]:
    """(family, param) for a spec, with the reference's checks and messages
    (src/num_seq_dispatch.hpp:120-170 and the plugin constructors)."""
    sid, params = int(spec.seq_id), spec.seq_params
    if sid in (num_seq_id.mersenne, num_seq_id.fibonacci, num_seq_id.lucas, num_seq_id.tribonacci, PEANO):
        return sid, 0
    if sid in (num_seq_id.proth, num_seq_id.riesel):
        k = _parse_u64(params)
        which = "Proth number" if sid == num_seq_id.proth else "Riesel sequence"
        if k is None:
            raise RuntimeError(f"Missing or invalid k value `{params}' in {which} spec")
        if k == 0:
            raise ValueError(("Proth" if sid == num_seq_id.proth else "Riesel") + " parameter k must be non-zero")
        return sid, k
    if sid == num_seq_id.smarandache:
        base = 10 if params == "" else _parse_u64(params)
        if base is None:
            raise RuntimeError(f"Invalid base `{params}' for Smarandache numbers")
        if not 2 <= base <= 64:
            raise RuntimeError(f"Base `{base}' is not supported for Smarandache numbers")
        return sid, base
    if sid in (num_seq_id.proth_fixed_n, num_seq_id.riesel_fixed_n):
        n = _parse_u64(params)
        which = "Proth number" if sid == num_seq_id.proth_fixed_n else "Riesel sequence"
        if n is None:
            raise RuntimeError(f"Missing or invalid n value `{params}' in {which} spec")
        if n == 0:
            raise ValueError("Invalid n value zero for Riesel/Proth fixed n")
        return sid, n
    raise RuntimeError(f"Unexpected number sequence id: {sid}")


# -------------------------------------------------------------- options
@dataclass
class trial_factoring_options:
    """src/trial_factoring_options.hpp:15-31."""
    n0: int
    n1: int
    f0: int
    f1: int
    output_path: Optional[str] = None
    max_factors_per_number: int = 32


@dataclass
class tf_runtime_options:
    """src/trial_factoring_options.hpp:36-59 (defaults :30-41 of the .cpp)."""
    threads_count: int = 4
    checkpoint_period: float = 360.0
    progress_period: float = 1.0
    is_progress_enabled: bool = True
    segment_length: int = 1 << 26
    device_id: int = 0
    grid_size: Optional[int] = None
    block_size: Optional[int] = None


# -------------------------------------------------------------- results
@dataclass
class factors_buffer:
    """Host factors buffer in the reference layout (src/factors_buffer.hpp:77-86)."""
    n0: int
    max_factors_per_number: int
    counts: np.ndarray
    factors: np.ndarray

    @classmethod
    def empty(cls, n0: int, numbers: int, max_factors: int) -> "factors_buffer":
        return cls(n0, max_factors, np.zeros(numbers, np.uint32), np.zeros(numbers * max_factors, np.uint64))

    @property
    def numbers_count(self) -> int:
        return int(self.counts.size)

    def to_factoring_results(self) -> "factoring_results":
        """Sorts each term's stored factors (src/factors_buffer.hpp:123-138)."""
        m = self.max_factors_per_number
        f = self.factors.reshape(self.numbers_count, m)
        lists = []
        for i, c in enumerate(self.counts.tolist()):
            lists.append(sorted(int(x) for x in f[i, : min(c, m)]))
        return factoring_results(self.n0, lists, [int(c) for c in self.counts.tolist()])


class factoring_results:
    """src/factoring_results.hpp:346-525."""

    def __init__(self, n0: int, factor_lists: list, found_counts: list):
        self._n0 = n0
        self._lists = factor_lists
        self._found = found_counts

    def n0(self) -> int:
        return self._n0

    def size(self) -> int:
        return len(self._lists)

    def __len__(self) -> int:
        return len(self._lists)

    def empty(self) -> bool:
        return not self._lists

    def __getitem__(self, i: int) -> list:
        return self._lists[i]

    def max_factors_count(self) -> int:
        return max(self._found, default=0)

    def factors_count(self) -> int:
        return sum(self._found)

    def __str__(self) -> str:
        out = io.StringIO()
        for i, fl in enumerate(self._lists):
            out.write(f"{self._n0 + i} - {', '.join(str(p) for p in fl)}\n")
        return out.getvalue()


# ----------------------------------------------------------- checkpoint
CHECKPOINT_FILE_VERSION = 1


def _w_str(b: io.BytesIO, s: str) -> None:
    data = s.encode()
    b.write(struct.pack("=Q", len(data)))
    b.write(data)


def write_checkpoint(path: str, spec: num_seq_spec, opts: trial_factoring_options, last_processed_prime: int,
                     buf: factors_buffer) -> None:
    """Native-endian LP64 layout of src/checkpoint.cpp:172-198 (temp file + rename)."""
    b = io.BytesIO()
    b.write(struct.pack("=II", CHECKPOINT_FILE_VERSION, int(spec.seq_id)))
    _w_str(b, spec.seq_params)
    b.write(struct.pack("=QQQQ", opts.n0, opts.n1, opts.f0, opts.f1))
    _w_str(b, opts.output_path or "")
    b.write(struct.pack("=IQ", opts.max_factors_per_number, last_processed_prime))
    m = buf.max_factors_per_number
    b.write(struct.pack("=QIQ", buf.numbers_count, m, buf.n0))
    f = buf.factors.reshape(buf.numbers_count, m)
    for i, c in enumerate(buf.counts.tolist()):
        b.write(struct.pack("=I", c))
        b.write(f[i, : min(c, m)].astype("=u8").tobytes())
    tmp = f"{path}.tmp_{time.time_ns()}"
    try:
        fh = open(tmp, "wb")
    except OSError:  # the reference's message (src/checkpoint.cpp:181-184)
        raise RuntimeError(f"Could not create temporary file `{tmp}'") from None
    with fh:
        fh.write(b.getvalue())
    os.replace(tmp, path)


def load_checkpoint(path: str):
    """src/checkpoint.cpp:200-225 -> (spec, opts, last_processed_prime, factors_buffer) or None."""
    try:
        data = open(path, "rb").read()
    except OSError:
        return None
    pos = 0

    def take(fmt):
        nonlocal pos
        sz = struct.calcsize(fmt)
        if pos + sz > len(data):
            raise RuntimeError(f"Truncated checkpoint file `{path}'")
        v = struct.unpack_from(fmt, data, pos)
        pos += sz
        return v

    def take_str():
        nonlocal pos
        (n,) = take("=Q")
        if pos + n > len(data):
            raise RuntimeError(f"Truncated checkpoint file `{path}'")
        s = data[pos:pos + n].decode()
        pos += n
        return s

    (version,) = take("=I")
    if version != CHECKPOINT_FILE_VERSION:
        raise RuntimeError(f"Unexpected version number `{version}' found in checkpoint file")
    (sid,) = take("=I")
    spec = num_seq_spec(sid, take_str())
    n0, n1, f0, f1 = take("=QQQQ")
    out_path = take_str() or None
    (maxf,) = take("=I")
    opts = trial_factoring_options(n0, n1, f0, f1, out_path, maxf)
    (last,) = take("=Q")
    numbers, m, bn0 = take("=QIQ")
    buf = factors_buffer.empty(bn0, numbers, m)
    f = buf.factors.reshape(numbers, m)
    for i in range(numbers):
        (c,) = take("=I")
        buf.counts[i] = c
        k = min(c, m)
        if k:
            vals = take(f"={k}Q")
            f[i, :k] = vals
    return spec, opts, last, buf


# ---------------------------------------------------------------- engine
class Engine:
    """One device context (ctd_open / ctd_close)."""

    def __init__(self, device: int = 0):
        self._L = N.load()
        h = ctypes.c_void_p()
        rc = self._L.ctd_open(device, ctypes.byref(h))
        if rc:
            raise N.CtdError(rc, f"ctd_open({device}) failed: {self._L.ctd_strerror(rc).decode()}")
        self._h = h

    def close(self) -> None:
        if self._h:
            self._L.ctd_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, rc: int, what: str) -> None:
        if rc:
            msg = self._L.ctd_last_error(self._h).decode() or self._L.ctd_strerror(rc).decode()
            raise N.CtdError(rc, f"{what}: {msg}")

    def device_info(self) -> dict:
        name = ctypes.create_string_buffer(256)
        mem = ctypes.c_uint64()
        sms = ctypes.c_int()
        self._check(self._L.ctd_device_info(self._h, name, 256, ctypes.byref(mem), ctypes.byref(sms)), "device_info")
        return {"name": name.value.decode(), "total_mem": mem.value, "sm_count": sms.value}

    def set_launch(self, grid_size: int = 0, block_size: int = 0) -> None:
        self._check(self._L.ctd_set_launch(self._h, grid_size, block_size), "set_launch")

    def prime_count(self, lo: int, hi: int) -> int:
        """Number of primes in [lo, hi) (ctd_sieve with no output array)."""
        count = ctypes.c_uint64()
        rc = self._L.ctd_sieve(self._h, lo, hi, None, 0, ctypes.byref(count))
        if rc not in (0, N.CTD_ERR_CAPACITY):
            self._check(rc, "ctd_sieve")
        return count.value

    def sieve(self, lo: int, hi: int) -> np.ndarray:
        """Primes in [lo, hi) from the device sieve (ctd_sieve)."""
        count = ctypes.c_uint64()
        # first call sizes the output
        rc = self._L.ctd_sieve(self._h, lo, hi, None, 0, ctypes.byref(count))
        if rc not in (0, N.CTD_ERR_CAPACITY):
            self._check(rc, "ctd_sieve")
        out = np.empty(max(count.value, 1), np.uint64)
        rc = self._L.ctd_sieve(self._h, lo, hi, out.ctypes.data_as(N.p64), count.value, ctypes.byref(count))
        self._check(rc, "ctd_sieve")
        return out[: count.value]

    def run_plain(self, job: N.CtdJob, buf: factors_buffer, resume_after_prime: int = 0,
                  segment_length: int = 0, callback=None) -> None:
        """ctd_run_plain with a host factors buffer (updated in place)."""
        def _cb(_user, prog, snapshot):
            if callback is None:
                return N.CTD_CB_CONTINUE
            return int(callback(prog.contents, bool(snapshot)) or 0)

        cb = N.PROGRESS_CB(_cb)
        rc = self._L.ctd_run_plain(self._h, ctypes.byref(job), buf.counts.ctypes.data_as(N.p32),
                                   buf.factors.ctypes.data_as(N.p64), resume_after_prime, segment_length, cb, None)
        self._check(rc, "ctd_run_plain")

    def get_tuning(self, family: int) -> dict:
        """Launch/tiling parameters in force for a family (ctd_get_tuning)."""
        t = N.CtdTuning()
        self._check(self._L.ctd_get_tuning(self._h, family, ctypes.byref(t)), "ctd_get_tuning")
        return t.as_dict()

    def set_tuning(self, family: int, tuning: dict | None) -> None:
        """Sets (or with None resets) a family's parameters (ctd_set_tuning)."""
        if tuning is None:
            self._check(self._L.ctd_set_tuning(self._h, family, None), "ctd_set_tuning")
            return
        t = N.CtdTuning(**{k: int(v) for k, v in tuning.items()})
        self._check(self._L.ctd_set_tuning(self._h, family, ctypes.byref(t)), "ctd_set_tuning")

    def get_tuning_for(self, family: int, prime_bits: int) -> dict:
        """Parameters in force for a family at primes of `prime_bits` bits (ctd_get_tuning_for)."""
        t = N.CtdTuning()
        self._check(self._L.ctd_get_tuning_for(self._h, family, prime_bits, ctypes.byref(t)), "ctd_get_tuning_for")
        return t.as_dict()

    def set_tuning_for(self, family: int, prime_bits: int, tuning: dict | None) -> None:
        """Sets (or with None clears) a family's entry for one prime width (ctd_set_tuning_for)."""
        if tuning is None:
            self._check(self._L.ctd_set_tuning_for(self._h, family, prime_bits, None), "ctd_set_tuning_for")
            return
        t = N.CtdTuning(**{k: int(v) for k, v in tuning.items()})
        self._check(self._L.ctd_set_tuning_for(self._h, family, prime_bits, ctypes.byref(t)), "ctd_set_tuning_for")

    def autotune(self, job: N.CtdJob, budget_s: float = 2.0) -> dict:
        """Measures and applies the fastest parameters for the job's family (ctd_autotune)."""
        t = N.CtdTuning()
        self._check(self._L.ctd_autotune(self._h, ctypes.byref(job), budget_s, ctypes.byref(t)), "ctd_autotune")
        return t.as_dict()

    def batch_run(self, jobs: list, bufs: list, segment_length: int = 0, use_graph: bool = True) -> None:
        """ctd_batch_run: several jobs in one chunk-major, graph-captured pass."""
        n = len(jobs)
        arr = (N.CtdJob * n)(*jobs)
        cps = (N.p32 * n)(*[b.counts.ctypes.data_as(N.p32) for b in bufs])
        fps = (N.p64 * n)(*[b.factors.ctypes.data_as(N.p64) for b in bufs])
        self._check(self._L.ctd_batch_run(self._h, arr, n, cps, fps, segment_length, 1 if use_graph else 0),
                    "ctd_batch_run")


    def batch_graph_stats(self) -> dict:
        """Graphs ctd_batch_run instantiated, updated in place and replayed."""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._L.ctd_batch_graph_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
                    "ctd_batch_graph_stats")
        return {"instantiations": a.value, "updates": b.value, "replays": c.value}


class Server:
    """Continuous-batching server over ctd_serve_* (one device context)."""

    def __init__(self, eng: Engine, memory_budget: int = 160 << 30, max_active: int = 256,
                 segment_length: int = 1 << 30):
        self._eng = eng
        self._L = eng._L
        h = ctypes.c_void_p()
        eng._check(self._L.ctd_serve_open(eng.handle, memory_budget, max_active, segment_length, ctypes.byref(h)),
                   "ctd_serve_open")
        self._h = h
        self._jobs: dict = {}

    def submit(self, job: N.CtdJob) -> int:
        jid = ctypes.c_uint64()
        self._eng._check(self._L.ctd_serve_submit(self._h, ctypes.byref(job), ctypes.byref(jid)), "ctd_serve_submit")
        self._jobs[jid.value] = job
        return jid.value

    def tick(self) -> list[int]:
        cap = max(len(self._jobs), 1)
        ids = (ctypes.c_uint64 * cap)()
        nd = ctypes.c_uint32()
        self._eng._check(self._L.ctd_serve_tick(self._h, ids, cap, ctypes.byref(nd)), "ctd_serve_tick")
        return [ids[i] for i in range(min(nd.value, cap))]

    def fetch(self, jid: int) -> factors_buffer:
        job = self._jobs.pop(jid)
        buf = factors_buffer.empty(job.n0, job.n1 - job.n0, job.max_factors)
        self._eng._check(self._L.ctd_serve_fetch(self._h, jid, buf.counts.ctypes.data_as(N.p32),
                                                 buf.factors.ctypes.data_as(N.p64)), "ctd_serve_fetch")
        return buf

    def status(self) -> dict:
        a, q, m = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
        self._L.ctd_serve_status(self._h, ctypes.byref(a), ctypes.byref(q), ctypes.byref(m))
        return {"active": a.value, "queued": q.value, "memory_used": m.value}

    def close(self) -> None:
        if self._h:
            self._L.ctd_serve_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_engines: dict = {}


def engine(device: int = 0) -> Engine:
    """A process-wide context per device."""
    e = _engines.get(device)
    if e is None:
        e = _engines[device] = Engine(device)
    return e


def make_job(spec: num_seq_spec, opts: trial_factoring_options) -> N.CtdJob:
    fam, param = dispatch(spec)
    return N.CtdJob(fam, opts.max_factors_per_number, param, opts.n0, opts.n1, opts.f0, opts.f1)


# ------------------------------------------------------------ front end
class _Progress:
    """The '[x% done][prime][Elapsed][ETA]' line (src/progress.cpp:70-104)."""

    def __init__(self, start, target, period, out):
        self.start, self.target, self.period, self.out = start, target, period, out
        self.t0 = self.last = time.monotonic()
        self.width = len(str(target))

    @staticmethod
    def _dur(s):
        h, m = int(s // 3600), int((s % 3600) // 60)
        return f"{h:02d}:{m:02d}:{int(s % 60):02d}"

    def update(self, current, last_prime):
        now = time.monotonic()
        if now - self.last < self.period and current != self.target:
            return
        pct = ((current - self.start) * 10_000_000_000 // max(self.target - self.start, 1)) / 100_000_000.0
        el = now - self.t0
        line = f"\r{' ' * 128}\r[{pct:6.2f}% done][{last_prime:>{self.width}}][Elapsed {self._dur(el)}]"
        if current != self.target and pct > 0:
            line += f"[ETA {self._dur((100 - pct) / pct * el)}]"
        self.out.write(line)
        self.out.flush()
        self.last = now

    def end(self):
        self.out.write("\n")


def _trial_factor(spec, opts, rt, out, checkpoint_path, resume_state):
    rt = rt or tf_runtime_options()
    out = out if out is not None else sys.stdout
    if opts.n1 <= opts.n0:
        out.write(f"Range [{opts.n0}, {opts.n1}[ is empty, no number to process...\n")
        return factoring_results(opts.n0, [], [])
    if opts.f1 <= opts.f0:
        out.write(f"Range [{opts.f0}, {opts.f1}[ is empty, no prime numbers to divide by...\n")
        return factoring_results(opts.n0, [], [])
    job = make_job(spec, opts)
    eng = engine(rt.device_id)
    if rt.grid_size or rt.block_size:
        eng.set_launch(rt.grid_size or 0, rt.block_size or 0)
    out.write("Trial factoring starts, results will be written to "
              + (f"file `{opts.output_path}'" if opts.output_path else "the console.") + "\n")
    out.write(f"TF range is [{opts.f0}, {opts.f1}[.\n")
    if resume_state is not None:
        last, buf = resume_state
        out.write(f"Resuming at the smallest prime > {last}.\n")
    else:
        last, buf = 0, factors_buffer.empty(opts.n0, opts.n1 - opts.n0, opts.max_factors_per_number)
    f0 = last + 1 if last else opts.f0
    prog = _Progress(f0, opts.f1, rt.progress_period, out) if rt.is_progress_enabled else None
    last_write = [time.monotonic()]

    def cb(p, snapshot):
        if snapshot:
            write_checkpoint(checkpoint_path, spec, opts, p.last_prime, buf)
            last_write[0] = time.monotonic()
            return N.CTD_CB_CONTINUE
        if prog and p.last_prime:
            prog.update(p.segment_end, p.last_prime)
        if checkpoint_path and p.last_prime and time.monotonic() - last_write[0] >= rt.checkpoint_period:
            return N.CTD_CB_SNAPSHOT
        return N.CTD_CB_CONTINUE

    t0 = time.monotonic()
    eng.run_plain(job, buf, resume_after_prime=last, segment_length=rt.segment_length, callback=cb)
    if prog:
        prog.end()
    out.write(f"Trial factoring took {time.monotonic() - t0:.6g}s\n")
    results = buf.to_factoring_results()
    if opts.output_path:
        with open(opts.output_path, "w") as fh:
            fh.write(str(results))
    else:
        out.write(str(results))
    if checkpoint_path and os.path.exists(checkpoint_path):
        os.remove(checkpoint_path)
    return results


def trial_factor(spec: num_seq_spec, opts: trial_factoring_options, rt: tf_runtime_options | None = None,
                 out=None) -> factoring_results:
    """src/trial_factoring.hpp:21-27: with an output path, `<path>.chkpnt`
    receives periodic checkpoints (src/trial_factoring.cpp:44-60)."""
    ck = f"{opts.output_path}.chkpnt" if opts.output_path else None
    return _trial_factor(spec, opts, rt, out, ck, None)


def resume_trial_factoring(checkpoint_path: str, rt: tf_runtime_options | None = None, out=None) -> factoring_results:
    """src/trial_factoring.hpp:32-37 / src/trial_factoring.cpp:66-92."""
    out = out if out is not None else sys.stdout
    out.write(f"Resuming from checkpoint `{checkpoint_path}'...\n")
    data = load_checkpoint(checkpoint_path)
    if data is None:
        raise RuntimeError(f"Failed to load checkpoint data from file `{checkpoint_path}'")
    spec, opts, last, buf = data
    ck = f"{opts.output_path}.chkpnt" if opts.output_path else None
    return _trial_factor(spec, opts, rt, out, ck, (last, buf))
