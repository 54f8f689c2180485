"""Build recipe for the in-tree native parts of cutrialdive_gb300.

* ``libctd_gpu.so`` -- the CUDA engine and its C ABI (include/ctd_gpu.h),
  compiled by nvcc for sm_103a only;
* ``bin/cutrialdive`` -- the C++ command-line drop-in linked against it.

Translation units compile in parallel; up-to-date outputs are kept.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libctd_gpu.so")
CLI = os.path.join(PKG, "bin", "cutrialdive")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE]

CU_SOURCES = ["ctd_residue.cu", "ctd_sieve.cu", "ctd_engine.cu", "ctd_noalloc.cu", "ctd_batch.cu"]
HEADERS = ["ctd_arith.cuh", "ctd_smarandache.cuh", "ctd_internal.h"]
CLI_SOURCES = ["cli/main.cpp", "cli/command_line.cpp", "cli/results.cpp"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libctd_gpu.so")
    return path


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build_library(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "ctd_gpu.h")]
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + headers):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    if _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], verbose)
        os.replace(tmp, LIB)
    return LIB


PROBE = os.path.join(PKG, "libctd_probe.so")


def build_probe(verbose: bool = False) -> str:
    """libctd_probe.so: the integer-throughput probe bench.py uses as the
    roofline denominator (not part of the trial-factoring path)."""
    src = os.path.join(CSRC, "ctd_probe.cu")
    if _newer(PROBE, [src]):
        tmp = PROBE + ".tmp"
        _run([nvcc()] + NVCC_FLAGS + ["-shared", "-o", tmp, src], verbose)
        os.replace(tmp, PROBE)
    return PROBE


def build_cli(verbose: bool = False) -> str | None:
    srcs = [os.path.join(CSRC, s) for s in CLI_SOURCES]
    if not all(os.path.exists(s) for s in srcs):
        return None
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    deps = srcs + [os.path.join(CSRC, "cli", h) for h in os.listdir(os.path.join(CSRC, "cli")) if h.endswith(".hpp")]
    deps += [LIB, os.path.join(INCLUDE, "ctd_gpu.h")]
    if _newer(CLI, deps):
        tmp = CLI + ".tmp"
        cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-I", INCLUDE, "-o", tmp] + srcs + [
            "-L", PKG, "-lctd_gpu", f"-Wl,-rpath,{PKG}", "-Wl,-rpath,$ORIGIN/..", "-pthread"]
        _run(cmd, verbose)
        os.replace(tmp, CLI)
    return CLI


def build_all(verbose: bool = False) -> dict:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        probe = ex.submit(build_probe, verbose)
        lib = build_library(verbose)
        probe = probe.result()
    cli = build_cli(verbose)
    return {"lib": lib, "cli": cli, "probe": probe}


if __name__ == "__main__":
    print(build_all(verbose=True))
