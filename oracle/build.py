"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Produces ``oracle/libctd_oracle.so`` from ``ctd_oracle.c`` with gcc, and --
when the read-only reference checkout is present -- the reference's own CPU
engine under ``oracle/_ref/`` (see ``build_ref.sh``).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libctd_oracle.so")
# the reference checkout: $CTD_REFERENCE_ROOT, else /root/reference
REF_ROOT = os.environ.get("CTD_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")


def build_oracle(verbose: bool = False) -> str:
    src = os.path.join(HERE, "ctd_oracle.c")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "ctd_oracle.h"))
    ):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu11", "-shared", "-fPIC", "-pthread", "-Wall",
           "-o", LIB + ".tmp", src]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_reference(verbose: bool = False) -> str | None:
    """Compile the reference CPU engine when its sources are mounted here."""
    if not os.path.isdir(REF_SRC):
        return None
    script = os.path.join(HERE, "build_ref.sh")
    out = os.path.join(HERE, "_ref", "cutrialdive_ref")
    try:
        subprocess.check_call(["bash", script, REF_ROOT], stdout=None if verbose else subprocess.DEVNULL)
    except (subprocess.CalledProcessError, FileNotFoundError) as exc:  # pragma: no cover
        print(f"oracle/_ref: reference build failed: {exc}", file=sys.stderr)
        return None
    return out if os.path.exists(out) else None


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference(verbose=True))
