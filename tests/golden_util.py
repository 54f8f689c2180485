"""Helpers shared by the parity tests: parsing the golden-file command
lines and rebuilding full factor files from their sparse form."""
from __future__ import annotations

import hashlib

FAMILY_IDS = {"mersenne": 0, "proth": 1, "riesel": 2, "smarandache": 3, "fibonacci": 4, "lucas": 5,
              "proth_fixed_n": 6, "riesel_fixed_n": 7, "tribonacci": 8}


def parse_args(args: str) -> dict:
    """The subset of the CLI the golden cases use -> job fields."""
    toks = args.split()
    d = {"max_factors": 32}
    i = 0
    while i < len(toks):
        t = toks[i]
        v = toks[i + 1] if i + 1 < len(toks) else None
        if t == "--num-seq":
            name, _, params = v.partition(",")
            d["family"] = FAMILY_IDS[name]
            d["spec"] = (name, params)
            if name == "smarandache":
                d["param"] = int(params) if params else 10
            elif name in ("mersenne", "fibonacci", "lucas", "tribonacci"):
                d["param"] = 0
            else:
                d["param"] = int(params)
        elif t == "-s":
            d["n0"] = int(v)
        elif t == "-e":
            d["n1"] = int(v)
        elif t == "--tf-bits":
            d["f0"], d["f1"] = 2, (1 << int(v)) if int(v) < 64 else 2**64 - 1
        elif t == "--tf-start":
            d["f0"] = int(v)
        elif t == "--tf-end":
            d["f1"] = int(v)
        elif t == "--max-factors-per-number":
            d["max_factors"] = int(v)
        i += 2
    return d


def expand(n0: int, n1: int, nonempty: list) -> str:
    by_n = {int(ln.split(" - ", 1)[0]): ln for ln in nonempty}
    return "".join(by_n.get(n, f"{n} - ") + "\n" for n in range(n0, n1))


def sha256(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()
