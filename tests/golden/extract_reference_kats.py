"""Extracts the reference's known-answer tables into reference_kats.json.

Reads the cutrialdive test and self-test sources (read as text, never
compiled or run) and writes the tables the oracle is pinned to:

* mu64 / mu128 / mul128hi cases  -- tests/test_modular.cpp:55-185
* sieve known answers            -- src/autotests.cpp:136-351
* Smarandache value tables       -- tests/smarandache_tests.cpp:45-310
  (literal values, or the naive concatenation the test computes)

Usage: python tests/golden/extract_reference_kats.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def c_int_expr(expr: str) -> int:
    """Evaluate a C++ integer constant expression of literals, shifts and + - * ( )."""
    def lit(m: re.Match) -> str:
        t = m.group(1)
        if t.startswith(("0x", "0X")):
            return str(int(t, 16))
        if t.startswith(("0b", "0B")):
            return str(int(t[2:], 2))
        if len(t) > 1 and t.startswith("0"):  # C++ octal literal
            return str(int(t, 8))
        return t

    e = expr.replace("'", "")
    e = re.sub(r"\b(0[xX][0-9a-fA-F]+|0[bB][01]+|\d+)(?:ull|ul|u|ll|ULL|UL|U|LL)?\b", lit, e)
    e = re.sub(r"uint64_t\((.*?)\)", r"(\1)", e)
    if not re.fullmatch(r"[0-9a-fA-Fxb()+\-*<> ]+", e):
        raise ValueError(f"unsupported expression: {expr!r}")
    return int(eval(e, {"__builtins__": {}}))  # noqa: S307 - restricted to integer literals/operators


def u128(expr: str) -> int:
    m = re.fullmatch(r"\s*\(__uint128_t\{(0x[0-9a-fA-F]+)(?:ull)?\}\s*<<\s*64\)\s*\|\s*(0x[0-9a-fA-F]+)ull\s*", expr)
    if m:
        return (int(m.group(1), 16) << 64) | int(m.group(2), 16)
    return c_int_expr(expr)


def split_top(s: str) -> list[str]:
    """Split on top-level commas."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [x.strip() for x in out]


def table_rows(text: str, start_marker: str) -> list[tuple[int, str]]:
    """(line, row) for each `{ ... }` row of the to_array table after a marker."""
    i = text.index(start_marker)
    j = text.index("});", i)
    body_start = text.index("({", i) + 2
    body = text[body_start:j]
    rows, depth, cur, line0 = [], 0, "", text[:body_start].count("\n") + 1
    line = line0
    row_line = line
    for ch in body:
        if ch == "\n":
            line += 1
        if ch == "{":
            if depth == 0:
                cur = ""
                row_line = line
                depth += 1
                continue
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth == 0:
                rows.append((row_line, cur))
                continue
        if depth > 0:
            cur += ch
    return rows


FINGERPRINT_PRIMES = [1000003, 4294967291, 18446744073709551557]


def fingerprint(v: int) -> dict:
    """Exact identity of a big value without storing it: bit length, SHA-256
    of its little-endian bytes, and residues mod a few primes."""
    import hashlib

    nbytes = max(1, (v.bit_length() + 7) // 8)
    return {"bits": v.bit_length(),
            "sha256_le": hashlib.sha256(v.to_bytes(nbytes, "little")).hexdigest(),
            "mod": {str(p): v % p for p in FINGERPRINT_PRIMES}}


def naive_smarandache(base: int, n: int) -> int:
    v = 0
    for i in range(1, n + 1):
        d, m = 1, i
        while m >= base:
            m //= base
            d += 1
        v = v * base**d + i
    return v


def extract(ref_root: str) -> dict:
    tm = open(os.path.join(ref_root, "tests/test_modular.cpp")).read()
    mu64 = []
    for line, row in table_rows(tm, '"[barrett][mu64]"'):
        p, mu = split_top(row)
        mu64.append({"p": c_int_expr(p), "mu": c_int_expr(mu), "src": f"tests/test_modular.cpp:{line}"})
    mu128 = []
    for line, row in table_rows(tm, '"[barrett][mu128]"'):
        p, mu = split_top(row)
        mu128.append({"p": c_int_expr(p), "mu": str(u128(mu)), "src": f"tests/test_modular.cpp:{line}"})
    mulhi = []
    for line, row in table_rows(tm, '"[mulhi128]"'):
        a, b, r = split_top(row)
        mulhi.append({"a": str(u128(a)), "b": str(u128(b)), "hi": str(u128(r)), "src": f"tests/test_modular.cpp:{line}"})

    at = open(os.path.join(ref_root, "src/autotests.cpp")).read()
    sieve = []
    for m in re.finditer(r"auto primes = sieve\((.*?)\);", at):
        line = at[: m.start()].count("\n") + 1
        args = split_top(m.group(1))
        s_assign = None
        if "s - 1" in args[0]:
            sm = re.search(r"auto s = (.*?);", at[: m.start()][-200:])
            s_assign = c_int_expr(sm.group(1))
        lo = c_int_expr(args[0].replace("s", str(s_assign))) if s_assign is not None else c_int_expr(args[0])
        hi = c_int_expr(args[1].replace("s", str(s_assign))) if s_assign is not None else c_int_expr(args[1])
        block = at[m.end(): at.find("auto primes = sieve(", m.end()) if at.find("auto primes = sieve(", m.end()) > 0 else len(at)]
        case = {"lo": lo, "hi": hi, "src": f"src/autotests.cpp:{line}"}
        em = re.search(r"expected\s*=\s*\{(.*?)\};", block, re.S)
        if em:
            case["expected"] = [c_int_expr(x) for x in split_top(em.group(1))]
        cm = re.search(r"expectedCount\s*=\s*(\d+);", block)
        if cm:
            case["count"] = int(cm.group(1))
        if "primes.size()) {" in block and "expected" not in case and "count" not in case:
            case["count"] = 0  # `if (primes.size())` -> none expected
        um = re.search(r"primes.size\(\) != 1 \|\| primes.front\(\) != (\d+)", block)
        if um:
            case["expected"] = [int(um.group(1))]
        sieve.append(case)

    st = open(os.path.join(ref_root, "tests/smarandache_tests.cpp")).read()
    sm_values = []
    for m in re.finditer(r"ctd::smarandache<(\d+)>::value\(tc\.n\)", st):
        base = int(m.group(1))
        start = st.rfind("std::to_array<sm_value_case>", 0, m.start())
        for line, row in table_rows(st[start - 1:], "std::to_array<sm_value_case>"):
            n_s, v_s = split_top(row)
            n = c_int_expr(n_s)
            vm = re.fullmatch(r"IntT\{uint64_t\{(.*)\}\}", v_s)
            sv = re.fullmatch(r'IntT\{"(\d+)"\}', v_s)
            nv = re.fullmatch(r"smarandache\((\d+),\s*(\d+)\)", v_s)
            if vm:
                val = c_int_expr(vm.group(1))
            elif sv:
                val = int(sv.group(1))
            elif nv:
                val = naive_smarandache(int(nv.group(1)), int(nv.group(2)))
            else:
                raise ValueError(v_s)
            real_line = st[:start].count("\n") + line
            sm_values.append({"base": base, "n": n, **fingerprint(val),
                              "src": f"tests/smarandache_tests.cpp:{real_line}"})
    return {"mu64": mu64, "mu128": mu128, "mul128hi": mulhi, "sieve": sieve, "smarandache_values": sm_values}


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CTD_REFERENCE_ROOT", "/root/reference")
    data = extract(root)
    out = os.path.join(HERE, "reference_kats.json")
    with open(out, "w") as fh:
        json.dump(data, fh, indent=1)
    print({k: len(v) for k, v in data.items()}, "->", out)
