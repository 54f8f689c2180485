#!/usr/bin/env bash
# Builds the reference's own CPU trial-factoring engine (cutrialdive 1.2.0,
# CPU build) from its unmodified sources into oracle/_ref/cutrialdive_ref.
# The reference checkout is the first argument, else $CTD_REFERENCE_ROOT,
# else /root/reference.  Test infrastructure only: it pins the oracle
# and produces the committed golden factor files; nothing in the product
# loads it.
#
# The reference build needs two libraries that are not installed as
# development packages here; oracle/refshim/ provides our stand-ins:
#   - gmp.h: the documented mpz API bound to the installed GMP runtime
#     (libgmp.so.10);
#   - primesieve.hpp/.h: generate_primes() over the oracle's own sieve.
# The reference's CMake build is not run; its GPU, PRP (GWNUM) and LFP parts
# are not compiled.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${1:-${CTD_REFERENCE_ROOT:-/root/reference}}"
SRC="$REF_ROOT/src"
OUT="$HERE/_ref"
OBJ="$OUT/obj"
[ -d "$SRC" ] || { echo "reference sources not found at $SRC" >&2; exit 1; }
mkdir -p "$OBJ"
GMP_RT=$(ls /usr/lib/*-linux-gnu/libgmp.so.10 2>/dev/null | head -1 || true)
[ -n "$GMP_RT" ] || { echo "GMP runtime libgmp.so.10 not found" >&2; exit 1; }

CXXFLAGS=(-std=c++20 -O2 -DCUTRIALDIVE_HAS_PRIMESIEVE '-DCUTRIALDIVE_VERSION="1.2.0"'
          -I"$HERE/refshim" -I"$SRC" -w)
SOURCES=()
for f in "$SRC"/*.cpp "$SRC"/number_sequences/*.cpp; do
  case "$(basename "$f")" in
    prp.cpp) continue ;;   # needs GWNUM (CUTRIALDIVE_ENABLE_PRP only)
  esac
  SOURCES+=("$f")
done

compile() {
  local f="$1" o
  o="$OBJ/$(echo "${f#$SRC/}" | tr '/' '_').o"
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
    g++ "${CXXFLAGS[@]}" -c "$f" -o "$o"
  fi
  echo "$o"
}
export -f compile
export OBJ SRC
export CXXFLAGS_STR="${CXXFLAGS[*]}"

OBJS=()
pids=()
for f in "${SOURCES[@]}"; do
  o="$OBJ/$(echo "${f#$SRC/}" | tr '/' '_').o"
  OBJS+=("$o")
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
    g++ "${CXXFLAGS[@]}" -c "$f" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done

gcc -O2 -std=gnu11 -c "$HERE/ctd_oracle.c" -o "$OBJ/ctd_oracle.o"
g++ -o "$OUT/cutrialdive_ref" "${OBJS[@]}" "$OBJ/ctd_oracle.o" "$GMP_RT" -pthread
echo "$OUT/cutrialdive_ref"
