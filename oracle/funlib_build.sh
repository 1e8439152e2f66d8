#!/usr/bin/env bash
# Builds oracle/_ref/libref_funlib.so: the reference's source-waveform MEX
# file (src/cpucode/FunLib.cpp, unmodified) compiled for the host with g++
# against the test MEX stand-in (tests/mexstub).  TEST INFRASTRUCTURE ONLY:
# tests/golden/make_funlib_golden.py drives its mexFunction to pin
# fdtd_create_signal; the product never loads it.
#
# Usage: oracle/funlib_build.sh <reference_root>   (or $MAXWELL_REF)
set -euo pipefail
REF="${1:-${MAXWELL_REF:-}}"
if [ -z "$REF" ]; then
  echo "usage: funlib_build.sh <reference_root> (or set MAXWELL_REF)" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
STUB="$HERE/../tests/mexstub"
if [ ! -f "$REF/src/cpucode/FunLib.cpp" ]; then
  echo "funlib_build: $REF/src/cpucode/FunLib.cpp not found" >&2
  exit 2
fi
mkdir -p "$OUT"
gcc -O2 -fPIC -c "$STUB/mexstub.c" -I"$STUB" -o "$OUT/mexstub_funlib.o"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -I"$STUB" \
    "$REF/src/cpucode/FunLib.cpp" "$OUT/mexstub_funlib.o" -o "$OUT/libref_funlib.so"
echo "funlib_build: $OUT/libref_funlib.so"
