#!/usr/bin/env bash
# Builds oracle/_ref/libref_fdtd.so: the reference's own sources
# (src/gpu.h, src/simulation.h, src/simFDTD.cu, unmodified apart from the
# kernel-launch syntax) compiled for the host with g++, so that they run on
# the CPU.  TEST INFRASTRUCTURE ONLY: used to pin the oracle
# (tests/golden/make_golden.py), never by the product.
#
#   - oracle/ref_shim/ supplies cuda_runtime.h (host memory + a sequential
#     launch emulator) and a prologue; tests/mexstub/ supplies mex.h.
#   - The one rewrite is `k<<<cfg>>>(` -> `REF_LAUNCH(k, cfg)(`, applied while
#     streaming the sources into the compiler: no copy of the reference's
#     sources is written to disk.
#   - -ffp-contract=off keeps every float operation separately rounded, as in
#     the oracle; the reference's nvcc build may contract into FMA, which
#     moves results by rounding only.
#
# Usage: oracle/ref_build.sh <reference_root>   (or $MAXWELL_REF)
set -euo pipefail
REF="${1:-${MAXWELL_REF:-}}"
if [ -z "$REF" ]; then
  echo "usage: ref_build.sh <reference_root> (or set MAXWELL_REF)" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
STUB="$HERE/../tests/mexstub"
if [ ! -f "$REF/src/simulation.h" ]; then
  echo "ref_build: reference sources not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
gcc -O2 -fPIC -c "$STUB/mexstub.c" -I"$STUB" -o "$OUT/mexstub.o"
{
  echo '#include "ref_prologue.h"'
  echo "#line 1 \"$REF/src/gpu.h\""
  cat "$REF/src/gpu.h"
  echo "#line 1 \"$REF/src/simulation.h\""
  sed -e 's/^#include "gpu.h"//' \
      -e 's/\([A-Za-z_][A-Za-z0-9_]*\)<<<\([^>]*\)>>>/REF_LAUNCH(\1, \2)/g' \
      "$REF/src/simulation.h"
  echo "#line 1 \"$REF/src/simFDTD.cu\""
  sed -e 's/^#include "simulation.h"//' "$REF/src/simFDTD.cu"
  echo '#include "ref_harness.inc"'
} | g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -x c++ - \
      -I"$HERE/ref_shim" -I"$STUB" -x none "$OUT/mexstub.o" \
      -o "$OUT/libref_fdtd.so"
echo "ref_build: $OUT/libref_fdtd.so"
