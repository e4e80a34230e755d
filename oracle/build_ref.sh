#!/usr/bin/env bash
# Builds the test oracles (test infrastructure, not the product):
#   oracle/_build/liboracle.so  the C restatement (oracle/srs_oracle.c)
#   oracle/_ref/libsrsref.so    the reference's own cpu/RunSimulation.cpp,
#                               compiled where it lies under REF_ROOT, with
#                               oracle/ref_harness.cpp as its driver.
# The second library is built only when the reference tree is present.
# -ffp-contract=off keeps x86-64 and aarch64 builds bit-identical.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${SRS_REFERENCE_ROOT:-/root/reference}"
mkdir -p "$HERE/_build"
gcc -std=c99 -O2 -fPIC -shared -ffp-contract=off -D_DEFAULT_SOURCE \
    "$HERE/srs_oracle.c" -o "$HERE/_build/liboracle.so" -lm
if [ -f "$REF_ROOT/cpu/RunSimulation.cpp" ] && [ -f "$REF_ROOT/cpu/parameters.h" ]; then
  mkdir -p "$HERE/_ref"
  g++ -O2 -fPIC -shared -ffp-contract=off -w -I "$REF_ROOT/cpu" \
      "$REF_ROOT/cpu/RunSimulation.cpp" "$HERE/ref_harness.cpp" \
      -o "$HERE/_ref/libsrsref.so" -lm
fi
