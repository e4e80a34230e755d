#!/usr/bin/env bash
# Builds the test oracles (test infrastructure, not the product):
#   oracle/_build/liboracle.so   the C restatement (oracle/srs_oracle.c)
#   oracle/_ref/libsrsref.so     the reference's own cpu/RunSimulation.cpp,
#                                compiled where it lies under REF_ROOT, with
#                                oracle/ref_harness.cpp as its driver
#   oracle/_ref/libsrsref_io.so  the reference's own cpu/InitFuncs.cpp and
#                                cpu/OutputFuncs.cpp with oracle/ref_io_harness.cpp
#   oracle/_ref/linescan         the reference's line-scan tool linescan/main.cpp
# The last three are built only when the reference tree is present.  The
# reference's input/output files and its line-scan tool need MPI and Xerces-C;
# they compile against oracle/shim/ instead: a single-rank MPI stand-in and
# the subset of the Xerces DOM API they call.  Nothing of the reference's own
# build system (or of the vendored Xerces) is run.
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
      -o "$HERE/_ref/libsrsref.so" -lm &
  pids=($!)
  if [ -f "$REF_ROOT/cpu/InitFuncs.cpp" ] && [ -f "$REF_ROOT/cpu/OutputFuncs.cpp" ]; then
    g++ -O2 -fPIC -shared -ffp-contract=off -w -I "$HERE/shim" -I "$REF_ROOT/cpu" \
        "$REF_ROOT/cpu/InitFuncs.cpp" "$REF_ROOT/cpu/OutputFuncs.cpp" "$HERE/ref_io_harness.cpp" \
        -o "$HERE/_ref/libsrsref_io.so" -Wl,--no-undefined -lm &
    pids+=($!)
  fi
  if [ -f "$REF_ROOT/linescan/main.cpp" ]; then
    g++ -O2 -ffp-contract=off -w -I "$HERE/shim" -I "$REF_ROOT/linescan" \
        "$REF_ROOT/linescan/main.cpp" -o "$HERE/_ref/linescan" -lm &
    pids+=($!)
  fi
  for p in "${pids[@]}"; do wait "$p"; done
fi
