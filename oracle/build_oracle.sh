#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.  The
# engine's shared generator header (tc_gen_common.h) is included so that the
# oracle can draw the same seeded samples without loading the engine.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
gcc -O2 -fopenmp -fPIC -shared -std=c11 -Wall -Wextra \
    -I"$here/../hetegeneous_parallel_programming_gb300/csrc" \
    -o "$here/_build/libtc_oracle.so.tmp" "$here/tc_oracle.c" -lm
mv -f "$here/_build/libtc_oracle.so.tmp" "$here/_build/libtc_oracle.so"
