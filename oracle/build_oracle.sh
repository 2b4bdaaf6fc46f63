#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
gcc -O2 -fopenmp -fPIC -shared -std=c11 -Wall -Wextra -o "$here/_build/libtc_oracle.so.tmp" "$here/tc_oracle.c"
mv -f "$here/_build/libtc_oracle.so.tmp" "$here/_build/libtc_oracle.so"
