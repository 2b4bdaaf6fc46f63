#!/usr/bin/env bash
# Builds oracle/_ref/libtc_ref.so from the reference's own sources, read where
# they lie (nothing is copied into this repository): the reference's
# successful_push_pull/graph.cc, unchanged, plus oracle/ref_driver.cc, with
# the un-vendored GraphMiner headers it includes (VertexSet.h, scan.h)
# supplied by oracle/ref_shim/.  TEST INFRASTRUCTURE ONLY.
#
# Usage: oracle/build_ref.sh [reference root]   (default /root/reference)
# Exits 0 without building when the reference tree is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-/root/reference}"
src="$ref/successful_push_pull"
if [ ! -f "$src/graph.cc" ]; then
  echo "build_ref.sh: $src/graph.cc not found; oracle/_ref not built" >&2
  exit 0
fi
mkdir -p "$here/_ref"
g++ -O2 -std=c++17 -fopenmp -fPIC -shared -w \
    -I"$here/ref_shim" -I"$src" \
    -o "$here/_ref/libtc_ref.so.tmp" "$src/graph.cc" "$here/ref_driver.cc"
mv -f "$here/_ref/libtc_ref.so.tmp" "$here/_ref/libtc_ref.so"
