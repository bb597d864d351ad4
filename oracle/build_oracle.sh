#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so, and the
# reference's own CPU code into oracle/_ref/ when the reference tree is present.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
CC="${CC:-gcc}"
$CC -std=c11 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
  "$HERE/nrc_oracle.c" "$HERE/nrc_trace_oracle.c" -o "$HERE/_build/liboracle.so.tmp" -lm
mv -f "$HERE/_build/liboracle.so.tmp" "$HERE/_build/liboracle.so"
"$HERE/ref/build_ref.sh"
