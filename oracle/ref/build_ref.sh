#!/usr/bin/env bash
# Builds the reference's own CPU code for this path into oracle/_ref/libnrcref.so:
#   - test/main.cpp  Evaluate()/Train()  (Eigen fp16 MLP), via a stub device runtime
#   - shader/src/NRCRecord.glsl  NRCInputEncode()/NRCSphEncode(), compiled as C++ on glm
# Sources are read in place from the reference tree (REF_DIR, default /root/reference);
# nothing is copied. Outputs go only to oracle/_ref/. Exits 0 without building when
# the reference tree is absent (the GPU machine never has it).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-/root/reference}"
OUT="$HERE/../_ref"
if [ ! -f "$REF_DIR/test/main.cpp" ] || [ ! -f "$REF_DIR/shader/src/NRCRecord.glsl" ]; then
  echo "build_ref: reference tree not found at $REF_DIR; skipping"
  exit 0
fi
mkdir -p "$OUT"
ARCHFLAGS=""
case "$(uname -m)" in
  x86_64) ARCHFLAGS="-mavx2 -mfma -mf16c" ;;
  aarch64) ARCHFLAGS="-mcpu=native" ;;
esac
CXX="${CXX:-g++}"
# GLSL float literals are single precision; glm arithmetic follows GLSL's float rules.
$CXX -std=gnu++20 -O2 -fsingle-precision-constant -ffp-contract=off -fPIC -w -c \
  -I"$REF_DIR/dep/glm/include" -I"$REF_DIR/shader/src" "$HERE/ref_glsl.cpp" -o "$OUT/ref_glsl.o" &
$CXX -std=gnu++20 -O3 $ARCHFLAGS -fPIC -w -c \
  -I"$HERE/stub" -I"$REF_DIR/test" -I"$REF_DIR/test/eigen" "$HERE/ref_eval.cpp" -o "$OUT/ref_eval.o" &
wait
$CXX -shared -o "$OUT/libnrcref.so" "$OUT/ref_glsl.o" "$OUT/ref_eval.o"
echo "build_ref: wrote $OUT/libnrcref.so"
