#!/usr/bin/env bash
# Builds the reference's own CPU code for this path into oracle/_ref/libnrcref.so:
#   - test/main.cpp  Evaluate()/Train()  (Eigen fp16 MLP), via a stub device runtime
#   - shader/src/NRCRecord.glsl  NRCInputEncode()/NRCSphEncode(), compiled as C++ on glm
#   - shader/src/nrc_train_prepare.comp, nrc_optimize.comp and NN_nv.glsl's
#     NNLoadDA3_RelativeL2LuminanceLoss, turned into C++ text by glsl_to_cpp.py
#     (interface lines only) and compiled on glm
# Sources are read in place from the reference tree (REF_DIR; default
# /root/reference, else a reference tree mounted at baseline/_ref); nothing is
# copied into the repository. Outputs go only to oracle/_ref/. Exits 0 without
# building when no reference tree is found (a machine without the reference
# sources).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ -z "${REF_DIR:-}" ]; then
  REF_DIR=/root/reference
  if [ ! -f "$REF_DIR/test/main.cpp" ] && [ -f "$HERE/../../baseline/_ref/test/main.cpp" ]; then
    REF_DIR="$(cd "$HERE/../../baseline/_ref" && pwd)"
  fi
fi
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
PY="${PYTHON:-python3}"
SH="$REF_DIR/shader/src"
"$PY" "$HERE/glsl_to_cpp.py" compute "$SH/nrc_train_prepare.comp" ref_prepare_main "$OUT/nrc_train_prepare.inc"
"$PY" "$HERE/glsl_to_cpp.py" compute "$SH/nrc_optimize.comp" ref_optimize_main "$OUT/nrc_optimize.inc"
"$PY" "$HERE/glsl_to_cpp.py" function "$SH/NN_nv.glsl" NNLoadDA3_RelativeL2LuminanceLoss "$OUT/nn_loss.inc"
$CXX -std=gnu++20 -O2 -fsingle-precision-constant -ffp-contract=off -fPIC -w -c \
  -I"$REF_DIR/dep/glm/include" -I"$SH" -I"$OUT" "$HERE/ref_train.cpp" -o "$OUT/ref_train.o" &
wait
$CXX -shared -o "$OUT/libnrcref.so" "$OUT/ref_glsl.o" "$OUT/ref_eval.o" "$OUT/ref_train.o"
echo "build_ref: wrote $OUT/libnrcref.so"
