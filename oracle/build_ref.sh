#!/usr/bin/env bash
# Compiles the reference's own `.pre` reader/writer and edge extractor, from
# the sources where they lie under the read-only reference checkout, into
# oracle/_ref/ref_pre_tool.  Only the two reference files the `.pre` producer
# path needs are compiled (plus this repository's driver); the reference's
# own build system is not used.  Outputs go to oracle/_ref/ only.
set -euo pipefail
REF=${PIERCE_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/pierce/common/include" ]; then
  echo "reference sources not present at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
g++ -O2 -std=c++17 -ffp-contract=off \
  -I"$REF/pierce/common/include" -I"$REF/pierce/preprocess/src" -I"$CUDA_INC" \
  "$HERE/ref_pre_tool.cpp" "$REF/pierce/preprocess/src/EdgePreprocessor.cpp" \
  -o "$OUT/ref_pre_tool"
echo "built $OUT/ref_pre_tool"
