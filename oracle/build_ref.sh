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

# Grid statistics: generateGridStats shares its file with the reference
# preprocessor's main() (which needs tinyobjloader, absent), so the lines
# holding the function and its helpers are copied into a temporary
# directory outside this repository and included by ref_grid_tool.cpp.
SRC="$REF/pierce/preprocess/src/pierce_preprocess.cpp"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
sed -n '28,167p' "$SRC" > "$TMP/ref_grid_stats.inc"
# the extracted lines must start at the helpers and end with the function
head -1 "$TMP/ref_grid_stats.inc" | grep -q '#include <cmath>' &&
  grep -q '^void generateGridStats' "$TMP/ref_grid_stats.inc" &&
  tail -1 "$TMP/ref_grid_stats.inc" | grep -q '^}' || {
  echo "pierce_preprocess.cpp:28-167 is not generateGridStats with its helpers; skipping ref_grid_tool" >&2
  exit 0
}
g++ -O2 -std=c++17 -ffp-contract=off \
  -I"$REF/pierce/common/include" -I"$REF/pierce/preprocess/src" -I"$CUDA_INC" -I"$TMP" \
  "$HERE/ref_grid_tool.cpp" -o "$OUT/ref_grid_tool"
echo "built $OUT/ref_grid_tool"

# Grid selectivity estimate: the kernel (estimated_overlap.cu:8-41), the
# global averages (pierce_overlap_main.cpp:189-219) and the estimatePairs
# lambda of main() (pierce_overlap_main.cpp:376-471), copied into the same
# temporary directory and included by ref_estimate_tool.cpp.
KSRC="$REF/pierce/query/src/cuda/estimated_overlap.cu"
ASRC="$REF/pierce/query/src/applications/pierce_overlap_main.cpp"
sed -n '8,41p' "$KSRC" > "$TMP/ref_estimate_kernel.inc"
sed -n '189,219p' "$ASRC" > "$TMP/ref_estimate_helpers.inc"
sed -n '376,471p' "$ASRC" > "$TMP/ref_estimate_pairs.inc"
grep -q '^__global__ void estimateSelectivityKernel' "$TMP/ref_estimate_kernel.inc" &&
  tail -1 "$TMP/ref_estimate_kernel.inc" | grep -q '^}' &&
  grep -q '^float calculateGlobalAvgSize' "$TMP/ref_estimate_helpers.inc" &&
  grep -q '^float calculateGlobalAvgVolRatio' "$TMP/ref_estimate_helpers.inc" &&
  head -1 "$TMP/ref_estimate_pairs.inc" | grep -q 'auto estimatePairs = ' &&
  tail -1 "$TMP/ref_estimate_pairs.inc" | grep -q '^    };' || {
  echo "the estimate's source lines moved; skipping ref_estimate_tool" >&2
  exit 0
}
g++ -O2 -std=c++17 -ffp-contract=off \
  -I"$REF/pierce/common/include" -I"$CUDA_INC" -I"$TMP" \
  "$HERE/ref_estimate_tool.cpp" -o "$OUT/ref_estimate_tool"
echo "built $OUT/ref_estimate_tool"
