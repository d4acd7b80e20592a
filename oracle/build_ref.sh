#!/usr/bin/env bash
# Build the reference program (ActFlow_V3-2.cu + its two headers) from its own
# source files, unmodified, into oracle/_ref/.  This is the checker's copy of the
# reference: tests and the golden-fixture script run it, the product never does.
#
# Usage: oracle/build_ref.sh [SOURCE_DIR [OUT_DIR]]
#   SOURCE_DIR defaults to /root/reference (the read-only mount of the reference
#   repository).  The reference's own makefile targets CUDA 9.1 / sm_35, so this
#   recipe calls nvcc directly for sm_103a and links cuFFT, as the reference
#   README describes (README.md:6-9).  OUT_DIR defaults to oracle/_ref; the
#   benchmark's timing copy goes to baseline/_ref/bin.
set -euo pipefail
SRC="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="${2:-$HERE/_ref}"
mkdir -p "$OUT"
if [ ! -f "$SRC/ActFlow_V3-2.cu" ]; then
  echo "build_ref: $SRC/ActFlow_V3-2.cu not found" >&2
  exit 2
fi
NVCC="${NVCC:-nvcc}"
"$NVCC" -std=c++11 -O2 -gencode arch=compute_103a,code=sm_103a \
  -I"$SRC" "$SRC/ActFlow_V3-2.cu" -lcufft -o "$OUT/ActFlow_ref" -w
echo "built $OUT/ActFlow_ref"
