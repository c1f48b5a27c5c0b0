#!/usr/bin/env bash
# Build the reference library (ComputationalRobotics/psd_projection) from its
# own sources with nvcc, without its CMake (whose unconditional googletest
# FetchContent cannot run offline).  Output only into oracle/_ref/.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# REFERENCE_ROOT: the argument, else $PSDGB_REFERENCE_ROOT, else the
# read-only checkout this recipe was written for.
# The result is used by the tests to compare exported C++ symbols; it is a
# CUDA library and is never part of the product path.
set -euo pipefail
REF="${1:-${PSDGB_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT/obj"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
FLAGS=(-std=c++14 -O2 -Xcompiler -fPIC -gencode arch=compute_103a,code=sm_103a -I "$REF/include")
pids=()
for f in "$REF"/src/*.cu; do
  b="$(basename "$f" .cu)"
  "$NVCC" "${FLAGS[@]}" -c "$f" -o "$OUT/obj/$b.o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -shared -gencode arch=compute_103a,code=sm_103a -o "$OUT/libpsd_ref.so" "$OUT"/obj/*.o -lcublas -lcusolver -lcurand
nm -D --defined-only "$OUT/libpsd_ref.so" | awk '$2 == "T" {print $3}' | sort > "$OUT/symbols.txt"
echo "built $OUT/libpsd_ref.so"
