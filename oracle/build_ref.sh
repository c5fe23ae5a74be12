#!/bin/sh
# Builds the psvWave reference's own solver core, unmodified, into
# oracle/_ref/libpsv_ref.so, for use as the checker of the oracle port and
# as the maker of golden fixtures. Test infrastructure only.
#
# Inputs: the reference sources src/fdModel.cpp and src/contiguous_arrays.cpp
# where they lie (REF_SRC, required: the reference checkout's src/ folder;
# oracle/build.py passes it), plus the stand-in
# headers for the reference's absent Eigen and inih submodules in
# oracle/ref_shim. Flags follow the reference's release build
# (CMakeLists.txt: -O3, OpenMP, C++11-compatible code).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ -z "$REF_SRC" ]; then
  echo "build_ref.sh: set REF_SRC to the reference checkout's src/ folder" >&2
  exit 2
fi
if [ ! -f "$REF_SRC/fdModel.cpp" ]; then
  echo "build_ref.sh: reference sources not found at $REF_SRC; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -O3 -fopenmp -std=c++14 -fPIC -shared -w \
  -I"$HERE/ref_shim" -I"$REF_SRC" \
  "$REF_SRC/fdModel.cpp" "$REF_SRC/contiguous_arrays.cpp" "$HERE/ref_shim/ref_capi.cpp" \
  -o "$OUT/libpsv_ref.so.tmp"
mv "$OUT/libpsv_ref.so.tmp" "$OUT/libpsv_ref.so"
echo "built $OUT/libpsv_ref.so"
