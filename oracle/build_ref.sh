#!/usr/bin/env bash
# Build recipe for the reference kd-tree builder (TEST INFRASTRUCTURE ONLY).
#
# Compiles the reference's own builder translation units where they lie in
# the reference tree -- Kd-treeConstructor.cpp, Kd-treeConverter.cpp and
# MyMathUtility.cpp -- with oracle/ref_shim.h force-included, links them with
# oracle/ref_kdbuild.cpp, and writes the binary to oracle/_ref/ref_kdbuild.
# Nothing is copied out of the reference tree.  Only this recipe and the
# tests that call the binary read the reference location; the product never
# does.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   The reference checkout comes from the argument or, without one, from the
#   KDGR_REFERENCE_ROOT environment variable.  The script exits 0 and builds
#   nothing when neither names a tree holding the builder sources (the
#   prebuilt binary, if any, is used instead).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${KDGR_REFERENCE_ROOT:-}}"
KC="$REF/Kd-treeConverter_v0.9/Kd-treeConverter"
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$KC/Kd-treeConstructor.cpp" ]; then
  echo "build_ref: reference sources not given or not present (argument or KDGR_REFERENCE_ROOT); skipped"
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
# -ffp-contract=off: no fused multiply-add, as the reference's MSVC x64
# build (no /fp:contract) computes; the product builder uses the same flag.
# -fkeep-inline-functions: setInnerNode is declared inline in
# Kd-treeConstructor.h:84 but defined only in Kd-treeConstructor.cpp and
# called from Kd-treeConverter.cpp (MSVC emits it anyway; GCC needs the flag).
FLAGS=(-std=c++17 -O2 -fopenmp -ffp-contract=off -fkeep-inline-functions -w -I"$KC" -include "$HERE/ref_shim.h")
pids=()
for f in Kd-treeConstructor Kd-treeConverter MyMathUtility; do
  "$CXX" "${FLAGS[@]}" -c "$KC/$f.cpp" -o "$OUT/$f.o" &
  pids+=($!)
done
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_kdbuild.cpp" -o "$OUT/ref_kdbuild.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -fopenmp -o "$OUT/ref_kdbuild" "$OUT"/Kd-treeConstructor.o "$OUT"/Kd-treeConverter.o \
  "$OUT"/MyMathUtility.o "$OUT"/ref_kdbuild.o
echo "build_ref: $OUT/ref_kdbuild"
