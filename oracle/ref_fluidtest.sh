#!/usr/bin/env bash
# Compile the reference's own fluidtest sources (test/src/main.cpp and
# test/src/myfluidsystem.cpp, read where they lie) unchanged against this
# repository's FluidSystem drop-in (include/fluidsystem.h) and link them with
# libfluid.so: the drop-in proof.  Also builds oracle/_ref/geo_check, which
# links the reference's dumpToGeo (main renamed) to compare .geo output.
# Outputs go to oracle/_ref/ only.
# Usage: oracle/ref_fluidtest.sh [reference root]   (default $LIBFLUID_REFERENCE, else /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$HERE")"
REF="${1:-${LIBFLUID_REFERENCE:-/root/reference}}"
OUT="$HERE/_ref"
CUDA="${CUDA_HOME:-/usr/local/cuda}"
CXX="${CXX:-g++}"
if [ ! -f "$REF/test/src/main.cpp" ]; then
    echo "reference tree not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
INC=(-I"$HERE/ref_compat" -I"$ROOT/include" -I"$CUDA/include" -I"$REF/test/src")
LIBS=(-L"$ROOT/libfluid_gb300" -lfluid -lsph_gb300 -Wl,-rpath,"$ROOT/libfluid_gb300")
"$CXX" -std=c++14 -O1 -w "${INC[@]}" "$REF/test/src/main.cpp" "$REF/test/src/myfluidsystem.cpp" \
    -o "$OUT/ref_fluidtest" "${LIBS[@]}"
"$CXX" -std=c++14 -O1 -w "${INC[@]}" -Dmain=reference_fluidtest_main -c "$REF/test/src/main.cpp" -o "$OUT/ref_main.o"
"$CXX" -std=c++14 -O1 -w "${INC[@]}" -c "$REF/test/src/myfluidsystem.cpp" -o "$OUT/ref_myfluidsystem.o"
"$CXX" -std=c++14 -O1 -w "${INC[@]}" "$HERE/geo_check.cpp" "$OUT/ref_main.o" "$OUT/ref_myfluidsystem.o" \
    -o "$OUT/geo_check" "${LIBS[@]}"
rm -f "$OUT/ref_main.o" "$OUT/ref_myfluidsystem.o"
echo "built $OUT/ref_fluidtest and $OUT/geo_check"
