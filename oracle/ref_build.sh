#!/usr/bin/env bash
# Build the reference's own device code (NCCA/libfluid cudasrc, read where it
# lies) into oracle/_ref/libfluid_ref.cubin for sm_103a, and list the mangled
# names of its four __global__ kernels (from the symbol table of a host
# object of the same translation unit) in oracle/_ref/kernels.txt.
# Outputs go to oracle/_ref/ only; nothing is copied from the reference tree.
# Usage: oracle/ref_build.sh [reference root]   (default $LIBFLUID_REFERENCE, else /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${LIBFLUID_REFERENCE:-/root/reference}}"
OUT="$HERE/_ref"
NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
if [ ! -d "$REF/libfluid/cudasrc" ]; then
    echo "reference tree not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
INC=(-I"$HERE/ref_compat" -I"$REF/libfluid/include" -I"$REF/common/include" -I"$REF/libfluid/cudasrc")
FLAGS=(-std=c++17 -O3 -gencode arch=compute_103a,code=sm_103a -w)
"$NVCC" "${FLAGS[@]}" "${INC[@]}" -cubin "$HERE/ref_unity.cu" -o "$OUT/libfluid_ref.cubin"
"$NVCC" "${FLAGS[@]}" "${INC[@]}" -rdc=true -c "$HERE/ref_unity.cu" -o "$OUT/ref_unity_host.o"
nm "$OUT/ref_unity_host.o" | awk '{print $NF}' \
  | grep -E '^_Z[0-9]+(computeDensity|computeNormals|computeAllForces|correctVelocityXSPH)[A-Za-z0-9_]*$' \
  | sort -u > "$OUT/kernels.txt"
rm -f "$OUT/ref_unity_host.o"
test "$(wc -l < "$OUT/kernels.txt")" -eq 4
echo "built $OUT/libfluid_ref.cubin"
