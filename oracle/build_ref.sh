#!/bin/sh
# Build the reference's own sources into oracle/_ref/libfmmref.so (test infrastructure).
#
# The reference (ZiqiFrancisFan/FMBEM_GPU_C) is compiled where it lies; nothing is copied.
# GSL is absent from this image, so the project-written shim in oracle/gsl_shim stands in
# for it.  Run only where the reference tree is mounted; the library is a checker used to
# generate tests/golden fixtures, never a product dependency.
set -e
REF=${FMMBEM_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/octree.c" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
nvcc -std=c++14 -x cu -rdc=true -gencode arch=compute_103a,code=sm_103a -O2 -DMAX=400000 \
     -Xcompiler -fPIC -Xcompiler -ffp-contract=off -shared -w \
     -I"$HERE/gsl_shim" -I"$REF" \
     "$HERE/ref_capi.cu" "$REF/octree.c" "$REF/structs.cu" "$REF/translation.cu" "$REF/integral.cu" \
     "$HERE/gsl_shim/gsl_shim.c" -lcurand -o "$OUT/libfmmref.so"
echo "built $OUT/libfmmref.so"
