#!/bin/sh
# Compile the reference's own CPU solver and its libpca.so from the reference
# sources, in place, into oracle/_ref/ (git-ignored). Used only as a checker:
# tests and golden-fixture generation compare against these outputs. Where
# nvcc is present, also its hybrid CPU/GPU solver gpu/hybrid.cu for sm_103a
# (gpu_hybrid), which the benchmark's reference arm times as the reference's
# GPU baseline; a failure there leaves the CPU builds in place.
#
#   oracle/build_ref.sh REFERENCE_ROOT
#
# REFERENCE_ROOT is the argument, else $PCA_REFERENCE_ROOT. Without a
# reference tree there, this script exits 0 and builds nothing.
set -e
REF=${1:-${PCA_REFERENCE_ROOT:-}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/tools/enumerate.c" ]; then
    echo "build_ref: no reference tree at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
CFLAGS="-O2 -std=c99 -w"
gcc $CFLAGS -o "$OUT/enumerate" \
    "$REF/src/vm.c" "$REF/src/asm.c" "$REF/src/search_state.c" \
    "$REF/tasks/spec.c" "$REF/tools/enumerate.c"
gcc $CFLAGS -shared -fPIC -o "$OUT/libpca.so" \
    "$REF/src/vm.c" "$REF/src/asm.c" "$REF/src/search_state.c" "$REF/tasks/spec.c"
gcc $CFLAGS -o "$OUT/gen_tasks" \
    "$REF/src/vm.c" "$REF/src/asm.c" "$REF/src/search_state.c" \
    "$REF/tasks/spec.c" "$REF/tools/gen_tasks.c"
NVCC=$(command -v nvcc || echo "${CUDA_HOME:-/usr/local/cuda}/bin/nvcc")
if [ -f "$REF/gpu/hybrid.cu" ] && [ -x "$NVCC" ]; then
    "$NVCC" -O3 -w -gencode arch=compute_103a,code=sm_103a -o "$OUT/gpu_hybrid" \
        "$REF/gpu/hybrid.cu" "$REF/tasks/spec.c" "$REF/src/vm.c" "$REF/src/asm.c" \
        || { rm -f "$OUT/gpu_hybrid"; echo "build_ref: gpu_hybrid not built" >&2; }
fi
uname -m > "$OUT/.machine"
echo "build_ref: built $OUT/enumerate $OUT/libpca.so $OUT/gen_tasks"
