#!/bin/sh
# Stage the reference's sources for its CPU solver path (tools/enumerate.c
# and what it links: src/vm.c, src/asm.c, src/search_state.c, tasks/spec.c
# and their headers) and for its hybrid CPU/GPU solver (gpu/hybrid.cu) into
# baseline/_ref/src, which git ignores, so that the
# reference can be compiled from them on a machine without the reference
# tree (oracle/build_ref.sh; oracle/build.py does it when the staged copy
# exists). Nothing staged is committed.
#
#   oracle/stage_ref.sh REFERENCE_ROOT      (or $PCA_REFERENCE_ROOT set)
set -e
REF=${1:-${PCA_REFERENCE_ROOT:-}}
HERE=$(cd "$(dirname "$0")" && pwd)
DEST="$HERE/../baseline/_ref/src"
if [ -z "$REF" ] || [ ! -f "$REF/tools/enumerate.c" ]; then
    echo "stage_ref: no reference tree given; nothing staged" >&2
    exit 0
fi
mkdir -p "$DEST/src" "$DEST/tasks" "$DEST/tools" "$DEST/gpu"
for f in src/vm.c src/asm.c src/search_state.c src/pca.h src/search_state.h \
         tasks/spec.c tasks/spec.h tools/enumerate.c tools/gen_tasks.c gpu/hybrid.cu; do
    cp "$REF/$f" "$DEST/$f"
done
echo "stage_ref: staged the reference's solver sources in $DEST"
