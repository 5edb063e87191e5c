#!/bin/sh
# Compile the reference's own CUDA kernels, unmodified and where they lie,
# into device-only cubins for sm_103a, plus the parameter-layout header the
# harness needs.  Outputs go to oracle/_ref/ only (git-ignored; the cubins are
# device code and travel to the GPU machine).  Include paths as in
# solver/mix3d.mk (../include and ../src).  Needs the reference sources, so it
# runs on the build host, not on the GPU machine.
# The reference's location is REF (this recipe's default is the read-only
# mount of the build host); without its sources the recipe does nothing, so
# it can run anywhere (the GPU machine has no reference and uses the cubins built
# here).
set -e
REF=${REF:-/root/reference}
if [ ! -f "$REF/solver/cuDeriv.cu" ]; then
    echo "reference sources not found under REF=$REF: nothing to build"
    exit 0
fi
HERE=$(cd "$(dirname "$0")/.." && pwd)
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
mkdir -p "$OUT"
for f in solver/cuDeriv.cu solver/cuDivergence.cu src/LevelSet/lsTools.cu src/LevelSet/extrapol.cu; do
    b=$(basename "$f" .cu)
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 \
        -I"$REF/include" -I"$REF/src" -o "$OUT/ref_$b.cubin" "$REF/$f" 2> "$OUT/ref_$b.log"
done
"$NVCC" -O0 -I"$REF/include" -I"$REF/src" -o "$OUT/layout_probe" "$HERE/ref/layout_probe.cu" 2> "$OUT/layout_probe.log"
"$OUT/layout_probe" > "$OUT/arraydev_layout.h"
rm -f "$OUT/layout_probe"
echo "reference cubins and layout header in $OUT"
