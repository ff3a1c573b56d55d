#!/bin/sh
# build_ref.sh - builds oracle/_ref/ from the reference sources, for checking.
#
# TEST INFRASTRUCTURE.  Where the reference tree is present (REF below), the
# kernel bodies are cut from it by line range after a sha256 check of
# the file, together with its SimulationParams.h, into oracle/_ref/ (which
# git ignores, so no reference source enters the repository).  Whenever those
# pieces are present, it compiles:
#   oracle/_ref/libcfref.so      host build (ref_host_shim.cu), FP32 oracle
#                                and timed CPU baseline
#   oracle/_ref/libcfref_gpu.so  sm_103a build (ref_gpu_shim.cu), the
#                                reference kernel timed on the GPU
# Usage: oracle/build_ref.sh [--no-gpu]
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
# the reference checkout: $CELLFLOW_REFERENCE, else `reference` beside this repository
REF=${CELLFLOW_REFERENCE:-$HERE/../../reference}
SRC="$REF/cuda-native/src/ParticleSimulation.cu"
HDR="$REF/cuda-native/include/SimulationParams.h"
SRC_SHA=ce1da0c9b70d91365ead243f87d12a363f21474272e6b89410b45030274f7fcd
HDR_SHA=de03cdbb2ebedd1653f81e402e7b67e7c5d9c3356a8c0a8681533872d1d59d3b
NVCC=${NVCC:-nvcc}
WANT_GPU=1
[ "${1:-}" = "--no-gpu" ] && WANT_GPU=0

mkdir -p "$OUT"
if [ -f "$SRC" ] && [ -f "$HDR" ]; then
    echo "$SRC_SHA  $SRC" | sha256sum -c --quiet -
    echo "$HDR_SHA  $HDR" | sha256sum -c --quiet -
    sed -n '69,166p' "$SRC" > "$OUT/ref_step_kernel.inc"
    sed -n '188,277p' "$SRC" > "$OUT/ref_prox_kernel.inc"
    sed -n '280,424p' "$SRC" > "$OUT/ref_mesh_kernel.inc"
    sed -n '521,531p' "$SRC" > "$OUT/ref_force_table.inc"
    rm -f "$OUT/SimulationParams.h"
    cp "$HDR" "$OUT/SimulationParams.h"
    chmod u+w "$OUT/SimulationParams.h"
fi

if [ ! -f "$OUT/ref_step_kernel.inc" ]; then
    echo "build_ref: reference pieces absent; oracle/_ref not built" >&2
    exit 0
fi

"$NVCC" -O3 -std=c++17 -shared -Xcompiler -fPIC,-O3,-ffp-contract=off,-fopenmp \
    -I"$OUT" "$HERE/ref_host_shim.cu" -o "$OUT/libcfref.so.tmp" -lgomp
mv "$OUT/libcfref.so.tmp" "$OUT/libcfref.so"

if [ "$WANT_GPU" = 1 ]; then
    "$NVCC" -O3 -std=c++17 -shared -Xcompiler -fPIC \
        -gencode arch=compute_103a,code=sm_103a -lineinfo \
        -I"$OUT" "$HERE/ref_gpu_shim.cu" -o "$OUT/libcfref_gpu.so.tmp"
    mv "$OUT/libcfref_gpu.so.tmp" "$OUT/libcfref_gpu.so"
fi
echo "build_ref: built $OUT"
