#!/usr/bin/env bash
# Builds checkers from the reference's own sources, in place, into oracle/_ref/
# (git-ignored).  Test infrastructure only; needs the reference tree at $REF
# (default: ../reference relative to the repository root).
#
#   undir2dir             preprocess_CPU/Undir2Dir.c, the reference's CPU degree
#                         orientation (pins oracle.c:orc_orient)
#   tc128_sm103a.cubin    device code of src/WithoutPartition/ShareKernelTCV62_update_v1.cu
#                         (TC_128's Find_Triangle) for sm_103a, launched by
#                         oracle/ref_launch.cu to cross-check counts and time the
#                         reference kernel on the same GPU
#   var_*_sm103a.cubin    the reference's design-space variants of the same kernel
#                         (src/WithoutPartition/): shareMemSize.cu (64 threads),
#                         With_Atomic_op.cu (256 threads, one atomic per probe),
#                         Without_ShareMemory_TC.cu (2 threads, u64, binary search
#                         in global memory) -- timed beside TC_128 on the GB300
#
# src/WithPartition/without_sorting_tc.cu (wo_sort_tc_256) is compiled here only
# to show it builds; its kernel calls __syncthreads() inside `if (tid == 0)`
# (without_sorting_tc.cu:209-217), so it is never launched.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
# the reference tree: $REF, else a checkout named "reference" beside the repository
REF=${REF:-"$(dirname "$(dirname "$HERE")")/reference"}
OUT="$HERE/_ref"
NVCC=${NVCC:-/usr/local/cuda/bin/nvcc}
[ -d "$REF" ] || { echo "reference tree not found at $REF; skipping"; exit 0; }
mkdir -p "$OUT"
g++ -O2 -w -x c++ -I "$REF/preprocess_CPU" "$REF/preprocess_CPU/Undir2Dir.c" -o "$OUT/undir2dir"
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a \
    "$REF/src/WithoutPartition/ShareKernelTCV62_update_v1.cu" -o "$OUT/tc128_sm103a.cubin"
for v in shareMemSize:smem64 With_Atomic_op:atomic256 Without_ShareMemory_TC:nosmem2; do
    "$NVCC" -cubin -w -gencode arch=compute_103a,code=sm_103a \
        "$REF/src/WithoutPartition/${v%%:*}.cu" -o "$OUT/var_${v##*:}_sm103a.cubin"
done
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a \
    "$REF/src/WithPartition/without_sorting_tc.cu" -o "$OUT/wo_sort_sm103a.cubin.unused"
echo "built $(ls "$OUT" | tr '\n' ' ')"
