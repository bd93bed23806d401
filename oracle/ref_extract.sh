#!/bin/sh
# ref_extract.sh REFERENCE_ROOT OUT_DIR
#
# Assembles OUT_DIR/ref_kernels.inc and OUT_DIR/ref_blur.inc, the reference's device code that
# ref_host.cpp compiles for the CPU (test infrastructure: the oracle's pin). It takes line ranges
# of the reference's own sources unchanged, each behind a #line directive naming its file and
# line, and makes three mechanical rewrites:
#   1. `extern __shared__ float normalizedSPMap[];` (dynamic shared memory) becomes a pointer
#      to the host block's shared buffer;
#   2. readImageIntoSharedMemory is renamed readImageIntoSharedMemory_block, and ref_host_hooks.h
#      (included after it) defines readImageIntoSharedMemory as that loader between two barriers
#      of the block's threads: on the GPU the 32 threads of a block are one warp and run the
#      loader in step; as host threads they need the barriers;
#   3. the member GaussianBlurCUDA::CreateFilterKernel becomes the free function
#      GaussianBlurCUDA_CreateFilterKernel (it reads no member; ref_host.cpp plays the class).
# The sources are checked against the SHA-256 digests they had when this recipe was written, so
# another version of the reference fails here instead of compiling into something unchecked.
set -eu
REF="$1"
OUT="$2"
SRC="$REF/src"
mkdir -p "$OUT"

check() {
    got=$(sha256sum "$SRC/$1" | cut -d' ' -f1)
    if [ "$got" != "$2" ]; then
        echo "ref_extract: $SRC/$1 has digest $got, expected $2" >&2
        exit 1
    fi
}
check patchMatch.cu 6f86cfce17636d73280fd7e54130342fa9aec5acad26632e3aecbd5a26d81397
check array2d_refImg.cu e067f59376345497d6543962019e19726a5e9b86e6ac1064a229e6e52d3463fd
check array2d_wrapper.cu a2baae33723b143f1e29771622a46d6b73b103ff5b2ad2f2370ee89b6a292beb
check GaussianBlurCUDA.cu 847a3d4b96e9d9acca732416c4f1f03799768867c4800155baa93da3732bb15c

# part FILE FIRST LAST: lines FIRST..LAST of FILE behind a #line directive
part() {
    printf '#line %s "src/%s"\n' "$2" "$1"
    sed -n "$2,$3p" "$SRC/$1"
}

{
    echo "/* Generated by oracle/ref_extract.sh from the reference's sources: do not edit. */"
    # box sums of the reference window (Array2d_refImg::filterImage's kernels)
    part array2d_refImg.cu 4 67
    # initial random depth (Array2D_wrapper::randNumGen's kernel)
    part array2d_wrapper.cu 3 20
    # PatchMatch: constants, textures, NCC, argmin, reference tile, messages
    part patchMatch.cu 7 12
    part patchMatch.cu 27 37
    part patchMatch.cu 409 421
    part patchMatch.cu 433 715 |
        sed 's/^inline __device__ void readImageIntoSharedMemory(/inline __device__ void readImageIntoSharedMemory_block(/'
    echo '#include "ref_host_hooks.h"'
    # the kernels: computeAllCostGivenDepth, topToDown, downToTop
    part patchMatch.cu 775 1209 |
        sed 's/^\([[:space:]]*\)extern __shared__ float normalizedSPMap\[\];/\1float *normalizedSPMap = (float *)pmr_dynamic_shared;/'
} > "$OUT/ref_kernels.inc.tmp"

# both rewrites must have happened exactly as many times as expected
n1=$(grep -c 'readImageIntoSharedMemory_block(' "$OUT/ref_kernels.inc.tmp" || true)
n2=$(grep -c 'pmr_dynamic_shared;' "$OUT/ref_kernels.inc.tmp" || true)
if [ "$n1" != 1 ] || [ "$n2" != 2 ]; then
    echo "ref_extract: unexpected rewrite counts ($n1, $n2)" >&2
    exit 1
fi
mv "$OUT/ref_kernels.inc.tmp" "$OUT/ref_kernels.inc"

# GaussianBlurCUDA: widths, constant taps, the 2-D texture, the row and column kernels and the
# tap construction
{
    echo "/* Generated by oracle/ref_extract.sh from the reference's sources: do not edit. */"
    part GaussianBlurCUDA.cu 8 14
    part GaussianBlurCUDA.cu 19 22
    part GaussianBlurCUDA.cu 28 28
    part GaussianBlurCUDA.cu 39 70
    part GaussianBlurCUDA.cu 99 130 |
        sed 's/^void GaussianBlurCUDA::CreateFilterKernel(/static void GaussianBlurCUDA_CreateFilterKernel(/'
} > "$OUT/ref_blur.inc.tmp"
n3=$(grep -c '^static void GaussianBlurCUDA_CreateFilterKernel(' "$OUT/ref_blur.inc.tmp" || true)
if [ "$n3" != 1 ]; then
    echo "ref_extract: unexpected rewrite count ($n3)" >&2
    exit 1
fi
mv "$OUT/ref_blur.inc.tmp" "$OUT/ref_blur.inc"
