#!/bin/bash
# Builds the reference's own CUDA library (gpu_aln_pack.so) from its sources
# where they lie, into oracle/_ref/.  Test infrastructure only.
#
# The sources predate CUDA 13: three cufftResult enumerators and one
# cudaDeviceProp field they name no longer exist.  Instead of editing the
# sources, the missing names are supplied on the command line: the three
# enumerators become distinct integers (they are only case labels of an error
# printer) and the removed field reads another int field of the same struct
# (it is only printed by print_gpu_info).
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT: the argument, else $GPUISAC_REFERENCE_ROOT, else
#   /root/reference; exits 2 when no sources are found there
set -euo pipefail
REF="${1:-${GPUISAC_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/cuda/gpu_aln_noref.cu" ]; then
    echo "reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
nvcc -gencode arch=compute_103a,code=sm_103a -O2 -std=c++11 -shared -Xcompiler -fPIC \
    -DCUFFT_PARSE_ERROR=1001 -DCUFFT_LICENSE_ERROR=1002 -DCUFFT_INCOMPLETE_PARAMETER_LIST=1003 \
    -DkernelExecTimeoutEnabled=integrated \
    -I "$REF/cuda" "$REF/cuda/gpu_aln_common.cu" "$REF/cuda/gpu_aln_noref.cu" \
    -o "$OUT/gpu_aln_pack.so" -lcufft -lcublas
echo "$OUT/gpu_aln_pack.so"
