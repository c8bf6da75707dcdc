#!/bin/sh
# Compiles the reference's own CUDA-C step kernels (Kairzhan/DUGKS-GPU
# src/dugks.cu, unmodified, read where it lies) into device-code cubins for
# sm_103a, FP64 and PREC4 builds, against the single-rank MPI declarations of
# ref_shim/.  TEST INFRASTRUCTURE ONLY (oracle of the reference's GPU path).
#   sh oracle/build_ref.sh REFERENCE_ROOT
# (or REFERENCE_ROOT in the environment).  Without a reference tree it keeps
# whatever was built before and exits 0.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${REFERENCE_ROOT:-}}
if [ -z "$REF" ]; then
    echo "build_ref: no reference root given; keeping any prebuilt cubins" >&2
    exit 0
fi
SRC="$REF/src/dugks.cu"
if [ ! -f "$SRC" ]; then
    echo "build_ref: $SRC not found; keeping any prebuilt cubins" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
NVCC=${NVCC:-nvcc}
FLAGS="-cubin -std=c++17 -gencode arch=compute_103a,code=sm_103a -O3 -I$HERE/ref_shim -w"
$NVCC $FLAGS "$SRC" -o "$HERE/_ref/dugks_f64.cubin" &
$NVCC $FLAGS -DPREC4 "$SRC" -o "$HERE/_ref/dugks_f32.cubin" &
wait
