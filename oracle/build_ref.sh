#!/bin/sh
# Builds, from the reference's unmodified sources read where they lie
# (Kairzhan/DUGKS-GPU src/), TEST INFRASTRUCTURE ONLY, into oracle/_ref/:
#  * its CUDA-C step kernels (src/dugks.cu) as device-code cubins for sm_103a,
#    FP64 and PREC4 builds -- the oracle of the reference's GPU path;
#  * its own driver and I/O (src/main.cu, numerics.cu, parallel.cu, cuda.cu,
#    checks.cu, output.cu, lbm_d3q19.cu) linked, in place of src/dugks.cu,
#    against this repository's legacy-name libraries (libdugks_legacy.so,
#    libdugks_legacy_prec4.so): ref_main_legacy and ref_main_legacy_prec4,
#    the reference's main() driving the GB300 engine.  These are host
#    binaries of the machine that builds them.
# Both use the single-rank MPI of ref_shim/.
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

# the reference's driver over the legacy-name libraries (needs them built first)
PKG="$HERE/../dugks-gpu_gb300"
if [ -f "$PKG/libdugks_legacy.so" ] && [ -f "$PKG/libdugks_legacy_prec4.so" ]; then
    for V in f64 prec4; do
        (
            OBJ="$HERE/_ref/legacy_$V"
            mkdir -p "$OBJ"
            DEF=""; LIB=dugks_legacy; OUT=ref_main_legacy
            if [ "$V" = prec4 ]; then DEF="-DPREC4"; LIB=dugks_legacy_prec4; OUT=ref_main_legacy_prec4; fi
            for T in main numerics parallel cuda checks output lbm_d3q19; do
                $NVCC -std=c++17 -O2 -w $DEF -I"$HERE/ref_shim" -c "$REF/src/$T.cu" -o "$OBJ/$T.o"
            done
            ${CC:-gcc} -O2 -c "$HERE/ref_shim/mpi_single.c" -o "$OBJ/mpi_single.o"
            $NVCC -o "$HERE/_ref/$OUT" "$OBJ"/*.o -L"$PKG" -l$LIB -ldugks_gb300 -Xlinker -rpath -Xlinker '$ORIGIN/../../dugks-gpu_gb300'
        ) &
    done
else
    echo "build_ref: legacy-name libraries not built; skipping the reference's driver" >&2
fi
wait
