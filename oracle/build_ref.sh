#!/bin/sh
# Builds oracle/_ref/libglintref.so from the reference's own CPU sources where
# they lie (never copied into this repository) plus oracle/ref_driver.cpp.
# Test infrastructure only; the product never loads the result.
#
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $GLINT_REFERENCE_ROOT, else a directory named "reference"
#   beside this repository)
#
#   REF_OPT overrides the optimisation flags and REF_LIB the library's name,
#   e.g. REF_OPT="-g" REF_LIB=libglintref_asshipped.so for the reference's own
#   Makefile flags (src/Makefile:13: -g, no -O); REF_CPU_ONLY=1 skips the GPU
#   part below.
#
# Flags: -O2 -ffp-contract=off so that FP64 expressions are evaluated with one
# rounding per operation on every host (GCC contracts a*b+c into an FMA by
# default on aarch64; x86-64 without -mfma never does).  The Boost stub in
# oracle/ref_stub stands in for the uninstalled program_options header, which
# util/config.h includes but the CPU stages never call.
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${GLINT_REFERENCE_ROOT:-$(cd "$HERE/../.." && pwd)/reference}}
SRC="$REF/src"
OUT="$HERE/_ref"
if [ ! -d "$SRC/tracing" ]; then
    echo "reference sources not found under $SRC" >&2
    exit 2
fi
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
mkdir -p "$OUT"
CXX=${CXX:-g++}
OPT=${REF_OPT:-"-O2 -ffp-contract=off"}
LIB=${REF_LIB:-libglintref.so}
TAG=$(echo "$LIB" | tr -c 'A-Za-z0-9\n' '_')
FLAGS="-std=c++17 $OPT -fPIC -w -I$HERE/ref_stub -I$SRC -I$CUDA_INC -pthread -fopenmp"
objs=""
for f in filter refinement meeting workbench step_merge analyze; do
    $CXX $FLAGS -c "$SRC/tracing/$f.cpp" -o "$OUT/$f.$TAG.o" &
    objs="$objs $OUT/$f.$TAG.o"
done
# the compaction tool, its main() renamed so that merge_dump can be called
$CXX $FLAGS -Dmain=glint_ref_compaction_tool_main -c "$SRC/tools/compaction.cpp" -o "$OUT/compaction.$TAG.o" &
$CXX $FLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.$TAG.o" &
wait
$CXX -shared -o "$OUT/$LIB" $objs "$OUT/compaction.$TAG.o" "$OUT/ref_driver.$TAG.o" -pthread -fopenmp -lm
rm -f $objs "$OUT/compaction.$TAG.o" "$OUT/ref_driver.$TAG.o"
echo "built $OUT/$LIB"
[ "${REF_CPU_ONLY:-0}" = 1 ] && exit 0

# The reference's GPU kernels (cuda/geometry.cu, unmodified) as an sm_103a
# cubin, and the byte layout of the structures they take, for
# oracle/ref_gpu_driver.cpp.  Both are independent of the host CPU, so they
# run on the GPU machine as built here.
NVCC=${NVCC:-${CUDA_HOME:-/usr/local/cuda}/bin/nvcc}
if [ -x "$NVCC" ]; then
    $CXX -std=c++17 -O0 -w -I$HERE/ref_stub -I$SRC -I$CUDA_INC -pthread -fopenmp \
        "$HERE/ref_gpu_layout.cpp" -o "$OUT/ref_gpu_layout"
    "$OUT/ref_gpu_layout" > "$OUT/ref_gpu_layout.h"
    rm -f "$OUT/ref_gpu_layout"
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 --extended-lambda -w \
        -I$HERE/ref_stub -I$SRC "$SRC/cuda/geometry.cu" -o "$OUT/geometry.cubin"
    echo "built $OUT/geometry.cubin"
fi
