#!/bin/sh
# Builds the reference's own hot-path sources into oracle/_ref/ (test
# infrastructure).  Reads the sources where they lie; copies none of them.
#   $1 = reference project root (default: $VBM3D_REFERENCE, else
#        /root/reference, where this container mounts it)
#   --where       print the reference project root and exit
#   --if-present  build only if the reference sources are there (exit 0
#                 quietly otherwise, as on machines without them)
# Outputs:
#   oracle/_ref/libvbm3d_ref_exact.so  -O2, no fast-math, no FP contraction:
#       the parity oracle (IEEE float arithmetic in source order)
#   oracle/_ref/libvbm3d_ref_fast.so   the reference's CMake flags
#       (-O3 -ffast-math -fomit-frame-pointer, CMakeLists.txt:15) + OpenMP:
#       the reference as shipped, for the noise floor and CPU timing
#   oracle/_ref/libtvl1_ref.so   the reference's TV-L1 library
#       (tvl1flow/tvl1flow_lib.c and the files it includes), single thread,
#       no FP contraction: the pin of the TV-L1 restatement
#   oracle/_ref/libms_ref.so   the reference's multiscaler programs
#       (multiscaler/{multiscaler,decompose,recompose,merge_coarse}.cpp):
#       the pin of the multiscaler restatement
# FFTW3f is not installed: oracle/fftw_shim supplies REDFT10/REDFT01.
set -e
MODE=""
case "$1" in
    --where|--if-present) MODE=$1; shift ;;
esac
REF=${1:-${VBM3D_REFERENCE:-/root/reference}}
if [ "$MODE" = "--where" ]; then
    echo "$REF"
    exit 0
fi
if [ ! -d "$REF/src" ]; then
    [ "$MODE" = "--if-present" ] && exit 0
    echo "reference sources not found under $REF" >&2
    exit 1
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
SRC="$REF/src"
INC="-I$HERE/fftw_shim -I$SRC -I$SRC/Utilities -I$HERE/../include"
CXXSRC="$SRC/vbm3d.cpp $SRC/lib_transforms.cpp $SRC/Utilities/Utilities.cpp $HERE/ref_harness/ref_harness.cpp"
build() {
    name=$1; shift
    tmp=$(mktemp -d)
    for f in $CXXSRC; do
        b=$(basename "$f" .cpp)
        g++ -std=c++11 -w -fPIC -fopenmp -include ctime -include cassert -include algorithm "$@" $INC -c "$f" -o "$tmp/$b.o" &
    done
    gcc -std=c99 -fPIC "$@" -I"$HERE/fftw_shim" -c "$HERE/fftw_shim/fftw_shim.c" -o "$tmp/fftw_shim.o" &
    wait
    g++ -shared -fopenmp -o "$OUT/$name" "$tmp"/*.o -lm
    rm -rf "$tmp"
}
build libvbm3d_ref_exact.so -O2 -ffp-contract=off -fno-fast-math
build libvbm3d_ref_fast.so -O3 -ffast-math -fomit-frame-pointer
gcc -std=c99 -w -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -I"$REF/tvl1flow" \
    "$HERE/ref_harness/tvl1_ref_harness.c" -lm -o "$OUT/libtvl1_ref.so"
# the multiscaler programs, each main renamed, over the FFTW stand-in and
# an in-memory image table (ms_ref_harness.cpp) in place of iio
MS="$REF/multiscaler"
tmp=$(mktemp -d)
MSFLAGS="-std=c++11 -w -O2 -ffp-contract=off -fno-fast-math -fPIC -I$HERE/fftw_shim -I$MS"
g++ $MSFLAGS -c "$MS/multiscaler.cpp" -o "$tmp/multiscaler.o" &
g++ $MSFLAGS -Dmain=ms_decompose_main -c "$MS/decompose.cpp" -o "$tmp/decompose.o" &
g++ $MSFLAGS -Dmain=ms_recompose_main -c "$MS/recompose.cpp" -o "$tmp/recompose.o" &
g++ $MSFLAGS -Dmain=ms_merge_coarse_main -c "$MS/merge_coarse.cpp" -o "$tmp/merge_coarse.o" &
g++ $MSFLAGS -c "$HERE/ref_harness/ms_ref_harness.cpp" -o "$tmp/ms_ref_harness.o" &
gcc -std=c99 -O2 -ffp-contract=off -fno-fast-math -fPIC -I"$HERE/fftw_shim" -c "$HERE/fftw_shim/fftw_shim.c" -o "$tmp/fftw_shim.o" &
wait
g++ -shared -o "$OUT/libms_ref.so" "$tmp"/*.o -lm
rm -rf "$tmp"
echo "built $OUT"
