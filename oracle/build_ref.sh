#!/bin/sh
# Builds the reference's own hot-path sources into oracle/_ref/ (test
# infrastructure).  Reads the sources where they lie; copies none of them.
#   $1 = reference project root (default /root/reference)
# Outputs:
#   oracle/_ref/libvbm3d_ref_exact.so  -O2, no fast-math, no FP contraction:
#       the parity oracle (IEEE float arithmetic in source order)
#   oracle/_ref/libvbm3d_ref_fast.so   the reference's CMake flags
#       (-O3 -ffast-math -fomit-frame-pointer, CMakeLists.txt:15) + OpenMP:
#       the reference as shipped, for the noise floor and CPU timing
#   oracle/_ref/libtvl1_ref.so   the reference's TV-L1 library
#       (tvl1flow/tvl1flow_lib.c and the files it includes), single thread,
#       no FP contraction: the pin of the TV-L1 restatement
# FFTW3f is not installed: oracle/fftw_shim supplies REDFT10/REDFT01.
set -e
REF=${1:-/root/reference}
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
echo "built $OUT"
