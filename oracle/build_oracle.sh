#!/bin/sh
# Builds the oracle restatement (test infrastructure) into oracle/_build/.
# IEEE float arithmetic in source order: no fast-math, no FP contraction.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_build"
gcc -std=c99 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    -I"$HERE" -I"$HERE/fftw_shim" \
    "$HERE/vbm3d_oracle.c" "$HERE/fftw_shim/fftw_shim.c" -lm \
    -o "$HERE/_build/liboracle.so"
gcc -std=c99 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -I"$HERE" \
    "$HERE/tvl1_oracle.c" -lm -o "$HERE/_build/libtvl1_oracle.so"
# The same restatement with the reference's own CMake flags (CMakeLists.txt:15,
# -O3 -ffast-math -fomit-frame-pointer, OpenMP): the CPU baseline's timing
# build, where the reference's sources are absent.  Not a parity oracle
# (fast-math reorders the sums).
gcc -std=c99 -O3 -ffast-math -fomit-frame-pointer -fopenmp -fPIC -shared \
    -I"$HERE" -I"$HERE/fftw_shim" \
    "$HERE/vbm3d_oracle.c" "$HERE/fftw_shim/fftw_shim.c" -lm \
    -o "$HERE/_build/liboracle_fast.so"
