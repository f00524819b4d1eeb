#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/libkmoracle.so.
# -ffp-contract=off pins the float rounding of the restated summation order on
# both x86-64 and aarch64 hosts (gcc contracts a*b+c into FMA by default on
# aarch64).
set -e
here="$(cd "$(dirname "$0")" && pwd)"
gcc -O3 -std=c11 -fopenmp -ffp-contract=off -fno-fast-math -fPIC -shared \
    -o "$here/libkmoracle.so" "$here/kmeans_oracle.c" -lm
