#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
# Usage: sh oracle/build_oracle.sh
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared \
    -o "$here/_build/libsph_oracle.so" "$here/sph_oracle.cpp"
