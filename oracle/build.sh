#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/liboracle.so.
# -ffp-contract=off keeps every multiply and add separately rounded, as the
# reference's x86 -O2 -msse4 build did; explicit std::fma calls are the only
# fused operations.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -fopenmp \
    "$HERE/oracle.cpp" -o "$HERE/liboracle.so"
echo "build: $HERE/liboracle.so"
