#!/bin/sh
# Builds the oracle (CPU restatement; test infrastructure only) into oracle/_build/.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared \
    -o "$HERE/_build/liboracle.so" "$HERE/oracle.cpp"
