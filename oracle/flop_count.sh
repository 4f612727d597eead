#!/bin/sh
# Prints the algorithmic flops per element used by bench.py's element-kernel roofline.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O1 -I "$HERE/../include" -o "$HERE/_build/flop_count" "$HERE/flop_count.cpp"
"$HERE/_build/flop_count"
