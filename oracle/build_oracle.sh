#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/liborc.so.
# -ffp-contract=off keeps every multiply-add exactly as written (gcc contracts
# a*b+c into fma by default on aarch64), so results are identical on x86_64
# and on the Arm GPU hosts.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -fopenmp \
    -o "$HERE/_build/liborc.so.tmp" "$HERE/faust_oracle.cpp"
mv "$HERE/_build/liborc.so.tmp" "$HERE/_build/liborc.so"
