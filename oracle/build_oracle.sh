#!/bin/sh
# Builds the oracle (test infrastructure) into oracle/_build/liborc.so.
# -ffp-contract=off and no fast-math: the estimator's f64 arithmetic must round
# exactly as the reference's Rust f64 code does (both call the platform libm).
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CXX:-g++} -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    "$here/fbk_oracle.cpp" -o "$here/_build/liborc.so.tmp"
mv "$here/_build/liborc.so.tmp" "$here/_build/liborc.so"
