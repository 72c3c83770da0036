#!/bin/sh
# Builds the host oracle (test infrastructure) into oracle/_build/liboracle.so.
# Portable flags only: the same recipe runs on x86_64 and aarch64 hosts.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
g++ -O3 -std=c++17 -fopenmp -fPIC -shared -Wall -o "$here/_build/liboracle.so.tmp" "$here/dmr_oracle.cpp"
mv "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
