#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
g++ -std=c++20 -O3 -fPIC -shared -fopenmp "$here/oracle.cpp" -o "$here/_build/liboracle.so.tmp"
mv "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
