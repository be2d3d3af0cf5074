#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
# Usage: oracle/build.sh            (portable -O2, OpenMP over modes)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
g++ -O2 -std=c++17 -fPIC -shared -fopenmp \
    -o "$here/_build/libdiscoeb_oracle.so" "$here/discoeb_oracle.cpp"
