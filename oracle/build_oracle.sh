#!/usr/bin/env bash
# Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CC:-gcc} -std=c11 -O2 -fopenmp -ffp-contract=off -fno-fast-math -fPIC -shared \
    -Wall -Wno-unknown-pragmas \
    "$here/oracle.c" "$here/render.c" -o "$here/_build/liboracle.so" -lm
echo "built $here/_build/liboracle.so"
