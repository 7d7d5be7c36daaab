#!/usr/bin/env bash
# Compile the reference's own compute shaders (read in place from the
# reference checkout) as C++ through the GLSL shim into oracle/_ref/.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The checkout is the argument, else $NATRIX_REFERENCE_ROOT, else the
# read-only checkout this recipe was written against (/root/reference).
# Exits 0 without building when the reference sources are absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${NATRIX_REFERENCE_ROOT:-/root/reference}}"
shaders="$ref/natrix/core/shaders/originals"
demo="$ref/demo/shaders"
if [ ! -f "$shaders/shader.Poisson.comp" ]; then
    echo "reference shaders not found under $ref; oracle/_ref not built"
    exit 0
fi
mkdir -p "$here/_ref"
${CXX:-g++} -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared \
    -Wno-unused-variable -Wno-narrowing \
    -I "$here/ref_shim" -I "$shaders" -I "$demo" \
    "$here/ref_kernels.cpp" -o "$here/_ref/libnatrix_ref.so"
echo "built $here/_ref/libnatrix_ref.so"
