#!/usr/bin/env bash
# Builds oracle/_ref/libngrav_ref.so: the reference's own CPU Barnes-Hut path
# compiled from its sources where they lie (nothing is copied into this
# repository), with the reference's compiler flags
# (projects/nbody_core/CMakeLists.txt:35-37; CMake's default C++20 dialect
# with extensions is gnu++20) and this project's glm-compatible header in
# place of glm. Only the GL-free sources are compiled.
#
# Test infrastructure only: the result is the checker, never the product.
# Usage: oracle/build_ref.sh [reference-root]   (default: $NGRAV_REFERENCE or /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${NGRAV_REFERENCE:-/root/reference}}"
SRC="$REF/projects/nbody_core"
if [ ! -f "$SRC/src/Tree.cpp" ]; then
    echo "build_ref: reference sources not found under $SRC" >&2
    exit 3
fi
mkdir -p "$HERE/_ref"
g++ -std=gnu++20 -O3 -march=native -funroll-loops -fopenmp -fPIC -shared \
    -I "$HERE/ref_shim" -I "$SRC/include" \
    "$SRC/src/Tree.cpp" "$SRC/src/Solvers.cpp" "$SRC/src/Integrator.cpp" "$SRC/src/MutualFmm.cpp" \
    "$SRC/src/Scenarios.cpp" \
    "$HERE/ref_driver.cpp" \
    -o "$HERE/_ref/libngrav_ref.so.tmp"
mv "$HERE/_ref/libngrav_ref.so.tmp" "$HERE/_ref/libngrav_ref.so"
echo "build_ref: $HERE/_ref/libngrav_ref.so"
# The reference's run-directory writer (framework/src/OutputWriter.cpp, with
# fw::Deck and its vendored TOML parser), driven by writer_driver.cpp: the
# source of the byte-level writer fixture.
FW="$REF/framework"
g++ -std=gnu++20 -O2 -DNGRAV_WRITER_REF \
    -I "$FW/include" -I "$FW/third_party" \
    "$FW/src/OutputWriter.cpp" "$FW/src/Deck.cpp" "$HERE/writer_driver.cpp" \
    -o "$HERE/_ref/ref_writer.tmp"
mv "$HERE/_ref/ref_writer.tmp" "$HERE/_ref/ref_writer"
echo "build_ref: $HERE/_ref/ref_writer"
# Where the reference's headers are, for the CPU test that compiles the
# INTEGRATION.md binding against them (tests/test_binding.py).
echo "$REF" > "$HERE/_ref/REF_ROOT"
