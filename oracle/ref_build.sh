#!/bin/sh
# Builds the golden-vector probe from the reference's own headers and its
# src/Directivity.cpp (the receiver directivity table builders).
# Usage: oracle/ref_build.sh [REFERENCE_ROOT]   (default /root/reference)
# Output: oracle/_ref/ref_probe (git-ignored). Test infrastructure only.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-/root/reference}"
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O1 -ffp-contract=off -fno-fast-math \
    -I "$HERE/ref_stubs" -I "$REF/include" \
    "$HERE/ref_probe.cpp" "$REF/src/Directivity.cpp" -o "$HERE/_ref/ref_probe"
