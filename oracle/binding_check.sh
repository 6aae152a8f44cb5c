#!/bin/sh
# Compile-and-link check of the librtacx binding against the reference's own
# headers (test infrastructure; outputs only under oracle/_ref, git-ignored):
# tests/cpp/binding/real_headers.cpp compiles the binding statements of
# tests/cpp/binding/sensor_instance2d_rtacx.inc inside a class derived from
# the reference's SensorInstance2D_Complex (include/rtac_simulation/
# SensorInstance2D.h), with the rtac_base stand-ins of oracle/ref_stubs_binding
# and oracle/ref_stubs, then links the object into a shared library against
# rtac_simulation_gb300/librtacx.so with every symbol resolved.
# Usage: oracle/binding_check.sh [REFERENCE_ROOT]
# The tree is REFERENCE_ROOT, else $RTAC_SIMULATION_REFERENCE, else the
# container's read-only mount /root/reference. Without a reference tree
# nothing is checked and the script says so and exits 0.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$HERE")"
REF="${1:-${RTAC_SIMULATION_REFERENCE:-/root/reference}}"
if [ ! -d "$REF/include/rtac_simulation" ]; then
    echo "binding_check.sh: no reference tree at $REF; nothing checked"
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O1 -fPIC -Wall -c \
    -I "$ROOT/tests/cpp/binding" -I "$HERE/ref_stubs_binding" -I "$HERE/ref_stubs" -I "$REF/include" \
    -I "$ROOT/include" "$ROOT/tests/cpp/binding/real_headers.cpp" -o "$HERE/_ref/binding_real_headers.o"
g++ -shared -Wl,--no-undefined -o "$HERE/_ref/binding_real_headers.so" "$HERE/_ref/binding_real_headers.o" \
    -L "$ROOT/rtac_simulation_gb300" -lrtacx
echo "binding_check.sh: compiled against $REF/include and linked to librtacx.so"
