#!/bin/sh
# Builds, from the reference tree, the test-infrastructure programs that
# record golden vectors (outputs only under oracle/_ref, git-ignored):
#   _ref/ref_probe          the reference's own Binner.h / Waveform.h and
#                           src/Directivity.cpp on the host (g++), with the
#                           host stand-ins of oracle/ref_stubs;
#   _ref/ref_sparse2d.cubin the reference's own src/SensorInstance2D.cu
#                           (do_sparse_convolve_2d_f and the KernelView2D
#                           texture lookup) for sm_103a (nvcc), with the
#                           device stand-ins of oracle/ref_stubs_cuda; it is
#                           launched by oracle/ref_sparse_harness.cpp on a
#                           GPU machine (tests/golden/make_ref_pings.py);
#   _ref/ref_sparse1d.cubin the same for src/SensorInstance1D.cu
#                           (do_sparse_convolve_1d_f, KernelView1D).
# Usage: oracle/ref_build.sh [REFERENCE_ROOT]
# The tree is REFERENCE_ROOT, else $RTAC_SIMULATION_REFERENCE, else the
# container's read-only mount /root/reference. Without a reference tree (a
# GPU machine, which only runs what was built from it) nothing is built and
# the script exits 0.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${RTAC_SIMULATION_REFERENCE:-/root/reference}}"
if [ ! -d "$REF/src" ]; then
    echo "ref_build.sh: no reference tree at $REF; nothing built"
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O1 -ffp-contract=off -fno-fast-math \
    -I "$HERE/ref_stubs" -I "$REF/include" \
    "$HERE/ref_probe.cpp" "$REF/src/Directivity.cpp" -o "$HERE/_ref/ref_probe"
NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -diag-suppress 20012 \
    -I "$HERE/ref_stubs_cuda" -I "$REF/include" \
    "$REF/src/SensorInstance2D.cu" -o "$HERE/_ref/ref_sparse2d.cubin"
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -diag-suppress 20012 \
    -I "$HERE/ref_stubs_cuda" -I "$REF/include" \
    "$REF/src/SensorInstance1D.cu" -o "$HERE/_ref/ref_sparse1d.cubin"
