#!/bin/sh
# Builds oracle/_ref/libmbref.so: the reference's own mbsolve-lib sources and
# its solver_cpu_fdtd / solver_cpu_fdtd_red time loops, compiled where they
# lie in the reference tree (nothing is copied), plus oracle/ref_driver.cpp.
# The reference's CMake build is not used: it needs Eigen, which is absent.
# Usage: oracle/build_ref.sh [reference-root]   (default /root/reference)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${MBSOLVE_REFERENCE:-/root/reference}}
OUT="$HERE/_ref"
if [ ! -d "$REF/mbsolve-lib/src" ]; then
    echo "reference tree not found at $REF" >&2
    exit 1
fi
mkdir -p "$OUT"
${CXX:-g++} -O2 -std=c++17 -fopenmp -fPIC -shared -DUSE_OMP_SIMD=1 -w \
    -I"$REF/mbsolve-lib/include" -I"$REF/solver-cpu/include" \
    "$REF/mbsolve-lib/src/device.cpp" "$REF/mbsolve-lib/src/material.cpp" \
    "$REF/mbsolve-lib/src/record.cpp" "$REF/mbsolve-lib/src/result.cpp" \
    "$REF/mbsolve-lib/src/scenario.cpp" "$REF/mbsolve-lib/src/solver.cpp" \
    "$REF/mbsolve-lib/src/writer.cpp" \
    "$HERE/ref_driver.cpp" -o "$OUT/libmbref.so"
echo "built $OUT/libmbref.so"
