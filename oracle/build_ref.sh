#!/bin/sh
# Builds oracle/_ref/libmbref.so: the reference's own mbsolve-lib sources and
# its solver_cpu_fdtd / solver_cpu_fdtd_red time loops, compiled where they
# lie in the reference tree (nothing is copied), plus oracle/ref_driver.cpp.
# The reference's CMake build is not used: it needs Eigen, which is absent.
# Usage: oracle/build_ref.sh [reference-root]
#   (default: $MBSOLVE_REFERENCE, else a checkout named "reference" beside
#   this repository)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${MBSOLVE_REFERENCE:-$HERE/../../reference}}
OUT="$HERE/_ref"
if [ ! -d "$REF/mbsolve-lib/src" ]; then
    echo "reference tree not found at $REF" >&2
    exit 1
fi
# REF_CXXFLAGS / REF_LIB: optimisation flags and library name (the CPU
# baseline's calibration builds libmbref_baseline.so with the reference's
# own solver-cpu flags)
FLAGS=${REF_CXXFLAGS:--O2}
LIB=${REF_LIB:-libmbref.so}
mkdir -p "$OUT"
${CXX:-g++} $FLAGS -std=c++17 -fopenmp -fPIC -shared -DUSE_OMP_SIMD=1 -w \
    -I"$REF/mbsolve-lib/include" -I"$REF/solver-cpu/include" \
    "$REF/mbsolve-lib/src/device.cpp" "$REF/mbsolve-lib/src/material.cpp" \
    "$REF/mbsolve-lib/src/record.cpp" "$REF/mbsolve-lib/src/result.cpp" \
    "$REF/mbsolve-lib/src/scenario.cpp" "$REF/mbsolve-lib/src/solver.cpp" \
    "$REF/mbsolve-lib/src/writer.cpp" \
    "$HERE/ref_driver.cpp" -o "$OUT/$LIB"
echo "built $OUT/$LIB"
