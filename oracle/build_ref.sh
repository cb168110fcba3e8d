#!/bin/sh
# Builds the reference harness: simpimc's own headers from the reference checkout (unmodified,
# read in place) compiled against the shim in oracle/refshim/, with the reference's release flags
# (CMakeLists.txt:57-75: -O3 -ffast-math, NDEBUG) but without -fopenmp: the OpenMP reductions of
# the actions then run in loop order (deterministic fixtures), and an index error inside one of
# those loops is reported instead of terminating the process. Output: oracle/_ref/libsimpimc_ref.so.
# Test infrastructure only; needs the checkout, so it runs only where that exists.
# With REF_OPENMP=1 it builds oracle/_ref/libsimpimc_ref_omp.so instead, with -fopenmp as the
# reference's release build has it: the timing of the reference's own OpenMP model (one chain, the
# action loops over threads), not the fixtures.
#
# Usage: [REF_OPENMP=1] sh oracle/build_ref.sh [path to the reference checkout, default /root/reference]
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-/root/reference}
mkdir -p "$HERE/_ref"
OUT="$HERE/_ref/libsimpimc_ref.so"
OMP=""
if [ "${REF_OPENMP:-0}" = "1" ]; then
    OUT="$HERE/_ref/libsimpimc_ref_omp.so"
    OMP="-fopenmp"
fi
${CXX:-g++} -std=c++17 -O3 -ffast-math -DNDEBUG $OMP -fPIC -shared -w \
    -I "$HERE/refshim" -I "$REF/src" "$HERE/refharness.cc" -o "$OUT"
