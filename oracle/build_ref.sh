#!/bin/sh
# Builds the reference harness: simpimc's own headers from the reference checkout (unmodified,
# read in place) compiled against the shim in oracle/refshim/, with the reference's release flags
# (CMakeLists.txt:57-75: -O3 -ffast-math, NDEBUG) but without -fopenmp: the OpenMP reductions of
# the actions then run in loop order (deterministic fixtures), and an index error inside one of
# those loops is reported instead of terminating the process. Output: oracle/_ref/libsimpimc_ref.so.
# Test infrastructure only; needs the checkout, so it runs where that exists (not on the GPU machine).
#
# Usage: sh oracle/build_ref.sh [path to the reference checkout, default /root/reference]
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-/root/reference}
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O3 -ffast-math -DNDEBUG -fPIC -shared -w \
    -I "$HERE/refshim" -I "$REF/src" "$HERE/refharness.cc" -o "$HERE/_ref/libsimpimc_ref.so"
