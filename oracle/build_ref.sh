#!/bin/sh
# ORACLE (test infrastructure only).
# Compiles oracle/_ref/libshref.so from the reference's own per-cell headers
# where they lie in the sledgehamr tree (source/utils/sledgehamr_utils.h,
# source/kernels.h, projects/*/kernels_*.h, MinimalExample.h) together with
# the oracle drivers.  Nothing is copied out of the reference tree.
# Usage: sh oracle/build_ref.sh [REFERENCE_ROOT]
# The tree is the argument, else $SLEDGEHAMR_REF_ROOT, else a directory
# named "reference" beside this repository.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${SLEDGEHAMR_REF_ROOT:-$HERE/../../reference}}
if [ ! -d "$REF/source" ]; then
    echo "build_ref: no reference tree at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O2 -ffp-contract=off -fPIC -shared -fopenmp \
    -include "$HERE/ref_shim/ref_prelude.h" \
    -I"$HERE/ref_shim" -I"$REF/source/utils" -I"$REF/source" -I"$REF/projects" -I"$HERE" \
    "$HERE/ref_harness.cpp" -o "$HERE/_ref/libshref.so"
echo "built $HERE/_ref/libshref.so"
