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
# the reference's integrators (rkn.cpp, lsssprk3.cpp, leapfrog.cpp) compiled
# unchanged against the AMReX stand-in of ref_shim_int, driven by
# ref_integrators.cpp with the Rhs of libshref.so
${CXX:-g++} -std=c++17 -O2 -ffp-contract=off -fPIC -shared \
    -include "$HERE/ref_shim/ref_prelude.h" \
    -I"$HERE/ref_shim_int" -I"$REF/source/integrators" -I"$REF/source" -I"$REF/source/utils" \
    "$HERE/ref_integrators.cpp" "$REF/source/integrators/rkn.cpp" \
    "$REF/source/integrators/lsssprk3.cpp" "$REF/source/integrators/leapfrog.cpp" \
    -L"$HERE/_ref" -lshref -Wl,-rpath,'$ORIGIN' -Wl,--no-undefined \
    -o "$HERE/_ref/libshref_int.so"
echo "built $HERE/_ref/libshref_int.so"
