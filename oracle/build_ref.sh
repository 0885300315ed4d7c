#!/bin/sh
# Compiles a few of FEDDLib's own sources (Helper.cpp and the Laplace /
# Navier-Stokes element classes) where they lie in the reference tree,
# against this project's stub Trilinos headers (oracle/refshim), into
# oracle/_ref/libfeddref.so.  Test infrastructure only; needs the reference
# tree, so it runs in the build container and is skipped where it is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${FEDDLIB_REF:-/root/reference}
[ -d "$REF/feddlib/core" ] || { echo "reference tree not found; skipping oracle/_ref"; exit 0; }
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -w \
    -I"$HERE/refshim" -I"$REF" \
    "$HERE/ref_driver.cpp" "$REF/feddlib/core/FE/Helper.cpp" \
    -o "$HERE/_ref/libfeddref.so"
echo "built $HERE/_ref/libfeddref.so"
