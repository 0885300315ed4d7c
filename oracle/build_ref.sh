#!/bin/sh
# Compiles a few of FEDDLib's own sources where they lie in the reference
# tree, against this project's stub Trilinos headers (oracle/refshim), into
# oracle/_ref/libfeddref.so: Helper.cpp, the Laplace / Navier-Stokes /
# generalized-Newtonian element classes, and (through ref_fe_driver.cpp and
# the stub FE class of ref_fe_stub.hpp) the FE members extracted from
# FE_def.hpp by extract_fe_members.py -- FE_def.hpp itself needs Trilinos
# (Thyra, Xpetra) and the un-vendored aceinterface.hpp and does not compile
# here.  Test infrastructure only; skipped where the tree is absent.
# FEDDLIB_REF names the FEDDLib source tree; without it the recipe looks at
# the build container's read-only mount of the reference.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${FEDDLIB_REF:-/root/reference}
[ -d "$REF/feddlib/core" ] || { echo "reference tree not found; skipping oracle/_ref"; exit 0; }
mkdir -p "$HERE/_ref"
${PYTHON:-python3} "$HERE/extract_fe_members.py" "$REF" "$HERE/_ref/fe_members.inc"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -w \
    -I"$HERE/refshim" -I"$HERE" -I"$HERE/_ref" -I"$REF" \
    "$HERE/ref_driver.cpp" "$HERE/ref_fe_driver.cpp" "$REF/feddlib/core/FE/Helper.cpp" \
    -o "$HERE/_ref/libfeddref.so"
echo "built $HERE/_ref/libfeddref.so"
