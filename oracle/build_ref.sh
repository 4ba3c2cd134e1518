#!/bin/sh
# ORACLE — builds oracle/_ref/libqsi_ref.so from the reference's own
# components/operator/src/operator.cpp (and the headers it includes, where they
# lie under the reference checkout) plus oracle/ref_harness.cpp.  Only the
# output goes into oracle/_ref/.  Usage: oracle/build_ref.sh [REFERENCE_ROOT]
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fopenmp -fPIC -shared \
    -I"$HERE/ref_shim" -I"$REF/components/operator/include" -I"$REF/components/common/include" \
    "$REF/components/operator/src/operator.cpp" "$HERE/ref_harness.cpp" \
    -o "$HERE/_ref/libqsi_ref.so"
echo "$HERE/_ref/libqsi_ref.so"
