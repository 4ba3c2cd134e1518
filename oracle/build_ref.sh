#!/bin/sh
# ORACLE — builds oracle/_ref/libqsi_ref.so from the reference's own
# components/operator/src/operator.cpp (and the headers it includes, where they
# lie under the reference checkout) plus oracle/ref_harness.cpp.  Only the
# output goes into oracle/_ref/.  Usage: oracle/build_ref.sh REFERENCE_ROOT
# (or QSI_REFERENCE_ROOT in the environment): the qsi_subspace_ED checkout.
set -e
REF=${1:-$QSI_REFERENCE_ROOT}
if [ -z "$REF" ]; then
    echo "usage: $0 REFERENCE_ROOT (the qsi_subspace_ED checkout)" >&2
    exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fopenmp -fPIC -shared \
    -I"$HERE/ref_shim" -I"$REF/components/operator/include" -I"$REF/components/common/include" \
    "$REF/components/operator/src/operator.cpp" "$HERE/ref_harness.cpp" \
    -o "$HERE/_ref/libqsi_ref.so"
echo "$HERE/_ref/libqsi_ref.so"
