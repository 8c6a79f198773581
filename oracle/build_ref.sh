#!/bin/sh
# Builds oracle/_ref/libref_grouporder.so from the reference's GroupOrder.h as it
# lies in the reference tree (read-only; nothing is copied).  Two shim headers
# stand in for MSVC-only system headers; __declspec is defined away.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $ISE_REFERENCE_ROOT, else /root/reference, where this build found it)
set -e
REF=${1:-${ISE_REFERENCE_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/k-Factorization/Utils/Include/GroupOrder.h" ]; then
    echo "reference tree not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/shim"
: > "$OUT/shim/vcruntime.h"
echo 'typedef const wchar_t *LPCWSTR;' > "$OUT/shim/wtypes.h"
${CXX:-g++} -std=c++20 -O2 -fPIC -shared -w -fpermissive -D'__declspec(x)=' \
    -I "$OUT/shim" -I "$REF/k-Factorization/Utils/Include" \
    -I "$REF/k-Factorization/TripleSys/Include" \
    "$HERE/ref_harness/group_order_ref.cpp" -o "$OUT/libref_grouporder.so"
echo "built $OUT/libref_grouporder.so"
