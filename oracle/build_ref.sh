#!/bin/sh
# Builds oracle/_ref/libref_harness.so from the reference's host C++ headers,
# included in place from the reference checkout (default /root/reference).
# Test infrastructure only; exits 0 without building when the checkout is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${BSF_REFERENCE_DIR:-/root/reference}
if [ ! -f "$REF/native/src/p20_exact_math.hpp" ]; then
    echo "reference checkout not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -I"$REF/native/src" \
    -o "$HERE/_ref/libref_harness.so" "$HERE/ref_harness.cpp"
echo "built $HERE/_ref/libref_harness.so"
