#!/bin/sh
# TEST INFRASTRUCTURE ONLY.  Builds oracle/_ref/libref_rng.so from the
# reference's random sampler header where it lies (read-only), with the
# oracle's glm shim; nothing of the reference is copied.  Exits 0 without
# building when the reference tree is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${SPRAY_REFERENCE_DIR:-/root/reference}
[ -f "$REF/deps/embree/random_sampler.h" ] || { echo "reference sources absent: oracle/_ref not built"; exit 0; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -I "$HERE/ref_shim" -I "$REF/deps/embree" \
    "$HERE/ref_rng.cpp" -o "$HERE/_ref/libref_rng.so"
echo "$HERE/_ref/libref_rng.so"
