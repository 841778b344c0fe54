#!/bin/sh
# Compiles the reference's BVH kernel text (OpenCL C, from the LuxCore source
# tree) for the CPU through oracle/refcl_prelude.h, into oracle/_ref/.
# Test infrastructure only: the result pins the oracle (tests/golden/).
# Usage: oracle/build_ref.sh [path to the LuxCore source tree]
set -e
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/include/luxrays/accelerators/bvh.cl" ]; then
	echo "reference tree not found at $REF" >&2
	exit 1
fi
mkdir -p "$HERE/_ref"
g++ -O2 -ffp-contract=off -fno-fast-math -fno-strict-aliasing -fPIC -shared -std=c++17 -pthread \
	-w -I "$HERE" -I "$REF/include" "$HERE/refcl_harness.cpp" -o "$HERE/_ref/liblrx_refcl.so.tmp"
mv "$HERE/_ref/liblrx_refcl.so.tmp" "$HERE/_ref/liblrx_refcl.so"
echo "$HERE/_ref/liblrx_refcl.so"
