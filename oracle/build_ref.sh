#!/bin/sh
# Compiles the reference's BVH and MBVH kernel texts (OpenCL C, from the
# LuxCore source tree) for the CPU through oracle/refcl_prelude.h, into
# oracle/_ref/.
# Test infrastructure only: the result pins the oracle (tests/golden/).
# Usage: oracle/build_ref.sh [path to the LuxCore source tree]
# The tree is the argument, else $LUXCORE_REFERENCE_TREE, else the copy this
# project was developed beside.  Exits 3 (nothing built) when it is absent,
# as on a machine that has only this repository.
set -e
REF="${1:-${LUXCORE_REFERENCE_TREE:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/include/luxrays/accelerators/bvh.cl" ]; then
	echo "reference tree not found at $REF" >&2
	exit 3
fi
mkdir -p "$HERE/_ref"
# bvh.cl (BVHKernel) and mbvh.cl (MBVHKernel with transforms and motion systems)
for h in refcl_harness:liblrx_refcl refcl_mbvh_harness:liblrx_refcl_mbvh; do
	src="${h%%:*}"; lib="${h##*:}"
	g++ -O2 -ffp-contract=off -fno-fast-math -fno-strict-aliasing -fPIC -shared -std=c++17 -pthread \
		-w -I "$HERE" -I "$REF/include" "$HERE/$src.cpp" -o "$HERE/_ref/$lib.so.tmp" &
done
wait
for lib in liblrx_refcl liblrx_refcl_mbvh; do
	mv "$HERE/_ref/$lib.so.tmp" "$HERE/_ref/$lib.so"
	echo "$HERE/_ref/$lib.so"
done
