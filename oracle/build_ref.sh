#!/bin/sh
# Compiles the reference's BVH and MBVH kernel texts (OpenCL C, from the
# LuxCore source tree) for the CPU through oracle/refcl_prelude.h, into
# oracle/_ref/, and stitches its CUDA BVH kernel text there for the GPU arm.
# Test infrastructure only: the result pins the oracle (tests/golden/).
# Usage: oracle/build_ref.sh [--tree] [path to the LuxCore source tree]
# The tree is the argument, else $LUXCORE_REFERENCE_TREE, else the copy this
# project was developed beside.  Exits 3 (nothing built) when it is absent,
# as on a machine that has only this repository.  --tree only prints the
# tree's path (tests that compile against its headers use it).
set -e
PRINT_TREE=0
if [ "$1" = "--tree" ]; then PRINT_TREE=1; shift; fi
REF="${1:-${LUXCORE_REFERENCE_TREE:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/include/luxrays/accelerators/bvh.cl" ]; then
	echo "reference tree not found at $REF" >&2
	exit 3
fi
if [ "$PRINT_TREE" = 1 ]; then
	echo "$REF"
	exit 0
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
# The reference's CUDA BVH kernel text, for the same-GPU arm
# (oracle/refcu_harness.cpp compiles it with NVRTC at run time): the OpenCL
# emulation prefix CUDADevice::GetKernelSource puts first
# (src/luxrays/devices/cudadevice.cpp:235-241), then BVHKernel's page defines
# and kernel files in its order (src/luxrays/accelerators/bvhaccelhw.cpp:173-202),
# for one vertex page and one node page.  Text only: it stays in oracle/_ref/.
I="$REF/include"
{
	cat "$I/luxrays/devices/cudadevice_oclemul_types.cl" "$I/luxrays/devices/cudadevice_math.cl" \
		"$I/luxrays/devices/cudadevice_oclemul_funcs.cl"
	printf '#define BVH_VERTS_PAGE_COUNT 1\n#define BVH_NODES_PAGE_COUNT 1\n#define BVH_VERTS_PAGE0 1\n#define BVH_NODES_PAGE0 1\n'
	for f in luxrays/luxrays_types.cl luxrays/core/epsilon_types.cl luxrays/core/epsilon_funcs.cl \
			luxrays/core/geometry/point_types.cl luxrays/core/geometry/vector_types.cl \
			luxrays/core/geometry/ray_types.cl luxrays/core/geometry/ray_funcs.cl \
			luxrays/core/geometry/bbox_types.cl luxrays/core/geometry/bbox_funcs.cl \
			luxrays/core/geometry/triangle_types.cl luxrays/core/geometry/triangle_funcs.cl \
			luxrays/core/bvh/bvhbuild_types.cl luxrays/accelerators/bvh.cl; do
		cat "$I/$f"
	done
} > "$HERE/_ref/refcu_bvh_kernel.cu.tmp"
mv "$HERE/_ref/refcu_bvh_kernel.cu.tmp" "$HERE/_ref/refcu_bvh_kernel.cu"
echo "$HERE/_ref/refcu_bvh_kernel.cu"
