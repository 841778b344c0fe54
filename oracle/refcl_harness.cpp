// Runs the reference's own BVH kernel text (include/luxrays/accelerators/bvh.cl
// and the geometry .cl files it is stitched with, in the order of
// src/luxrays/accelerators/bvhaccelhw.cpp:189-202) on the CPU, one work item
// at a time -- TEST INFRASTRUCTURE, built by oracle/build_ref.sh from the
// reference tree into oracle/_ref/ and used only to pin the oracle.
#include <thread>
#include <vector>
#include <algorithm>

#include "refcl_prelude.h"

#define LUXRAYS_OPENCL_KERNEL 1
#define PARAM_RAY_EPSILON_MIN 1e-5f
#define PARAM_RAY_EPSILON_MAX 1e-1f
#define BVH_VERTS_PAGE_COUNT 1
#define BVH_NODES_PAGE_COUNT 1
#define BVH_VERTS_PAGE0 1
#define BVH_NODES_PAGE0 1

#undef NULL
#include "luxrays/luxrays_types.cl"
#include "luxrays/core/epsilon_types.cl"
#include "luxrays/core/epsilon_funcs.cl"
#include "luxrays/core/geometry/point_types.cl"
#include "luxrays/core/geometry/vector_types.cl"
#include "luxrays/core/geometry/ray_types.cl"
#include "luxrays/core/geometry/ray_funcs.cl"
#include "luxrays/core/geometry/bbox_types.cl"
#include "luxrays/core/geometry/bbox_funcs.cl"
#include "luxrays/core/geometry/triangle_types.cl"
#include "luxrays/core/geometry/triangle_funcs.cl"
#include "luxrays/core/bvh/bvhbuild_types.cl"
#include "luxrays/accelerators/bvh.cl"

static_assert(sizeof(Ray) == 48, "Ray");
static_assert(sizeof(RayHit) == 20, "RayHit");
static_assert(sizeof(BVHArrayNode) == 32, "BVHArrayNode");

extern "C" void refcl_bvh_trace(const void *rays, void *hits, unsigned int n,
		const void *verts, const void *nodes, int n_threads) {
	if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
	const unsigned int chunk = (n + n_threads - 1) / n_threads;
	std::vector<std::thread> th;
	for (int k = 0; k < n_threads; ++k) {
		const unsigned int b = k * chunk, e = std::min(n, b + chunk);
		if (b >= e) break;
		th.emplace_back([=]() {
			for (unsigned int i = b; i < e; ++i) {
				refcl_global_id = i;
				Accelerator_Intersect_RayBuffer((const Ray *)rays, (RayHit *)hits, n,
						(const Point *)verts, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
						(const BVHArrayNode *)nodes, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
			}
		});
	}
	for (auto &t : th) t.join();
}
