// Runs the reference's own MBVH kernel text (include/luxrays/accelerators/mbvh.cl
// and the .cl files it is stitched with, in the order of
// src/luxrays/accelerators/mbvhaccelhw.cpp:225-247, with one node page, one
// vertex page, transforms and motion systems) on the CPU, one work item at
// a time -- TEST INFRASTRUCTURE, built by oracle/build_ref.sh from the
// reference tree into oracle/_ref/ and used only to pin the oracle.  It
// walks the oracle's MBVH in MBVHKernel's upload layout (orc_mbvh_export).
#include <algorithm>
#include <thread>
#include <vector>

#include "refcl_prelude.h"
#include "lrx_oracle.h"

#define LUXRAYS_OPENCL_KERNEL 1
#define PARAM_RAY_EPSILON_MIN 1e-5f
#define PARAM_RAY_EPSILON_MAX 1e-1f
#define MBVH_VERTS_PAGE_COUNT 1
#define MBVH_NODES_PAGE_COUNT 1
#define MBVH_VERTS_PAGE0 1
#define MBVH_NODES_PAGE0 1
#define MBVH_HAS_TRANSFORMATIONS 1
#define MBVH_HAS_MOTIONSYSTEMS 1

#undef NULL
namespace refmbvh {

// OpenCL built-ins the motion / matrix / utility .cl files call, in single
// precision (std:: float overloads call acosf, sinf, ...)
static inline float acos(float x) { return std::acos(x); }
static inline float sin(float x) { return std::sin(x); }
static inline float cos(float x) { return std::cos(x); }
static inline float ceil(float x) { return std::ceil(x); }
static inline float floor(float x) { return std::floor(x); }
// OpenCL mix(x, y, a) = x + (y - x) * a
static inline float mix(float x, float y, float a) { return x + (y - x) * a; }
static inline float3 mix(const float3 &x, const float3 &y, float a) { return x + (y - x) * a; }
static inline int as_int(float f) { int i; std::memcpy(&i, &f, 4); return i; }
#define M_PI_F 3.14159265358979323846f

#include "luxrays/luxrays_types.cl"
#include "luxrays/core/epsilon_types.cl"
#include "luxrays/core/epsilon_funcs.cl"
#include "luxrays/core/geometry/point_types.cl"
#include "luxrays/core/geometry/vector_types.cl"
#include "luxrays/core/utils_funcs.cl"
#include "luxrays/core/geometry/matrix4x4_types.cl"
#include "luxrays/core/geometry/matrix4x4_funcs.cl"
#include "luxrays/core/geometry/quaternion_types.cl"
#include "luxrays/core/geometry/quaternion_funcs.cl"
#include "luxrays/core/geometry/ray_types.cl"
#include "luxrays/core/geometry/ray_funcs.cl"
#include "luxrays/core/geometry/bbox_types.cl"
#include "luxrays/core/geometry/bbox_funcs.cl"
#include "luxrays/core/geometry/transform_types.cl"
#include "luxrays/core/geometry/transform_funcs.cl"
#include "luxrays/core/geometry/motionsystem_types.cl"
#include "luxrays/core/geometry/motionsystem_funcs.cl"
#include "luxrays/core/geometry/triangle_types.cl"
#include "luxrays/core/geometry/triangle_funcs.cl"
#include "luxrays/core/bvh/bvhbuild_types.cl"
#include "luxrays/accelerators/mbvh.cl"

static_assert(sizeof(Ray) == 48, "Ray");
static_assert(sizeof(RayHit) == 20, "RayHit");
static_assert(sizeof(BVHArrayNode) == 32, "BVHArrayNode");

static void fill_decomposed(DecomposedTransform &d, const float R[16], const float st[6]) {
	std::memset(&d, 0, sizeof(d));
	d.Sx = st[0];
	d.Sy = st[1];
	d.Sz = st[2];
	std::memcpy(d.R.m, R, 64);
	d.Tx = st[3];
	d.Ty = st[4];
	d.Tz = st[5];
	d.Valid = true;
}

// The OpenCL InterpolatedTransform of one oracle interval (the reference
// byte-copies its C++ object, mbvhaccelhw.cpp:162-166).
static InterpolatedTransform to_ocl(const orc_interval &o) {
	InterpolatedTransform it;
	std::memset(&it, 0, sizeof(it));
	it.startTime = o.startTime;
	it.endTime = o.endTime;
	std::memcpy(it.start.m.m, o.start, 64);
	std::memcpy(it.end.m.m, o.end, 64);
	fill_decomposed(it.startT, o.R[0], o.ST[0]);
	fill_decomposed(it.endT, o.R[1], o.ST[1]);
	it.startQ.w = o.Q[0][0];
	it.startQ.v.x = o.Q[0][1];
	it.startQ.v.y = o.Q[0][2];
	it.startQ.v.z = o.Q[0][3];
	it.endQ.w = o.Q[1][0];
	it.endQ.v.x = o.Q[1][1];
	it.endQ.v.y = o.Q[1][2];
	it.endQ.v.z = o.Q[1][3];
	it.hasRotation = o.has[0];
	it.hasTranslation = o.has[1];
	it.hasScale = o.has[2];
	it.hasTranslationX = o.has[3];
	it.hasTranslationY = o.has[4];
	it.hasTranslationZ = o.has[5];
	it.hasScaleX = o.has[6];
	it.hasScaleY = o.has[7];
	it.hasScaleZ = o.has[8];
	it.isActive = o.has[9];
	return it;
}

}  // namespace refmbvh

extern "C" void refcl_mbvh_trace(const void *rays, void *hits, unsigned int n, const float *verts,
		const orc_bvh_node *nodes, unsigned long long n_nodes, const float *mats, unsigned long long n_mats,
		const uint32_t *motion_ranges, unsigned long long n_motions, const orc_interval *intervals,
		unsigned long long n_intervals, int n_threads) {
	using namespace refmbvh;
	// 16-byte aligned copies: the kernel reads nodes and matrices as float4
	std::vector<BVHArrayNode> nd(n_nodes);
	std::memcpy(nd.data(), nodes, 32 * n_nodes);
	std::vector<Matrix4x4> mx(std::max<unsigned long long>(1, n_mats));
	if (n_mats) std::memcpy(mx.data(), mats, 64 * n_mats);
	std::vector<MotionSystem> ms(std::max<unsigned long long>(1, n_motions));
	for (unsigned long long k = 0; k < n_motions; ++k) {
		ms[k].interpolatedTransformFirstIndex = motion_ranges[2 * k];
		ms[k].interpolatedTransformLastIndex = motion_ranges[2 * k + 1];
		ms[k].interpolatedInverseTransformFirstIndex = NULL_INDEX;
		ms[k].interpolatedInverseTransformLastIndex = NULL_INDEX;
	}
	std::vector<InterpolatedTransform> its(std::max<unsigned long long>(1, n_intervals));
	for (unsigned long long k = 0; k < n_intervals; ++k) its[k] = to_ocl(intervals[k]);
	if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
	const unsigned int chunk = (n + n_threads - 1) / n_threads;
	std::vector<std::thread> th;
	for (int k = 0; k < n_threads; ++k) {
		const unsigned int b = k * chunk, e = std::min(n, b + chunk);
		if (b >= e) break;
		th.emplace_back([=, &nd, &mx, &ms, &its]() {
			for (unsigned int i = b; i < e; ++i) {
				refcl_global_id = i;
				Accelerator_Intersect_RayBuffer((const Ray *)rays, (RayHit *)hits, n, mx.data(), ms.data(),
						its.data(), (const Point *)verts, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
						nullptr, nd.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
			}
		});
	}
	for (auto &t : th) t.join();
}
