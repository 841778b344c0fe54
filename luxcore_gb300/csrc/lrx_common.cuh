// Device data layout and the FP32 geometry shared by the builder and the
// traversal kernels.
//
// HBM layout of a scene (all arrays 16-B aligned, indices absolute):
//   WideNode   nodes[]    80 B: 8-wide BVH node, child boxes quantised to
//                          8 bits per plane relative to a per-node origin and
//                          a power-of-two scale per axis, rounded outward.
//   TriRecord  tris[]     48 B: (p0, triangleIndex) (e1, meshIndex) (e2, 0),
//                          leaf-contiguous, e1 = p1 - p0 and e2 = p2 - p0
//                          formed in FP32 exactly as Triangle::Intersect does.
//   InstRecord insts[]    80 B: world->local matrix rows + BLAS root / object.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lrx {

constexpr uint32_t kNull = 0xffffffffu;
constexpr int kStackSize = 64;       // traversal stack entries per ray
constexpr int kMaxTreeDepth = 30;    // per tree; TLAS + BLAS + 1 <= kStackSize
constexpr uint32_t kInstGroup = 0x00800000u;  // stack entry holds instance bits
constexpr uint32_t kInternalMetaBase = 0x38u;  // meta byte of internal slot s: 0x38 + s = (1 << 5) | (24 + s)

// Status word bits (lrx_scene_device_status)
constexpr uint32_t kStatusStackOverflow = 1u;
constexpr uint32_t kStatusVisitLimit = 2u;
constexpr uint32_t kStatusDeadline = 4u;

// Node words:
//   w[0] = (px, py, pz, ex | ey << 8 | ez << 16 | imask << 24)
//   w[1] = (child_base, tri_base, meta[0..3], meta[4..7])
//   w[2] = (qlo_x[0..3], qlo_x[4..7], qlo_y[0..3], qlo_y[4..7])
//   w[3] = (qlo_z[0..3], qlo_z[4..7], qhi_x[0..3], qhi_x[4..7])
//   w[4] = (qhi_y[0..3], qhi_y[4..7], qhi_z[0..3], qhi_z[4..7])
// Child slot s is internal iff imask bit s; its node index is
// child_base + popc(imask & ((1 << s) - 1)).  Every meta byte is
// (bit run << 5) | bit position of a 32-bit hit mask: a leaf slot's is
// (unary triangle count << 5) | offset from tri_base (offsets < 24), an
// internal slot's is (1 << 5) | (24 + s) -- bit 24 + s, which traversal
// XORs with the ray's octant -- and an empty slot's is 0 (no bits).
struct alignas(16) WideNode {
	uint4 w[5];
};
static_assert(sizeof(WideNode) == 80, "WideNode is 80 bytes");

// The 64-byte record of a node with at most 4 children (LRX_NODES_COMPACT4):
//   w[0] = as WideNode's (origin, exponents, imask over the 8 octant slots)
//   w[1] = (child_base, tri_base, meta[0..3], qlo_x[0..3])
//   w[2] = (qlo_y[0..3], qlo_z[0..3], qhi_x[0..3], qhi_y[0..3])
//   w[3] = (qhi_z[0..3], 0, 0, 0)
// Position p holds the p-th occupied slot of the 80-byte record in slot
// order, with its meta byte unchanged: an internal child's still names its
// octant slot s (bit 24 + s), and its node index is still child_base +
// popc(imask & ((1 << s) - 1)).
struct alignas(16) Node4 {
	uint4 w[4];
};
static_assert(sizeof(Node4) == 64, "Node4 is 64 bytes");

struct alignas(16) TriRecord {
	float4 a, b, c;
};
static_assert(sizeof(TriRecord) == 48, "TriRecord is 48 bytes");

// rows r0..r3 of Transform::mInv (row-major); info = (BLAS root node,
// object index or kNull, flags, 0).  flags bit 0: identity (plain objects).
struct alignas(16) InstRecord {
	float4 r0, r1, r2, r3;
	uint4 info;
};
static_assert(sizeof(InstRecord) == 80, "InstRecord is 80 bytes");
constexpr uint32_t kInstIdentity = 1u;
// Motion instance: its transform is sampled at the ray's time from a motion
// system -- info.w = offset (in 16-byte units from the instance array's
// base) of its first MotionInterval, r0.x = their count (as uint bits).
constexpr uint32_t kInstMotion = 2u;

// One InterpolatedTransform of a motion system (motionsystem.cpp:33-160),
// decomposed on the host: start/end matrices, the rotation matrix of the
// start decomposition, scales, translations and unit quaternions (w,x,y,z).
// The parts of Slerp (quaternion.cpp:143-165) that depend only on the two
// quaternions -- the sign of their dot product, which branch it takes, and
// phi = acosf(|dot|), sinf(phi) -- are evaluated once on the host.
struct alignas(16) MotionInterval {
	uint32_t flags;
	float start_time, end_time, phi;
	float start_m[16], end_m[16], start_r[16];
	float s0[3], t0[3], s1[3], t1[3];
	float q0[4], q1[4];
	float sin_phi, pad[3];
};
static_assert(sizeof(MotionInterval) == 304, "MotionInterval is 304 bytes");
// MotionInterval::flags
constexpr uint32_t kMiActive = 1u, kMiRotation = 2u, kMiTransX = 4u, kMiTransY = 8u, kMiTransZ = 16u,
		   kMiScaleX = 32u, kMiScaleY = 64u, kMiScaleZ = 128u;
// Slerp of this interval: kMiSlerpLinear when 1 - |dot(q0, q1)| <= 1e-6
// (plain lerp weights), kMiSlerpNegate when dot(q0, q1) <= 0 (q1 negated)
constexpr uint32_t kMiSlerpLinear = 0x100u, kMiSlerpNegate = 0x200u;
constexpr uint32_t kMiTrans = kMiTransX | kMiTransY | kMiTransZ, kMiScale = kMiScaleX | kMiScaleY | kMiScaleZ;

#if defined(__CUDACC__)
// ---------------------------------------------------------------------------
// Round-to-nearest FP32 helpers: every product and sum rounds separately, so
// no FMA contraction changes a result relative to the reference's CPU code.
// ---------------------------------------------------------------------------

__device__ __forceinline__ float3 rn_sub(float3 a, float3 b) {
	return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}

// Dot(v1, v2) = v1.x*v2.x + v1.y*v2.y + v1.z*v2.z  (vector.h:151-153)
__device__ __forceinline__ float rn_dot(float3 a, float3 b) {
	return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

// Cross(v1, v2)  (vector.h:159-163)
__device__ __forceinline__ float3 rn_cross(float3 a, float3 b) {
	return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
			__fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
			__fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// Triangle::Intersect (include/luxrays/core/geometry/triangle.h:55-89) with
// e1 = p1 - p0 and e2 = p2 - p0 precomputed (same FP32 subtraction).  The
// reciprocal is the correctly rounded IEEE 1.f / divisor.  The maxt test is
// written so a NaN t fails it (the caller's `t < rayHit->t` would drop it);
// STRICT also fails t == maxt (that caller test, bvhaccel.cpp:233, folded in
// for any-hit).
template <bool STRICT>
__device__ __forceinline__ bool tri_intersect(float3 o, float3 d, float mint, float maxt,
		float3 p0, float3 e1, float3 e2, float &t, float &b1, float &b2) {
	const float3 s1 = rn_cross(d, e2);
	const float divisor = rn_dot(s1, e1);
	if (divisor == 0.f) return false;
	const float invDivisor = __frcp_rn(divisor);
	const float3 dv = rn_sub(o, p0);
	b1 = __fmul_rn(rn_dot(dv, s1), invDivisor);
	if (b1 < 0.f) return false;
	const float3 s2 = rn_cross(dv, e1);
	b2 = __fmul_rn(rn_dot(d, s2), invDivisor);
	if (b2 < 0.f) return false;
	const float b0 = __fsub_rn(__fsub_rn(1.f, b1), b2);
	if (b0 < 0.f) return false;
	t = __fmul_rn(rn_dot(e2, s2), invDivisor);
	// a NaN mint rejects nothing (as `t < ray.mint` in the reference); a NaN t
	// fails the maxt side
	if (t < mint) return false;
	return STRICT ? t < maxt : t <= maxt;
}

// InvTransform * Point (transform.h:144-156): three rows plus the w divide,
// skipped when w == 1 exactly.
__device__ __forceinline__ float3 xform_point(const float4 &r0, const float4 &r1, const float4 &r2,
		const float4 &r3, float3 p) {
	float3 q = make_float3(
			__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r0.x, p.x), __fmul_rn(r0.y, p.y)), __fmul_rn(r0.z, p.z)), r0.w),
			__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r1.x, p.x), __fmul_rn(r1.y, p.y)), __fmul_rn(r1.z, p.z)), r1.w),
			__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r2.x, p.x), __fmul_rn(r2.y, p.y)), __fmul_rn(r2.z, p.z)), r2.w));
	const float w = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r3.x, p.x), __fmul_rn(r3.y, p.y)), __fmul_rn(r3.z, p.z)), r3.w);
	if (w != 1.f) {
		const float inv = __frcp_rn(w);  // Point::operator/ (point.h:100-103)
		q = make_float3(__fmul_rn(inv, q.x), __fmul_rn(inv, q.y), __fmul_rn(inv, q.z));
	}
	return q;
}

// InvTransform * Vector (transform.h:186-193)
__device__ __forceinline__ float3 xform_vector(const float4 &r0, const float4 &r1, const float4 &r2, float3 v) {
	return make_float3(
			__fadd_rn(__fadd_rn(__fmul_rn(r0.x, v.x), __fmul_rn(r0.y, v.y)), __fmul_rn(r0.z, v.z)),
			__fadd_rn(__fadd_rn(__fmul_rn(r1.x, v.x), __fmul_rn(r1.y, v.y)), __fmul_rn(r1.z, v.z)),
			__fadd_rn(__fadd_rn(__fmul_rn(r2.x, v.x), __fmul_rn(r2.y, v.y)), __fmul_rn(r2.z, v.z)));
}

// MachineEpsilon::E(float) (epsilon.h:50-55): |bits(x)+0x80 - x| clamped to
// [1e-5, 1e-1].
__device__ __forceinline__ float machine_eps(float v) {
	const float n = __uint_as_float(__float_as_uint(v) + 0x80u);
	const float e = fabsf(__fsub_rn(n, v));
	return e > 1e-5f ? (e < 1e-1f ? e : 1e-1f) : 1e-5f;
}

// Order-preserving float <-> uint mapping for atomicMin/atomicMax on floats.
__device__ __forceinline__ uint32_t f2ord(float f) {
	const uint32_t u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
	return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

#endif  // __CUDACC__

}  // namespace lrx
