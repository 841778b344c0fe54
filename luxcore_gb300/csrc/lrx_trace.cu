// Ray traversal kernels: closest-hit and any-hit queries of luxrays::Ray
// buffers against the 8-wide compressed BVH, flat (one BVH over all plain
// meshes) or two-level (top-level BVH over objects, each leaf an instance
// record with the world->local transform of an instanced mesh).
//
// Replaces the reference's GPU kernels Accelerator_Intersect_RayBuffer of
// include/luxrays/accelerators/bvh.cl:45-260 and mbvh.cl:61-383 and the CPU
// walks BVHAccel::Intersect / MBVHAccel::Intersect
// (src/luxrays/accelerators/bvhaccel.cpp:170-260, mbvhaccel.cpp:252-357).
// Results follow the CPU semantics: closest hit with t in [mint, maxt] from
// the same FP32 Triangle::Intersect; at equal t the lowest
// (meshIndex, triangleIndex) wins, so the answer does not depend on the
// traversal order.  Masked rays are skipped without writing (bvh.cl:243-244);
// rays with a NaN or infinite origin/direction component, or a NaN maxt,
// are misses.
//
// Loop structure (after Ylitie, Karras and Laine 2017): a node group (child
// base + 8 internal-child hit bits in octant order + the internal mask) and
// a triangle group (triangle base + 24 hit bits) per lane.  One node is
// expanded per iteration; the triangles it yields are tested right away
// unless fewer than `postpone` lanes of the warp are testing triangles at
// that moment (__activemask, no waiting) while node work remains -- then the
// group is pushed and tested later, which keeps lanes in step.
#include <algorithm>
#include <atomic>

#include "lrx_common.cuh"
#include "lrx_internal.h"

namespace lrx {

struct ActiveRay {
	float3 o, d, idir;
	uint32_t oct;
};

__device__ __forceinline__ void make_active(ActiveRay &r, float3 o, float3 d) {
	r.o = o;
	r.d = d;
	r.idir = make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
	r.oct = (r.idir.x < 0.f ? 1u : 0u) | (r.idir.y < 0.f ? 2u : 0u) | (r.idir.z < 0.f ? 4u : 0u);
}

struct NodeHits {
	uint32_t child_base, tri_base, imask;
	uint32_t ihits;  // internal children, bit j = slot (j ^ oct)
	uint32_t tmask;  // leaf triangles, bit k = triangle tri_base + k
};

// Variant bits (lrx_trace_config.variant):
constexpr uint32_t kVarMinMax3 = 1u;      // compile time: 3-input min/max for the slab tests
constexpr uint32_t kVarSceneEvictLast = 2u;  // runtime: node/triangle loads keep L2 lines (evict_last)
constexpr uint32_t kVarStreamRays = 4u;   // runtime: ray loads / hit stores stream past L2 (evict_first)
constexpr uint32_t kVarOccupancy = 8u;    // compile time: register budget for 20 blocks of 64 per SM

// 3-input max / min (max.f32 d, a, b, c on sm_100+): a NaN input is
// dropped like fmaxf/fminf drop it.
__device__ __forceinline__ float max3f(float a, float b, float c) {
	float d;
	asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
	return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
	float d;
	asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
	return d;
}

__device__ __forceinline__ uint64_t evict_last_policy() {
	uint64_t pol;
	asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
	return pol;
}

// Read-only 16-B scene load, optionally with an L2 evict_last policy.
__device__ __forceinline__ uint4 ld_scene(const uint4 *p, bool keep, uint64_t pol) {
	if (!keep) return __ldg(p);
	uint4 v;
	asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
			: "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p), "l"(pol));
	return v;
}

__device__ __forceinline__ float4 ld_scene_f4(const float4 *p, bool keep, uint64_t pol) {
	const uint4 v = ld_scene(reinterpret_cast<const uint4 *>(p), keep, pol);
	return make_float4(__uint_as_float(v.x), __uint_as_float(v.y), __uint_as_float(v.z), __uint_as_float(v.w));
}

// Packed FP32 pair arithmetic (fma.rn.f32x2 / add.rn.f32x2, sm_100+): each
// half is rounded exactly like the scalar fmaf / __fadd_rn.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
	float2 d;
	asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\t"
	    "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\tmov.b64 pc, {%6, %7};\n\t"
	    "fma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;\n\t}"
			: "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
	return d;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
	float2 d;
	asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
	    "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
	    "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
			: "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
	return d;
}

// Plane distances of slots (4H + K, 4H + K + 1) on one axis: quantised bytes
// K, K+1 of w -> exact floats (PRMT builds 2^23 + b, the packed add takes
// 2^23 off exactly), then t = q * a + b per half, one rounding each.
template <int K>
__device__ __forceinline__ float2 plane_pair(uint32_t w, float a, float b) {
	const float2 q = make_float2(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + K)),
			__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + K + 1)));
	return fma2(add2(q, make_float2(-8388608.f, -8388608.f)), make_float2(a, a), make_float2(b, b));
}

// Slab test of the 8 quantised child boxes (N4: the 4 of a 64-byte
// record).  t = q * (scale * idir) + (origin - o) * idir; NaN plane
// distances (zero direction components) are dropped by fminf/fmaxf, which
// only ever keeps a child.  A hit child adds its meta bits to one 32-bit
// mask -- bits 0-23 its triangles, bit 24 + (slot ^ octant) an internal
// child -- with the octant XOR and the bit fields taken for four children at
// a time from a meta word; empty positions (meta 0) add nothing whatever
// their planes.
template <bool MM3, bool N4 = false>
__device__ __forceinline__ NodeHits intersect_node(const WideNode *__restrict__ nodes, uint32_t idx,
		const ActiveRay &r, float tmin, float tmax, bool keep, uint64_t pol) {
	constexpr int kWords = N4 ? 4 : 5;  // 16-byte words per record
	const uint4 *p = reinterpret_cast<const uint4 *>(nodes) + (size_t)kWords * idx;
	const uint4 w0 = ld_scene(p, keep, pol), w1 = ld_scene(p + 1, keep, pol), w2 = ld_scene(p + 2, keep, pol),
			w3 = ld_scene(p + 3, keep, pol);
	const uint4 w4 = N4 ? make_uint4(0u, 0u, 0u, 0u) : ld_scene(p + 4, keep, pol);
	NodeHits h;
	h.child_base = w1.x;
	h.tri_base = w1.y;
	h.imask = w0.w >> 24;
	const float sx = __uint_as_float((w0.w & 0xffu) << 23);
	const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
	const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
	const float ax = sx * r.idir.x, ay = sy * r.idir.y, az = sz * r.idir.z;
	const float bx = (__uint_as_float(w0.x) - r.o.x) * r.idir.x;
	const float by = (__uint_as_float(w0.y) - r.o.y) * r.idir.y;
	const float bz = (__uint_as_float(w0.z) - r.o.z) * r.idir.z;
	const bool px = r.idir.x >= 0.f, py = r.idir.y >= 0.f, pz = r.idir.z >= 0.f;
	// 80-byte record: qlo_x = w2.xy, qlo_y = w2.zw, qlo_z = w3.xy, qhi_x = w3.zw, qhi_y = w4.xy,
	// qhi_z = w4.zw, meta = w1.zw; 64-byte record: qlo_x = w1.w, qlo_y = w2.x, qlo_z = w2.y,
	// qhi_x = w2.z, qhi_y = w2.w, qhi_z = w3.x, meta = w1.z (one word each, four children)
	const uint32_t qlx[2] = {N4 ? w1.w : w2.x, w2.y}, qly[2] = {N4 ? w2.x : w2.z, w2.w};
	const uint32_t qlz[2] = {N4 ? w2.y : w3.x, w3.y}, qhx[2] = {N4 ? w2.z : w3.z, w3.w};
	const uint32_t qhy[2] = {N4 ? w2.w : w4.x, w4.y}, qhz[2] = {N4 ? w3.x : w4.z, w4.w};
	const uint32_t nx[2] = {px ? qlx[0] : qhx[0], px ? qlx[1] : qhx[1]};
	const uint32_t fx[2] = {px ? qhx[0] : qlx[0], px ? qhx[1] : qlx[1]};
	const uint32_t ny[2] = {py ? qly[0] : qhy[0], py ? qly[1] : qhy[1]};
	const uint32_t fy[2] = {py ? qhy[0] : qly[0], py ? qhy[1] : qly[1]};
	const uint32_t nz[2] = {pz ? qlz[0] : qhz[0], pz ? qlz[1] : qhz[1]};
	const uint32_t fz[2] = {pz ? qhz[0] : qlz[0], pz ? qhz[1] : qlz[1]};
	// per meta word: bit position (internal slots XORed with the octant) and bit run, bytewise
	uint32_t bpos[2] = {0u, 0u}, brun[2] = {0u, 0u};
#pragma unroll
	for (int H = 0; H < (N4 ? 1 : 2); ++H) {
		const uint32_t m4 = H ? w1.w : w1.z;
		const uint32_t inner4 = (m4 & (m4 << 1)) & 0x10101010u;  // bits 4 and 3 set: position >= 24
		bpos[H] = (m4 ^ ((inner4 >> 4) * r.oct)) & 0x1f1f1f1fu;
		brun[H] = (m4 >> 5) & 0x07070707u;
	}
	uint32_t hm = 0;
#define LRX_PAIR(S)                                                                                   \
	{                                                                                                 \
		constexpr int H = (S) >> 2, K = (S) & 3;                                                      \
		const float2 tnx = plane_pair<K>(nx[H], ax, bx), tny = plane_pair<K>(ny[H], ay, by);          \
		const float2 tnz = plane_pair<K>(nz[H], az, bz);                                              \
		const float2 tfx = plane_pair<K>(fx[H], ax, bx), tfy = plane_pair<K>(fy[H], ay, by);          \
		const float2 tfz = plane_pair<K>(fz[H], az, bz);                                              \
		const float tn0 = MM3 ? fmaxf(max3f(tnx.x, tny.x, tnz.x), tmin)                              \
				: fmaxf(fmaxf(tnx.x, tny.x), fmaxf(tnz.x, tmin));                                     \
		const float tf0 = MM3 ? fminf(min3f(tfx.x, tfy.x, tfz.x), tmax)                              \
				: fminf(fminf(tfx.x, tfy.x), fminf(tfz.x, tmax));                                     \
		const float tn1 = MM3 ? fmaxf(max3f(tnx.y, tny.y, tnz.y), tmin)                              \
				: fmaxf(fmaxf(tnx.y, tny.y), fmaxf(tnz.y, tmin));                                     \
		const float tf1 = MM3 ? fminf(min3f(tfx.y, tfy.y, tfz.y), tmax)                              \
				: fminf(fminf(tfx.y, tfy.y), fminf(tfz.y, tmax));                                     \
		if (tn0 <= tf0) hm |= ((brun[H] >> (8 * K)) & 0xffu) << ((bpos[H] >> (8 * K)) & 0xffu);      \
		if (tn1 <= tf1) hm |= ((brun[H] >> (8 * K + 8)) & 0xffu) << ((bpos[H] >> (8 * K + 8)) & 0xffu); \
	}
	LRX_PAIR(0) LRX_PAIR(2)
	if (!N4) {
		LRX_PAIR(4) LRX_PAIR(6)
	}
#undef LRX_PAIR
	h.ihits = hm >> 24;
	h.tmask = hm & 0x00ffffffu;
	return h;
}

__device__ __forceinline__ bool finite3(float3 v) {
	return isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
}

struct Counts {
	uint32_t nodes, tris, insts, rays;
};

// Traversal state of one ray between loop trips.
struct TravState {
	ActiveRay ray;             // in the current BVH's space (world, or an instance's local space)
	float3 wo, wd;             // world-space origin / direction
	float mint, best_t, best_b1, best_b2;
	float time;                // the ray's time (motion instances)
	uint32_t best_mesh, best_tri;
	uint32_t inst_obj;         // object of the instance being traversed (kNull at top level)
	uint32_t visits;
	int sp, inst_sp;           // stack depth; depth at which the current BLAS was entered (-1: none)
	uint2 ng, tg;              // node group, triangle (or instance) group
};
// The traversal stack lives apart from TravState so that the state's scalars
// stay in registers (a dynamically indexed member would put the whole
// struct in local memory).  With a shared-memory stack (LRX_VARIANT_SMEM_STACK,
// _SMEM_STACK16, _SMEM_STACK32) its first SD = 8, 16 or 32 entries -- the top
// of a short stack, where nearly all pushes and pops land -- are in shared
// memory instead, thread t's entry e at top[e * blockDim.x] (consecutive
// lanes in consecutive 8-byte words, no bank conflicts); deeper entries, the
// fallback when a walk goes deeper, stay in local memory.  SD trades
// local-memory traffic against shared memory (8 * SD bytes per thread, taken
// from the SM's L1) -- a per-scene choice of the autotuner.
typedef uint2 TravStack[kStackSize];
struct StackTop {
	uint2 *top;
	uint32_t stride;
};
template <int SD>
__device__ __forceinline__ void stack_put(TravStack &st, StackTop t, int i, uint2 v) {
	if (SD > 0 && i < SD) t.top[i * t.stride] = v;
	else st[i] = v;
}
template <int SD>
__device__ __forceinline__ uint2 stack_get(const TravStack &st, StackTop t, int i) {
	if (SD > 0 && i < SD) return t.top[i * t.stride];
	return st[i];
}

enum : int { kRayMasked = 0, kRayAnswered = 1, kRayTraverse = 2 };

// ---------------------------------------------------------------------------
// Launch deadline, counted in %globaltimer ticks of 1,024 ns (~1 us) from the
// launch's start: the first time any of its blocks or warps looked, kept in
// the launch's counter slot (zeroed again after the launch, so every
// execution, graph replays included, starts afresh).  It is checked only
// where rays are about to start, never inside a ray's walk -- a started ray
// is bounded by its visit budget:
// - persistent kernels: the claiming lane reads the timer on the claim that
//   crosses each kDeadlineCheckRays boundary of the claim counter; once the
//   deadline has passed it sets bit 31 of the counter, so every later claim
//   of the launch sees it in its atomic's return value and starts no ray;
// - one-ray-per-thread kernels: thread 0 of each block checks once, at the
//   block's start (or per tile in the tile queue kernel); a late block starts
//   none of its rays.
// ---------------------------------------------------------------------------
constexpr uint32_t kDeadlineCheckRays = 2048;
constexpr uint32_t kClaimLate = 0x80000000u;  // claims stay below 2^31 (kMaxFetchRays)

__device__ __forceinline__ uint32_t now_ticks() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return (uint32_t)(t >> 10);
}

// Per-launch counter slots of 256 bytes: words 0-3 claim counters (one per
// ray class of a queue launch; single-batch kernels use word 0), word 4 the
// count of blocks that have stopped claiming, word 32 -- a cache line of its
// own, away from the claim atomics -- the launch's start (its first reader's
// time in timer ticks | 1, so that 0 means not yet).
constexpr int kSlotWords = 64, kSlotFinished = 4, kSlotStart = 32;
__device__ uint32_t g_queue[kQueueSlots][kSlotWords];

// The launch's start.  Only the installer (one caller per launch) writes it;
// any other caller that finds it not yet written takes its own time, which is
// later and so only more lenient.  (Slot words are zero when a launch begins
// and are zeroed again after it; no compare-and-swap, so the first wave of
// blocks does not queue on one address.)
__device__ __forceinline__ uint32_t slot_start(uint32_t *slot, bool installer) {
	const uint32_t v = *reinterpret_cast<volatile uint32_t *>(&slot[kSlotStart]);
	if (v != 0u) return v;
	const uint32_t mine = now_ticks() | 1u;
	if (installer) *reinterpret_cast<volatile uint32_t *>(&slot[kSlotStart]) = mine;
	return mine;
}

// Slot protocol shared by the persistent kernels: a launch owns a slot, all
// zero at entry; every block adds itself to the finished count once it has
// stopped claiming work, and the last one zeroes the slot for its next user.
__device__ __forceinline__ void release_slot(uint32_t *slot) {
	if (threadIdx.x == 0) {
		__threadfence();
		if (atomicAdd(&slot[kSlotFinished], 1u) == gridDim.x - 1) {  // every block has stopped claiming work
#pragma unroll
			for (int w = 0; w < kSlotWords; ++w) slot[w] = 0u;
			__threadfence();
		}
	}
}

// The start a block counts the deadline from, and (one-ray-per-thread
// kernels) whether the block found the deadline passed; one copy per block.
__shared__ uint32_t s_launch_start, s_block_late;

// Block start (all threads of the block) of a persistent kernel: all of its
// blocks are resident from the launch's start, so each counts from its own
// start, with no memory access; expiry spreads through the claim counter.
__device__ __forceinline__ void note_block_start() {
	if (threadIdx.x == 0) s_launch_start = now_ticks();
	__syncthreads();
}

// True once `deadline_ticks` (non-zero, below 2^31) has passed since
// `start`.  The difference is signed: a reading a tick behind `start` (timer
// skew between SMs) is not past, and the timer's 2^32 wrap does not matter.
__device__ __forceinline__ bool past_deadline(uint32_t start, uint32_t deadline_ticks) {
	return deadline_ticks != 0u && (int32_t)(now_ticks() - start) > (int32_t)deadline_ticks;
}

// The claiming lane's deadline test (persistent kernels): `base` is the
// claim's atomicAdd result on `counter`.  Returns base, with kClaimLate set
// when the claim must start no ray.
__device__ __forceinline__ uint32_t claim_deadline(uint32_t base, uint32_t nidle, uint32_t *counter, uint32_t start,
		uint32_t deadline_ticks) {
	if (!(base & kClaimLate) && (base & (kDeadlineCheckRays - 1u)) < nidle && past_deadline(start, deadline_ticks)) {
		atomicOr(counter, kClaimLate);  // every later claim of the launch sees it
		base |= kClaimLate;
	}
	return base;
}

// ---------------------------------------------------------------------------
// Motion instances: the transform at a ray's time, from the host-decomposed
// intervals -- MotionSystem::Sample and InterpolatedTransform::Sample
// (src/luxrays/core/geometry/motionsystem.cpp:56-160, 333-337; the GPU
// kernel's MotionSystem_Sample, motionsystem_funcs.cl:21-115), with every
// product and sum rounded separately as in the CPU code.  Slerp's constant
// part (phi = acosf(|dot|), sinf(phi)) is evaluated on the host; its two
// time-dependent sines are CUDA's sinf, so a rotating instance's matrix can
// differ from the CPU's in the last bits, as the reference's own CPU and GPU
// paths differ.
// ---------------------------------------------------------------------------

struct MotionRows {
	float4 r0, r1, r2, r3;
};

__device__ __forceinline__ float lerp_rn(float t, float a, float b) {
	return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a)));
}

__device__ __forceinline__ MotionRows motion_sample(const MotionInterval *its, uint32_t n, float time) {
	uint32_t k = n - 1;  // the interval ending after `time` (upper_bound over the keyframe times)
	for (uint32_t i = 0; i < n; ++i)
		if (time < __ldg(&its[i].end_time)) {
			k = i;
			break;
		}
	const MotionInterval *it = its + k;
	const uint32_t f = __ldg(&it->flags);
	const float st = __ldg(&it->start_time), et = __ldg(&it->end_time);
	float m[16];
	if (!(f & kMiActive) || time <= st || time >= et) {
		const float *src = (!(f & kMiActive) || time <= st) ? it->start_m : it->end_m;
#pragma unroll
		for (int j = 0; j < 16; ++j) m[j] = __ldg(src + j);
	} else {
		const float le = __fdiv_rn(__fsub_rn(time, st), __fsub_rn(et, st));
		if ((f & kMiTrans) && !(f & (kMiScale | kMiRotation))) {  // translation only
#pragma unroll
			for (int j = 0; j < 16; ++j) m[j] = __ldg(it->start_m + j);
			if (f & kMiTransX) m[3] = lerp_rn(le, __ldg(&it->t0[0]), __ldg(&it->t1[0]));
			if (f & kMiTransY) m[7] = lerp_rn(le, __ldg(&it->t0[1]), __ldg(&it->t1[1]));
			if (f & kMiTransZ) m[11] = lerp_rn(le, __ldg(&it->t0[2]), __ldg(&it->t1[2]));
		} else {
			if (f & kMiRotation) {
				// Slerp (quaternion.cpp:143-165) then ToMatrix (:116-141)
				const float aw = __ldg(&it->q0[0]), ax = __ldg(&it->q0[1]), ay = __ldg(&it->q0[2]), az = __ldg(&it->q0[3]);
				const float bw = __ldg(&it->q1[0]), bx = __ldg(&it->q1[1]), by = __ldg(&it->q1[2]), bz = __ldg(&it->q1[3]);
				// sign, branch, phi and sinf(phi) come from the host (the same
				// float operations as the CPU's Slerp); the two time-dependent
				// sines are CUDA's sinf
				const float sign = (f & kMiSlerpNegate) ? -1.f : 1.f;
				float f1, f2;
				if (!(f & kMiSlerpLinear)) {
					const float phi = __ldg(&it->phi), sin_phi = __ldg(&it->sin_phi);
					f1 = __fdiv_rn(sinf(__fmul_rn(__fsub_rn(1.f, le), phi)), sin_phi);
					f2 = __fdiv_rn(sinf(__fmul_rn(le, phi)), sin_phi);
				} else {
					f1 = __fsub_rn(1.f, le);
					f2 = le;
				}
				const float g = __fmul_rn(sign, f2);
				const float w = __fadd_rn(__fmul_rn(aw, f1), __fmul_rn(bw, g));
				const float x = __fadd_rn(__fmul_rn(f1, ax), __fmul_rn(g, bx));
				const float y = __fadd_rn(__fmul_rn(f1, ay), __fmul_rn(g, by));
				const float z = __fadd_rn(__fmul_rn(f1, az), __fmul_rn(g, bz));
				const float xx = __fmul_rn(x, x), yy = __fmul_rn(y, y), zz = __fmul_rn(z, z);
				const float xy = __fmul_rn(x, y), xz = __fmul_rn(x, z), yz = __fmul_rn(y, z);
				const float xw = __fmul_rn(x, w), yw = __fmul_rn(y, w), zw = __fmul_rn(z, w);
				m[0] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(yy, zz)));
				m[4] = __fmul_rn(2.f, __fsub_rn(xy, zw));
				m[8] = __fmul_rn(2.f, __fadd_rn(xz, yw));
				m[1] = __fmul_rn(2.f, __fadd_rn(xy, zw));
				m[5] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(xx, zz)));
				m[9] = __fmul_rn(2.f, __fsub_rn(yz, xw));
				m[2] = __fmul_rn(2.f, __fsub_rn(xz, yw));
				m[6] = __fmul_rn(2.f, __fadd_rn(yz, xw));
				m[10] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(xx, yy)));
				m[3] = m[7] = m[11] = 0.f;
				m[12] = m[13] = m[14] = 0.f;
				m[15] = 1.f;
			} else {
#pragma unroll
				for (int j = 0; j < 16; ++j) m[j] = __ldg(it->start_r + j);
			}
			float S[3];
#pragma unroll
			for (int c = 0; c < 3; ++c)
				S[c] = (f & kMiScale) ? lerp_rn(le, __ldg(&it->s0[c]), __ldg(&it->s1[c])) : __ldg(&it->s0[c]);
#pragma unroll
			for (int row = 0; row < 3; ++row)
#pragma unroll
				for (int j = 0; j < 3; ++j) m[4 * row + j] = __fmul_rn(S[row], m[4 * row + j]);
			m[3] = (f & kMiTransX) ? lerp_rn(le, __ldg(&it->t0[0]), __ldg(&it->t1[0])) : __ldg(&it->t0[0]);
			m[7] = (f & kMiTransY) ? lerp_rn(le, __ldg(&it->t0[1]), __ldg(&it->t1[1])) : __ldg(&it->t0[1]);
			m[11] = (f & kMiTransZ) ? lerp_rn(le, __ldg(&it->t0[2]), __ldg(&it->t1[2])) : __ldg(&it->t0[2]);
		}
	}
	MotionRows r;
	r.r0 = make_float4(m[0], m[1], m[2], m[3]);
	r.r1 = make_float4(m[4], m[5], m[6], m[7]);
	r.r2 = make_float4(m[8], m[9], m[10], m[11]);
	r.r3 = make_float4(m[12], m[13], m[14], m[15]);
	return r;
}

// Reads ray i and sets up its traversal.  kRayMasked: skip it and write
// nothing (bvh.cl:243-244); kRayAnswered: the initial miss (t = maxt) is the
// answer -- empty scene, NaN/infinite origin or direction, NaN maxt;
// kRayTraverse: traverse.
__device__ __forceinline__ int ray_begin(const TraceArgs &a, uint32_t i, bool stream, TravState &s) {
	const float4 *rp = reinterpret_cast<const float4 *>(a.rays) + 3 * (size_t)i;
	float4 r0, r1, r2;
	if (stream) {
		r0 = __ldcs(rp);
		r1 = __ldcs(rp + 1);
		r2 = __ldcs(rp + 2);
	} else {
		r0 = __ldg(rp);
		r1 = __ldg(rp + 1);
		r2 = __ldg(rp + 2);
	}
	if (__float_as_uint(r2.y) & LRX_RAY_FLAGS_MASKED) return kRayMasked;
	s.wo = make_float3(r0.x, r0.y, r0.z);
	s.wd = make_float3(r0.w, r1.x, r1.y);
	s.mint = r1.z;
	s.best_t = r1.w;
	s.time = r2.x;
	s.best_b1 = 0.f;
	s.best_b2 = 0.f;
	s.best_mesh = kNull;
	s.best_tri = kNull;
	if (a.root == kNull || !finite3(s.wo) || !finite3(s.wd) || isnan(s.best_t)) return kRayAnswered;
	make_active(s.ray, s.wo, s.wd);
	s.sp = 0;
	s.inst_sp = -1;
	s.inst_obj = kNull;
	s.visits = 0;
	s.ng = make_uint2(a.root, (1u << (24 + s.ray.oct)) | 1u);
	s.tg = make_uint2(0u, 0u);
	return kRayTraverse;
}

// One trip of the traversal loop: expand one node (or take a popped group),
// test the triangles it yields (or enter one instance), pop when the node
// group is spent.  Returns true when the ray is finished: stack empty, any
// hit found, or abandoned -- stack overflow or visit budget spent, recorded
// in the status word, and s.sp set to -1 so the caller writes no hit.
// Every trip either expands a node -- spending the visit budget, which only
// instance entries raise, each by a bounded amount once per instance leaf
// bit -- or consumes a stack entry or an instance bit, so a ray finishes in
// a bounded number of trips.
// `sparse` (persistent kernels): the warp's ray counter is spent and fewer
// lanes than `postpone` still hold rays.  Triangle groups are then tested at
// once: deferring them could not gather `postpone` lanes any more, and only
// adds trips and delays the shrinking of t (bounce rays -0.7 % launch time).
//
// No path returns before the node test or the triangle loop: a push past
// the stack's end is dropped and counted, and the stack and visit bounds are
// checked once, at the end of the trip (before any pop, so a dropped entry
// is never read).  An early return on those never-taken paths would leave
// the lanes that pushed and those that did not without a point to
// reconverge before the node test, which the warp then ran twice.
template <bool ANY, bool TWO_LEVEL, bool COUNT, bool MM3, int SMEM = 0, bool MOTION = false, bool N4 = false>
__device__ __forceinline__ bool ray_step(const TraceArgs &a, TravState &s, TravStack &stack, bool keep, uint64_t pol,
		Counts &c, StackTop top = StackTop{nullptr, 0}, bool sparse = false) {
#define LRX_PUSH(V)                                                     \
	{                                                                   \
		if (s.sp < kStackSize) stack_put<SMEM>(stack, top, s.sp, (V));  \
		++s.sp;                                                         \
	}
	// the trip's bounds: a stack that overflowed, or the visit budget spent,
	// abandons the ray (status word bit, no hit written)
#define LRX_BOUNDS()                                                                              \
	if (s.sp > kStackSize || s.visits > a.visit_limit) {                                         \
		atomicOr(a.status, s.sp > kStackSize ? kStatusStackOverflow : kStatusVisitLimit);        \
		s.sp = -1;                                                                               \
		return true;                                                                             \
	}
	if (s.ng.y > 0x00ffffffu) {
		const uint32_t j = __ffs(s.ng.y >> 24) - 1;
		s.ng.y &= ~(1u << (24 + j));
		const uint32_t sl = j ^ s.ray.oct;
		const uint32_t node = s.ng.x + __popc(s.ng.y & ((1u << sl) - 1u) & 0xffu);
		if (s.ng.y > 0x00ffffffu) LRX_PUSH(s.ng);
		++s.visits;
		if (COUNT) ++c.nodes;
		const NodeHits h = intersect_node<MM3, N4>(a.nodes, node, s.ray, s.mint, s.best_t, keep, pol);
		s.ng = make_uint2(h.child_base, (h.ihits << 24) | h.imask);
		s.tg = make_uint2(h.tri_base, h.tmask);
	} else {
		s.tg = s.ng;  // a popped triangle (or, at top level, instance) group
		s.ng = make_uint2(0u, 0u);
	}
	if (TWO_LEVEL && s.inst_sp < 0) {
		if (s.tg.y) {
			// top-level leaf: enter one instance, keep the rest for later
			const uint32_t k = __ffs(s.tg.y) - 1;
			s.tg.y &= s.tg.y - 1;
			if (s.ng.y > 0x00ffffffu) LRX_PUSH(s.ng);
			if (s.tg.y) LRX_PUSH(s.tg);
			const InstRecord *ir = a.insts + s.tg.x + k;
			const uint4 info = __ldg(reinterpret_cast<const uint4 *>(&ir->info));
			if (COUNT) ++c.insts;
			s.inst_obj = info.y;
			s.visits -= min(a.blas_visits, s.visits);  // credit for the BLAS's walk
			if (info.z & kInstIdentity) {
				make_active(s.ray, s.wo, s.wd);
			} else if (MOTION && (info.z & kInstMotion)) {
				const MotionRows m = motion_sample(
						reinterpret_cast<const MotionInterval *>(reinterpret_cast<const char *>(a.insts) + 16ull * info.w),
						__float_as_uint(__ldg(&ir->r0.x)), s.time);
				make_active(s.ray, xform_point(m.r0, m.r1, m.r2, m.r3, s.wo), xform_vector(m.r0, m.r1, m.r2, s.wd));
			} else {
				const float4 m0 = __ldg(&ir->r0), m1 = __ldg(&ir->r1), m2 = __ldg(&ir->r2), m3 = __ldg(&ir->r3);
				make_active(s.ray, xform_point(m0, m1, m2, m3, s.wo), xform_vector(m0, m1, m2, s.wd));
			}
			s.inst_sp = s.sp;
			s.ng = info.x == kNull ? make_uint2(0u, 0u) : make_uint2(info.x, (1u << (24 + s.ray.oct)) | 1u);
			s.tg = make_uint2(0u, 0u);
			LRX_BOUNDS()
			return false;
		}
	} else {
		// Any-hit never defers: the hit it returns must depend only on the
		// ray and the tree, not on which rays share its warp.  The decision is
		// taken once per trip, as the lanes enter the triangle stage (taking it
		// again every iteration deferred a group in mid-loop too rarely to pay
		// for the test: bounce rays -0.7 %).
		if (!ANY && !sparse && s.tg.y && s.ng.y > 0x00ffffffu && __popc(__activemask()) < a.postpone) {
			LRX_PUSH(s.tg);  // test later, when the warp does triangles together
			s.tg.y = 0;
		}
		while (s.tg.y) {
			const uint32_t k = __ffs(s.tg.y) - 1;
			s.tg.y &= s.tg.y - 1;
			const float4 *tp = reinterpret_cast<const float4 *>(a.tris + s.tg.x + k);
			const float4 ta = ld_scene_f4(tp, keep, pol), tb = ld_scene_f4(tp + 1, keep, pol),
					tc = ld_scene_f4(tp + 2, keep, pol);
			if (COUNT) ++c.tris;
			float t, b1, b2;
			if (tri_intersect<ANY>(s.ray.o, s.ray.d, s.mint, s.best_t, make_float3(ta.x, ta.y, ta.z),
					make_float3(tb.x, tb.y, tb.z), make_float3(tc.x, tc.y, tc.z), t, b1, b2)) {
				const uint32_t tri = __float_as_uint(ta.w);
				uint32_t mesh = __float_as_uint(tb.w);
				if (TWO_LEVEL && mesh == kNull) mesh = s.inst_obj;
				// a hit counts only below the current t, as the reference's
				// `t < rayHit->t` (a NaN t, or t == maxt with no hit yet, never
				// does; tri_intersect has let only t <= best_t through, and for
				// any-hit only t < best_t); an exact tie with an earlier hit goes
				// to the lower (meshIndex, triangleIndex)
				if (ANY || t < s.best_t || (s.best_mesh != kNull &&
						(mesh < s.best_mesh || (mesh == s.best_mesh && tri < s.best_tri)))) {
					s.best_t = t;
					s.best_b1 = b1;
					s.best_b2 = b2;
					s.best_mesh = mesh;
					s.best_tri = tri;
					if (ANY) return true;
				}
			}
		}
	}
	LRX_BOUNDS()
	if (s.ng.y <= 0x00ffffffu) {
		if (TWO_LEVEL && s.inst_sp == s.sp) {  // this instance's BLAS is exhausted
			s.inst_sp = -1;
			s.inst_obj = kNull;
			make_active(s.ray, s.wo, s.wd);
		}
		if (s.sp == 0) return true;
		s.ng = stack_get<SMEM>(stack, top, --s.sp);
	}
	return false;
#undef LRX_BOUNDS
#undef LRX_PUSH
}

__device__ __forceinline__ void ray_write(const TraceArgs &a, uint32_t i, const TravState &s, bool stream) {
	uint32_t *hp = reinterpret_cast<uint32_t *>(a.hits) + 5 * (size_t)i;
	if (stream) {
		__stcs(hp, __float_as_uint(s.best_t));
		__stcs(hp + 1, __float_as_uint(s.best_b1));
		__stcs(hp + 2, __float_as_uint(s.best_b2));
		__stcs(hp + 3, s.best_mesh);
		__stcs(hp + 4, s.best_tri);
	} else {
		hp[0] = __float_as_uint(s.best_t);
		hp[1] = __float_as_uint(s.best_b1);
		hp[2] = __float_as_uint(s.best_b2);
		hp[3] = s.best_mesh;
		hp[4] = s.best_tri;
	}
}

// Traces ray `tid` of the batch `a` (through a.order when set) and writes its
// hit, unless the ray is abandoned.  Shared by the one-batch kernel and the
// multi-batch tile queue kernel (which test the deadline before calling).
template <bool ANY, bool TWO_LEVEL, bool COUNT, uint32_t CV>
__device__ __forceinline__ void trace_ray(const TraceArgs &a, uint32_t tid, bool active, Counts &cnt,
		StackTop top = StackTop{nullptr, 0}) {
	constexpr bool MM3 = (CV & kVarMinMax3) != 0;
	constexpr int SMEM = smem_stack_depth(CV);
	constexpr bool MOTION = (CV & kVarMotion) != 0;
	constexpr bool N4 = (CV & kVarNodes4) != 0;
	if (!active) return;
	const uint32_t i = a.order ? a.order[tid] : tid;  // the ray this thread traces
	const bool keep = (a.variant & kVarSceneEvictLast) != 0;
	const bool stream = (a.variant & kVarStreamRays) != 0;
	const uint64_t pol = keep ? evict_last_policy() : 0ull;
	TravState s;
	TravStack stack;
	const int k = ray_begin(a, i, stream, s);
	if (k == kRayMasked) return;
	if (k == kRayTraverse) {
		while (!ray_step<ANY, TWO_LEVEL, COUNT, MM3, SMEM, MOTION, N4>(a, s, stack, keep, pol, cnt, top)) {
		}
		if (s.sp < 0) return;  // abandoned
	}
	ray_write(a, i, s, stream);
	if (COUNT) cnt.rays += 1;
}

// Two-level builds: at most 896 threads per block leaves 72 registers a
// thread (no spills; instanced any hit +3 %); blocks are at most 512.
template <bool ANY, bool TWO_LEVEL, bool COUNT, uint32_t CV>
__global__ void __launch_bounds__((CV & kVarOccupancy) ? 64 : (TWO_LEVEL ? 896 : 1024), (CV & kVarOccupancy) ? 20 : 0)
k_trace(TraceArgs a) {
	extern __shared__ uint2 s_stack_top[];  // smem_stack_depth(CV) entries per thread, else empty
	const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
	// this thread's ray is on its way into L1 while thread 0 looks up the
	// launch's start: the block waits for the two at once
	if (tid < a.count) {
		const char *rp = static_cast<const char *>(a.rays) + 48 * (size_t)(a.order ? a.order[tid] : tid);
		asm volatile("prefetch.global.L1 [%0];" ::"l"(rp));
		asm volatile("prefetch.global.L1 [%0];" ::"l"(rp + 47));
	}
	if (threadIdx.x == 0) {
		const uint32_t start = slot_start(g_queue[a.launch_id % kQueueSlots], blockIdx.x == 0);
		s_block_late = past_deadline(start, a.deadline_ticks) ? 1u : 0u;
		if (s_block_late) atomicOr(a.status, kStatusDeadline);
	}
	__syncthreads();
	if (s_block_late) return;  // started after the deadline: none of the block's rays
	if (!COUNT && tid >= a.count) return;
	Counts cnt{0, 0, 0, 0};
	trace_ray<ANY, TWO_LEVEL, COUNT, CV>(a, tid, tid < a.count, cnt, StackTop{s_stack_top + threadIdx.x, blockDim.x});
	if (COUNT) {
		// every lane of the block reaches this point in the counting variant
		unsigned long long v[4] = {cnt.nodes, cnt.tris, cnt.insts, cnt.rays};
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			unsigned long long x = v[k];
#pragma unroll
			for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
			v[k] = x;
		}
		if ((threadIdx.x & 31) == 0) {
#pragma unroll
			for (int k = 0; k < 4; ++k) atomicAdd(&a.counters[k], v[k]);
		}
	}
	// the launch start is cleared after the launch (k_clear_launch_start)
}

// Zeroes the launch start of a one-ray-per-thread launch after it, on its
// stream, so its counter slot is all zero again for the slot's next user.
__global__ void k_clear_launch_start(uint32_t slot_index) {
	g_queue[slot_index][kSlotStart] = 0u;
}

uint32_t next_launch_id() {
	static std::atomic<uint32_t> next{0};
	return next.fetch_add(1u);
}

// Closest-hit order of two hits as ray_step's acceptance keeps them: the
// smaller t, and at an exact tie the lower (meshIndex, triangleIndex).  A
// ray with no hit yet holds (maxt, kNull, kNull); every hit ray_step accepts
// orders below it, and a hit at t == maxt is never accepted.  The order does
// not depend on the order the hits were found in, so parts of one ray's walk
// can run on different lanes and their best hits merge to the same answer.
__device__ __forceinline__ bool hit_key_less(float t, uint32_t mesh, uint32_t tri, float bt, uint32_t bmesh,
		uint32_t btri) {
	return t < bt || (t == bt && (mesh < bmesh || (mesh == bmesh && tri < btri)));
}

// Drain split (persistent fetch, closest hit), once the launch's rays
// are all claimed.  A warp's last rays would otherwise finish one node fetch
// at a time on a few lanes while the rest idle; here lanes with nothing to do
// take subtrees of them:
// - a helper pulls its owner's best hit when that orders below its own, so
//   it culls with every hit the ray has found so far;
// - the k-th free lane (lane order) pairs with the k-th working lane that has
//   stack entries; that lane pops its top entry (a node group, or a deferred
//   triangle group) and the free lane starts a walk of it with a copy of the
//   ray and of its best hit (so ties keep their order), as a helper of the
//   ray's owner -- the owner of the donor, when the donor is itself a helper.
//   The copy includes b1 and b2: a helper's best may be a hit its owner has
//   not seen yet, and the taker may hand it over first;
// - each owner adds its new helpers' lanes to `link` (a helper's `link` is
//   its owner's lane).
// Two-level scenes: a lane inside an instance's BLAS gives only entries of
// that BLAS (above its `inst_sp`), with the instance-space ray and the
// instance's object, and its taker walks them as a BLAS of its own (inst_sp
// 0: its walk ends where that BLAS is exhausted); a lane at top level gives
// TLAS entries with the world ray.  Either way the world ray and the ray's
// time go along, for the instances a TLAS walk enters.
// Every lane runs every ballot, shuffle and match here (the branches around
// them are warp-uniform).  A donated entry is walked exactly once, by its
// taker.  The pieces may visit nodes the one-lane walk would have culled (a
// helper learns of its owner's hits a trip late), but a lane culls only with
// the t of a hit the ray has, so no piece skips the triangle of the ray's
// best hit, and the merged answer is the one-lane answer.
template <int SMEM, bool TWO_LEVEL>
__device__ __forceinline__ void split_drain(TravState &s, TravStack &stack, StackTop top, uint32_t lane, uint32_t rid,
		bool &helper, bool waiting, uint32_t &link) {
	constexpr uint32_t kAll = 0xffffffffu;
	if (__any_sync(kAll, helper)) {
		const uint32_t src = helper ? link : lane;
		const float t = __shfl_sync(kAll, s.best_t, src);
		const float b1 = __shfl_sync(kAll, s.best_b1, src);
		const float b2 = __shfl_sync(kAll, s.best_b2, src);
		const uint32_t mesh = __shfl_sync(kAll, s.best_mesh, src);
		const uint32_t tri = __shfl_sync(kAll, s.best_tri, src);
		if (helper && hit_key_less(t, mesh, tri, s.best_t, s.best_mesh, s.best_tri)) {
			s.best_t = t;
			s.best_b1 = b1;
			s.best_b2 = b2;
			s.best_mesh = mesh;
			s.best_tri = tri;
		}
	}
	const bool isfree = rid == kNull && !helper;
	const uint32_t freem = __ballot_sync(kAll, isfree);
	if (freem == 0u) return;
	const bool working = (rid != kNull && !waiting) || helper;
	const uint32_t donors = __ballot_sync(kAll, working && s.sp > (TWO_LEVEL ? max(s.inst_sp, 0) : 0));
	if (donors == 0u) return;
	const uint32_t n = min(__popc(freem), __popc(donors));
	const uint32_t below = (1u << lane) - 1u;
	const uint32_t kf = __popc(freem & below);
	const bool take = isfree && kf < n;
	const bool give = ((donors >> lane) & 1u) && __popc(donors & below) < n;
	uint32_t src = lane;
	if (take) {
		uint32_t m = donors;  // the kf-th donor: drop the kf lowest set bits
		for (uint32_t j = 0; j < kf; ++j) m &= m - 1u;
		src = __ffs(m) - 1;
	}
	uint2 e = make_uint2(0u, 0u);
	if (give) e = stack_get<SMEM>(stack, top, --s.sp);
	e.x = __shfl_sync(kAll, e.x, src);
	e.y = __shfl_sync(kAll, e.y, src);
	const uint32_t root = __shfl_sync(kAll, helper ? link : lane, src);
	// the donor's ray and best hit (a lane that takes nothing reads its own)
	s.ray.o.x = __shfl_sync(kAll, s.ray.o.x, src);
	s.ray.o.y = __shfl_sync(kAll, s.ray.o.y, src);
	s.ray.o.z = __shfl_sync(kAll, s.ray.o.z, src);
	s.ray.d.x = __shfl_sync(kAll, s.ray.d.x, src);
	s.ray.d.y = __shfl_sync(kAll, s.ray.d.y, src);
	s.ray.d.z = __shfl_sync(kAll, s.ray.d.z, src);
	s.ray.idir.x = __shfl_sync(kAll, s.ray.idir.x, src);
	s.ray.idir.y = __shfl_sync(kAll, s.ray.idir.y, src);
	s.ray.idir.z = __shfl_sync(kAll, s.ray.idir.z, src);
	s.ray.oct = __shfl_sync(kAll, s.ray.oct, src);
	s.mint = __shfl_sync(kAll, s.mint, src);
	s.best_t = __shfl_sync(kAll, s.best_t, src);
	s.best_b1 = __shfl_sync(kAll, s.best_b1, src);
	s.best_b2 = __shfl_sync(kAll, s.best_b2, src);
	s.best_mesh = __shfl_sync(kAll, s.best_mesh, src);
	s.best_tri = __shfl_sync(kAll, s.best_tri, src);
	bool blas = false;
	if (TWO_LEVEL) {
		s.wo.x = __shfl_sync(kAll, s.wo.x, src);
		s.wo.y = __shfl_sync(kAll, s.wo.y, src);
		s.wo.z = __shfl_sync(kAll, s.wo.z, src);
		s.wd.x = __shfl_sync(kAll, s.wd.x, src);
		s.wd.y = __shfl_sync(kAll, s.wd.y, src);
		s.wd.z = __shfl_sync(kAll, s.wd.z, src);
		s.time = __shfl_sync(kAll, s.time, src);
		s.inst_obj = __shfl_sync(kAll, s.inst_obj, src);
		blas = __shfl_sync(kAll, s.inst_sp >= 0 ? 1u : 0u, src) != 0u;
	}
	if (take) {
		s.ng = e;
		s.tg = make_uint2(0u, 0u);
		s.sp = 0;
		s.visits = 0;
		if (TWO_LEVEL) s.inst_sp = blas ? 0 : -1;  // (inst_obj: the donor's, kNull at top level)
		helper = true;
		link = root;
	}
	// an owner's group: itself and the lanes that just became its helpers
	const uint32_t grp = __match_any_sync(kAll, take ? root : lane);
	if (rid != kNull) link |= grp & ~(1u << lane);
}

// ---------------------------------------------------------------------------
// Persistent single-batch kernel with warp-level ray fetch (after Aila and
// Laine 2009, "dynamic fetch"): resident warps loop until the batch's ray
// counter runs out.  Each trip a warp ballots its idle lanes; once at least
// `refill` are idle (or all are), the lowest idle lane claims that many rays
// with one atomicAdd and __shfl_sync hands each idle lane its index, so a
// warp keeps its lanes busy instead of idling behind its longest ray.  Then
// every busy lane runs one ray_step.
//
// Termination: a trip either advances some lane's ray (each ray finishes in
// a bounded number of trips, see ray_step) or, with every lane idle, claims
// 32 rays from the counter or leaves -- the counter only grows, so the
// claims run out.  Every ballot/shuffle is executed by all 32 lanes: the
// block is a whole number of warps, no lane leaves the loop alone (the exit
// test is warp-uniform), and `refill` is in [1, 32].
// Deadline: the claiming lane reads the timer; once the launch's deadline
// has passed, the warp still claims rays (so the counter runs out as
// before) but starts none of them -- their hits are not written and the
// status word records it -- while rays already started finish their walks.
// Drain loop (split builds), after the counter is spent: no rays are
// claimed any more, and each trip steps every lane that holds a walk (its
// own ray or a helper's subtree).  A walk finishes in a bounded number of
// trips, a donation moves a stack entry to a lane that then walks it, so the
// entries to walk only shrink; an owner whose walk is done waits only for
// its helpers' walks, each of which ends and clears its bit.  The loop ends
// when no lane holds a walk (a warp-uniform ballot), and every shuffle,
// ballot and match in it is executed by all 32 lanes.
// ---------------------------------------------------------------------------

// Two-level builds carry the world ray and instance state on top of the
// flat ones: 72 registers (7 blocks of 128 per SM) keep them from spilling,
// which is faster than 64 with spills (instanced closest hit +5.6 %).
template <bool ANY, bool TWO_LEVEL, uint32_t CV>
__global__ void __launch_bounds__(kTraceBlock, TWO_LEVEL ? 7 : 8) k_trace_fetch(TraceArgs a, uint32_t refill) {
	constexpr bool MM3 = (CV & kVarMinMax3) != 0;
	constexpr int SMEM = smem_stack_depth(CV);
	constexpr bool MOTION = (CV & kVarMotion) != 0;
	constexpr bool N4 = (CV & kVarNodes4) != 0;
	constexpr bool SPLIT = !ANY && (CV & kVarDrainSplit) != 0;
	extern __shared__ uint2 s_stack_top[];  // SMEM entries per thread with a shared-memory stack, else empty
	const StackTop top{s_stack_top + threadIdx.x, blockDim.x};
	uint32_t *slot = g_queue[a.launch_id % kQueueSlots];
	note_block_start();
	const bool keep = (a.variant & kVarSceneEvictLast) != 0;
	const bool stream = (a.variant & kVarStreamRays) != 0;
	const uint64_t pol = keep ? evict_last_policy() : 0ull;
	const uint32_t lane = threadIdx.x & 31u;
	TravState s;
	TravStack stack;
	Counts cnt{0, 0, 0, 0};
	uint32_t rid = kNull;  // ray this lane owns (kNull: none)
	bool drained = false;  // warp-uniform: the counter has passed the batch
	const uint32_t count = a.count_dev ? min(*a.count_dev, a.count) : a.count;  // rays to claim
	for (;;) {
		const uint32_t idle = __ballot_sync(0xffffffffu, rid == kNull);
		const uint32_t nidle = __popc(idle);
		if (!drained && nidle >= refill) {
			const uint32_t leader = __ffs(idle) - 1;
			uint32_t base = 0;
			if (lane == leader) {
				base = claim_deadline(atomicAdd(&slot[0], nidle), nidle, &slot[0], s_launch_start, a.deadline_ticks);
				if ((base & kClaimLate) && (base & ~kClaimLate) < count) atomicOr(a.status, kStatusDeadline);
			}
			base = __shfl_sync(0xffffffffu, base, leader);
			const bool late = (base & kClaimLate) != 0u;
			base &= ~kClaimLate;
			drained = base + nidle >= count;
			if (rid == kNull && !late) {
				const uint32_t idx = base + __popc(idle & ((1u << lane) - 1u));
				if (idx < count) {
					const uint32_t i = a.order ? a.order[idx] : idx;
					const int k = ray_begin(a, i, stream, s);
					if (k == kRayTraverse) rid = i;
					else if (k == kRayAnswered) ray_write(a, i, s, stream);
				}
			}
		}
		const uint32_t busy = __ballot_sync(0xffffffffu, rid != kNull);
		if (busy == 0u) {
			if (drained) break;
			continue;  // every lane idle: the next trip claims 32 rays
		}
		if (SPLIT && drained) break;  // the warp's last rays: the drain loop below
		const bool sparse = drained && __popc(busy) < a.postpone;  // warp-uniform
		if (rid != kNull &&
				ray_step<ANY, TWO_LEVEL, false, MM3, SMEM, MOTION, N4>(a, s, stack, keep, pol, cnt, top, sparse)) {
			if (s.sp >= 0) ray_write(a, rid, s, stream);  // an abandoned ray writes nothing
			rid = kNull;
		}
	}
	if (SPLIT) {
		// Drain loop (the counter is spent): lanes without a ray help the
		// warp's remaining rays (split_drain).  A helper lane walks a subtree
		// of the ray that lane `link` owns; an owner keeps its helpers' lanes
		// in `link`, and once its own walk is done it waits (`waiting`) for
		// them before writing; `lost`: some part of its walk was abandoned,
		// so it writes nothing.  Ends when no lane holds a ray or a subtree.
		bool helper = false, waiting = false, lost = false;
		uint32_t link = 0u;
		for (;;) {
			split_drain<SMEM, TWO_LEVEL>(s, stack, top, lane, rid, helper, waiting, link);
			const uint32_t busy = __ballot_sync(0xffffffffu, rid != kNull || helper);
			if (busy == 0u) break;
			const bool sparse = __popc(busy) < a.postpone;  // warp-uniform
			const bool fin = ((rid != kNull && !waiting) || helper) &&
					ray_step<ANY, TWO_LEVEL, false, MM3, SMEM, MOTION, N4>(a, s, stack, keep, pol, cnt, top, sparse);
			// helpers done this trip hand their best hit to their owners, one at a time
			for (uint32_t hf = __ballot_sync(0xffffffffu, helper && fin); hf; hf &= hf - 1u) {
				const uint32_t h = __ffs(hf) - 1;
				const float t = __shfl_sync(0xffffffffu, s.best_t, h);
				const float b1 = __shfl_sync(0xffffffffu, s.best_b1, h);
				const float b2 = __shfl_sync(0xffffffffu, s.best_b2, h);
				const uint32_t mesh = __shfl_sync(0xffffffffu, s.best_mesh, h);
				const uint32_t tri = __shfl_sync(0xffffffffu, s.best_tri, h);
				const uint32_t own = __shfl_sync(0xffffffffu, link, h);
				const bool hl = __shfl_sync(0xffffffffu, s.sp < 0 ? 1u : 0u, h) != 0u;
				if (lane == own) {
					link &= ~(1u << h);
					lost |= hl;
					if (hit_key_less(t, mesh, tri, s.best_t, s.best_mesh, s.best_tri)) {
						s.best_t = t;
						s.best_b1 = b1;
						s.best_b2 = b2;
						s.best_mesh = mesh;
						s.best_tri = tri;
					}
				}
			}
			if (helper) {
				if (fin) {
					helper = false;
					link = 0u;
				}
			} else if (rid != kNull) {
				if (fin) {
					waiting = true;
					lost |= s.sp < 0;
				}
				if (waiting && link == 0u) {
					if (!lost) ray_write(a, rid, s, stream);  // an abandoned ray writes nothing
					rid = kNull;
					waiting = lost = false;
				}
			}
		}
	}
	__syncthreads();
	release_slot(slot);
}

// ---------------------------------------------------------------------------
// Multi-batch queue kernel: one launch drains many ray batches (any mix of
// scenes and modes).  Persistent 64-thread blocks claim 64-ray tiles from a
// device work queue -- a counter in a slot of g_queue -- and trace them; the
// last block to leave resets the slot for its next use.  Every loop trip and
// barrier is block-uniform (the tile index is broadcast through shared
// memory), and the loop ends when the tiles run out.
// ---------------------------------------------------------------------------

__device__ __forceinline__ TraceArgs batch_args(const QueueParams &p, const QueueBatch &qb) {
	TraceArgs a{};
	a.order = qb.order_begin != kNull ? p.order + qb.order_begin : nullptr;
	a.nodes = qb.nodes;
	a.tris = qb.tris;
	a.insts = qb.insts;
	a.root = qb.root;
	a.two_level = (qb.flags >> 1) & 1u;
	a.rays = qb.rays;
	a.hits = qb.hits;
	a.count = qb.count;
	a.any_hit = qb.flags & 1u;
	a.status = qb.status;
	a.postpone = (qb.flags >> 8) & 0xffu;
	a.variant = (qb.flags >> 16) & 0xffu;
	a.visit_limit = qb.visit_limit;
	const uint32_t f = (qb.flags >> 24) & 31u;
	a.blas_visits = f ? 1u << f : 0u;
	a.deadline_ticks = p.deadline_ticks;
	a.launch_id = p.launch_id;
	return a;
}

template <uint32_t CV>
__global__ void __launch_bounds__(kTileRays, 12) k_trace_queue(const __grid_constant__ QueueParams p) {
	__shared__ uint32_t s_tile;
	uint32_t *slot = g_queue[p.slot];
	note_block_start();
	Counts cnt{0, 0, 0, 0};
	for (;;) {
		if (threadIdx.x == 0) {
			s_tile = atomicAdd(&slot[0], 1u);
			s_block_late = past_deadline(s_launch_start, p.deadline_ticks) ? 1u : 0u;
		}
		__syncthreads();
		const uint32_t tile = s_tile;
		const bool late = s_block_late != 0u;
		__syncthreads();
		if (tile >= p.total_tiles) break;
		uint32_t lo = 0, hi = p.n;  // last batch whose first tile is <= tile
		while (hi - lo > 1) {
			const uint32_t mid = (lo + hi) >> 1;
			if (p.b[mid].tile_begin <= tile) lo = mid;
			else hi = mid;
		}
		const QueueBatch &qb = p.b[lo];
		const TraceArgs a = batch_args(p, qb);
		const uint32_t tid = (tile - qb.tile_begin) * kTileRays + threadIdx.x;
		const bool active = tid < a.count && !late;  // past the deadline: the tile's rays are not started
		if (late && threadIdx.x == 0) atomicOr(a.status, kStatusDeadline);
		if (a.any_hit) {
			if (a.two_level) trace_ray<true, true, false, CV>(a, tid, active, cnt);
			else trace_ray<true, false, false, CV>(a, tid, active, cnt);
		} else {
			if (a.two_level) trace_ray<false, true, false, CV>(a, tid, active, cnt);
			else trace_ray<false, false, false, CV>(a, tid, active, cnt);
		}
		if (p.done_flags) {
			// completion notice per batch: every thread's hits are fenced, then
			// the block that finishes the batch's last tile raises its flag
			__threadfence_system();
			__syncthreads();
			if (threadIdx.x == 0) {
				const uint32_t ntiles = (qb.count + kTileRays - 1) / kTileRays;
				if (atomicAdd(&p.tiles_done[qb.user_index], 1u) + 1u == ntiles) {
					__threadfence_system();
					*reinterpret_cast<volatile uint32_t *>(&p.done_flags[qb.user_index]) = 1u;
				}
			}
		}
	}
	release_slot(slot);
}

// Adds n finished rays to batch bi's progress counter; the add that brings
// the batch to its count raises the batch's completion flag.  The hits the
// count covers were ordered before this thread's fence by a warp sync.
__device__ __forceinline__ void add_done(const QueueParams &p, uint32_t bi, uint32_t n) {
	const QueueBatch &qb = p.b[bi];
	__threadfence();
	if (atomicAdd(&p.tiles_done[qb.user_index], n) + n == qb.count) {
		__threadfence_system();
		*reinterpret_cast<volatile uint32_t *>(&p.done_flags[qb.user_index]) = 1u;
	}
}

// Warp-wide (every lane): orders all lanes' hit writes before lane 0 adds
// the warp's pending count of finished rays.
__device__ __forceinline__ void flush_done(const QueueParams &p, uint32_t bi, uint32_t n, uint32_t lane) {
	__syncwarp();
	if (n && lane == 0) add_done(p, bi, n);
}

// Index of the batch holding global ray g among batches [lo, hi) (the last
// one with ray_begin <= g).
__device__ __forceinline__ uint32_t batch_of_ray(const QueueParams &p, uint32_t g, uint32_t lo, uint32_t hi) {
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (p.b[mid].ray_begin <= g) lo = mid;
		else hi = mid;
	}
	return lo;
}

// One ray class of a queue launch -- batches [class_batch[c], class_batch[c+1]),
// all of one mode and one scene kind -- drained by persistent warps with
// warp-level ray fetch from the class's own counter, exactly as k_trace_fetch
// drains one batch; lanes of a warp may hold rays of different batches
// (scenes) of the class.  Completion flags count finished rays per batch: a
// warp keeps a pending count while its finishing lanes stay in one batch and
// adds it to the batch's counter (after a warp sync and a fence that order
// the hits before it) every 16 trips, when the batch changes and at the end;
// a trip whose finishing lanes span batches adds per batch group
// (__match_any_sync).  The add that brings a batch to its count raises the
// batch's flag.  Termination as k_trace_fetch: each trip steps a busy lane or
// claims rays, and the counter only grows.  Past the launch's deadline a
// warp's claims start no rays; each claimed ray then counts as finished
// (so every batch's flag is still raised) with its hit not written and its
// scene's status word recording the deadline.
template <bool ANY, bool TWO_LEVEL, bool MM3, bool FLAGS>
__device__ __forceinline__ void drain_class(const QueueParams &p, uint32_t c, uint32_t *counter, uint32_t lane,
		TravState &s, TravStack &stack) {
	const uint32_t cb = p.class_batch[c], ce = p.class_batch[c + 1];
	if (cb == ce) return;
	const uint32_t r0 = p.b[cb].ray_begin;
	const uint32_t nrays = (ce == p.n ? p.total_rays : p.b[ce].ray_begin) - r0;
	Counts cnt{0, 0, 0, 0};
	uint32_t rid = kNull;  // ray (index within its batch) this lane traces; kNull: idle
	uint32_t bi = cb;      // its batch
	bool drained = false;  // warp-uniform
	uint32_t pend_bi = 0, pend_n = 0, trip = 0;  // warp-uniform: finished rays not yet counted
	for (;;) {
		bool fin = false;  // this lane completed a ray in this trip
		const uint32_t idle = __ballot_sync(0xffffffffu, rid == kNull);
		const uint32_t nidle = __popc(idle);
		if (!drained && nidle >= p.refill) {
			const uint32_t leader = __ffs(idle) - 1;
			uint32_t base = 0;
			if (lane == leader) {
				base = atomicAdd(counter, nidle);
				if (!(base & kClaimLate) && (base & (kDeadlineCheckRays - 1u)) < nidle)
					base = claim_deadline(base, nidle, counter, slot_start(counter - c, base == 0u), p.deadline_ticks);
			}
			base = __shfl_sync(0xffffffffu, base, leader);
			const bool late = (base & kClaimLate) != 0u;
			base &= ~kClaimLate;
			drained = base + nidle >= nrays;
			if (rid == kNull) {
				const uint32_t g = base + __popc(idle & ((1u << lane) - 1u));
				if (g < nrays) {
					bi = batch_of_ray(p, r0 + g, cb, ce);
					if (late) {
						atomicOr(p.b[bi].status, kStatusDeadline);
						fin = true;
					} else {
						const TraceArgs a = batch_args(p, p.b[bi]);
						const uint32_t local = r0 + g - p.b[bi].ray_begin;
						const uint32_t i = a.order ? a.order[local] : local;  // the ray (sorted batches: permuted)
						const bool stream = (a.variant & kVarStreamRays) != 0;
						const int k = ray_begin(a, i, stream, s);
						if (k == kRayTraverse) {
							rid = i;
						} else {
							if (k == kRayAnswered) ray_write(a, i, s, stream);
							fin = true;
						}
					}
				}
			}
		}
		if (rid != kNull) {
			const TraceArgs a = batch_args(p, p.b[bi]);
			const bool keep = (a.variant & kVarSceneEvictLast) != 0;
			const uint64_t pol = keep ? evict_last_policy() : 0ull;
			if (ray_step<ANY, TWO_LEVEL, false, MM3>(a, s, stack, keep, pol, cnt)) {
				if (s.sp >= 0) ray_write(a, rid, s, (a.variant & kVarStreamRays) != 0);  // abandoned: no hit
				rid = kNull;
				fin = true;
			}
		}
		if (FLAGS) {
			const uint32_t fm = __ballot_sync(0xffffffffu, fin);
			bool flush = pend_n != 0 && ((++trip & 15u) == 0u);
			if (fm) {
				const uint32_t b0 = __shfl_sync(0xffffffffu, bi, __ffs(fm) - 1);
				const bool one = __all_sync(0xffffffffu, !fin || bi == b0);
				if (one && (pend_n == 0 || pend_bi == b0)) {
					pend_bi = b0;
					pend_n += __popc(fm);
				} else {
					flush_done(p, pend_bi, pend_n, lane);  // what was pending, then this trip's groups
					pend_n = 0;
					flush = false;
					if (one) {
						pend_bi = b0;
						pend_n = __popc(fm);
					} else if (fin) {
						const uint32_t peers = __match_any_sync(fm, bi);
						if (lane == __ffs(peers) - 1u) add_done(p, bi, __popc(peers));
					}
				}
			}
			const bool leaving = drained && __ballot_sync(0xffffffffu, rid != kNull) == 0u;
			if (flush || (leaving && pend_n)) {
				flush_done(p, pend_bi, pend_n, lane);
				pend_n = 0;
			}
			if (leaving) break;
			continue;
		}
		if (drained && __ballot_sync(0xffffffffu, rid != kNull) == 0u) break;
	}
}

// Multi-batch queue kernel with warp-level ray fetch: every warp drains the
// launch's four ray classes in turn (closest flat, closest two-level, any
// flat, any two-level), each with a loop specialised for its class; warps
// that find a class drained move on while others finish its last rays.
// FLAGS: the launch keeps completion flags (a separate build, so launches
// without them carry none of that state).
// TWO: the launch holds two-level batches (classes 1 and 3).  A launch of
// flat batches only takes the build without those loops, at 64 registers
// (8 blocks of 128 per SM) instead of 72.
template <uint32_t CV, bool FLAGS, bool TWO>
__global__ void __launch_bounds__(kTraceBlock, TWO ? 7 : 8) k_trace_queue_fetch(const __grid_constant__ QueueParams p) {
	constexpr bool MM3 = (CV & kVarMinMax3) != 0;
	uint32_t *slot = g_queue[p.slot];
	const uint32_t lane = threadIdx.x & 31u;
	TravState s;
	TravStack stack;
	drain_class<false, false, MM3, FLAGS>(p, 0, &slot[0], lane, s, stack);
	if (TWO) drain_class<false, true, MM3, FLAGS>(p, 1, &slot[1], lane, s, stack);
	drain_class<true, false, MM3, FLAGS>(p, 2, &slot[2], lane, s, stack);
	if (TWO) drain_class<true, true, MM3, FLAGS>(p, 3, &slot[3], lane, s, stack);
	__syncthreads();
	release_slot(slot);
}

__global__ void k_set_flag(uint32_t *flag) {
	__threadfence_system();
	*reinterpret_cast<volatile uint32_t *>(flag) = 1u;
}

lrx_status launch_set_flag(uint32_t *flag, cudaStream_t st) {
	k_set_flag<<<1, 1, 0, st>>>(flag);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

// hits[i] = src[i] for every masked ray i (src: the caller's host buffer,
// mapped); unmasked slots are left alone.
__global__ void k_restore_masked_hits(const float4 *__restrict__ rays, uint32_t n, const uint32_t *src,
		uint32_t *hits) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const uint32_t flags = __float_as_uint(__ldcs(rays + 3 * (size_t)i + 2).y);
	if (!(flags & LRX_RAY_FLAGS_MASKED)) return;
#pragma unroll
	for (int w = 0; w < 5; ++w) hits[5 * (size_t)i + w] = src[5 * (size_t)i + w];
}

lrx_status launch_restore_masked_hits(const void *d_rays, uint32_t n, const void *src, void *d_hits, cudaStream_t st) {
	if (n == 0) return LRX_OK;
	k_restore_masked_hits<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float4 *>(d_rays), n,
			static_cast<const uint32_t *>(src), static_cast<uint32_t *>(d_hits));
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

// Blocks of one kernel and block size resident on a device at once, per
// device, computed on first use.  Threads that race on a first use compute
// the same value; the relaxed atomics keep the cache free of data races.
constexpr int kMaxCachedDevices = 64;
struct ResidentCache {
	std::atomic<int> blocks[kMaxCachedDevices];
};

static lrx_status resident_blocks(ResidentCache &c, const void *fn, int block, size_t smem, int *out) {
	int dev = 0;
	LRX_CUDA(cudaGetDevice(&dev));
	const bool cached = dev >= 0 && dev < kMaxCachedDevices;
	if (cached) {
		const int v = c.blocks[dev].load(std::memory_order_relaxed);
		if (v > 0) {
			*out = v;
			return LRX_OK;
		}
	}
	int sms = 0, per_sm = 0;
	LRX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	LRX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem));
	const int v = std::max(1, sms * std::max(1, per_sm));
	if (cached) c.blocks[dev].store(v, std::memory_order_relaxed);
	*out = v;
	return LRX_OK;
}

lrx_status launch_trace_queue(const QueueParams &p, cudaStream_t st) {
	if (p.total_tiles == 0) return LRX_OK;
	if (p.fetch) {
		// 128-thread blocks resident per device, by [flags][two-level]
		static ResidentCache fetch_cache[2][2];
		const int fl = p.done_flags ? 1 : 0;
		const int two = (p.class_batch[1] != p.class_batch[2] || p.class_batch[3] != p.class_batch[4]) ? 1 : 0;
		const void *fn = fl ? (two ? (const void *)k_trace_queue_fetch<0u, true, true>
								 : (const void *)k_trace_queue_fetch<0u, true, false>)
						: (two ? (const void *)k_trace_queue_fetch<0u, false, true>
							   : (const void *)k_trace_queue_fetch<0u, false, false>);
		int resident = 0;
		lrx_status rc = resident_blocks(fetch_cache[fl][two], fn, kTraceBlock, 0, &resident);
		if (rc != LRX_OK) return rc;
		if (p.total_rays == 0 || p.refill < 1 || p.refill > 32) {
			set_error("queue fetch launch: empty or bad refill");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		const uint32_t grid = (uint32_t)std::min<uint64_t>(((uint64_t)p.total_rays + kTraceBlock - 1) / kTraceBlock,
				(uint64_t)resident);
		if (fl) {
			if (two) k_trace_queue_fetch<0u, true, true><<<grid, kTraceBlock, 0, st>>>(p);
			else k_trace_queue_fetch<0u, true, false><<<grid, kTraceBlock, 0, st>>>(p);
		} else {
			if (two) k_trace_queue_fetch<0u, false, true><<<grid, kTraceBlock, 0, st>>>(p);
			else k_trace_queue_fetch<0u, false, false><<<grid, kTraceBlock, 0, st>>>(p);
		}
		LRX_CUDA(cudaGetLastError());
		return LRX_OK;
	}
	static ResidentCache tile_cache;  // 64-thread blocks of the tile kernel
	int resident = 0;
	lrx_status rc = resident_blocks(tile_cache, (const void *)k_trace_queue<0u>, kTileRays, 0, &resident);
	if (rc != LRX_OK) return rc;
	const uint32_t grid = std::min<uint32_t>(p.total_tiles, (uint32_t)resident);
	k_trace_queue<0u><<<grid, kTileRays, 0, st>>>(p);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

// Persistent fetch launch: as many blocks as fit on the device at once (at
// most one ray per thread), all sharing one counter slot.
template <bool ANY, bool TWO_LEVEL, uint32_t CV>
static lrx_status launch_fetch(const TraceArgs &a, uint32_t bs, cudaStream_t st) {
	const size_t smem_bytes = sizeof(uint2) * smem_stack_depth(CV) * bs;
	static ResidentCache cache[kTraceBlock / 32];  // by block size 32, 64, 96, 128
	int resident = 0;
	const lrx_status rc = resident_blocks(cache[bs / 32 - 1], (const void *)k_trace_fetch<ANY, TWO_LEVEL, CV>, (int)bs,
			smem_bytes, &resident);
	if (rc != LRX_OK) return rc;
	const uint32_t grid = (uint32_t)std::min<uint64_t>(((uint64_t)a.count + bs - 1) / bs, (uint64_t)resident);
	const uint32_t refill = a.refill == 0 ? 16u : std::min(32u, a.refill);
	k_trace_fetch<ANY, TWO_LEVEL, CV><<<grid, bs, smem_bytes, st>>>(a, refill);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

lrx_status launch_trace(const TraceArgs &a_in, cudaStream_t st) {
	if (a_in.count == 0) return LRX_OK;
	TraceArgs a = a_in;
	a.launch_id = next_launch_id();  // its counter slot (persistent) or launch-start word
	uint32_t bs = a.block_size ? a.block_size : kTraceBlock;
	if (bs < 32 || bs > 512 || (bs & 31)) {
		set_error("trace block size must be a multiple of 32 in [32, 512]");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	const uint32_t grid = (a.count + bs - 1) / bs;
	const bool cnt = a.counters != nullptr;
	if (a.motion && a.two_level) {
		// motion scenes: builds of their own (no MINMAX3 / SMEM_STACK / occupancy
		// forms), so the static builds carry no motion code
		// (no drain split: its motion build spills, and closest hit lost 1-2 %)
		if ((a.variant & kVarPersistent) && !cnt && a.count <= kMaxFetchRays) {
			const uint32_t fbs = std::min(bs, kTraceBlock);
			return a.any_hit ? launch_fetch<true, true, kVarMotion>(a, fbs, st)
					: launch_fetch<false, true, kVarMotion>(a, fbs, st);
		}
		if (a.any_hit) {
			if (cnt) k_trace<true, true, true, kVarMotion><<<grid, bs, 0, st>>>(a);
			else k_trace<true, true, false, kVarMotion><<<grid, bs, 0, st>>>(a);
		} else {
			if (cnt) k_trace<false, true, true, kVarMotion><<<grid, bs, 0, st>>>(a);
			else k_trace<false, true, false, kVarMotion><<<grid, bs, 0, st>>>(a);
		}
		LRX_CUDA(cudaGetLastError());
		k_clear_launch_start<<<1, 1, 0, st>>>(a.launch_id % kQueueSlots);
		LRX_CUDA(cudaGetLastError());
		return LRX_OK;
	}
	if ((a.variant & kVarPersistent) && !cnt && a.count <= kMaxFetchRays) {
		// persistent warps with ray fetch; block size capped at kTraceBlock
		const uint32_t fbs = std::min(bs, kTraceBlock);
		const bool mm3 = (a.variant & kVarMinMax3) != 0;
		const uint32_t smem = smem_stack_bits(a.variant);
#define LRX_FETCH(A, T, N)                                                                                \
	(smem == kVarSmemStack32 ? launch_fetch<A, T, kVarSmemStack32 | N>(a, fbs, st)                          \
	 : smem == kVarSmemStack16 ? launch_fetch<A, T, kVarSmemStack16 | N>(a, fbs, st)                        \
	 : smem ? launch_fetch<A, T, kVarSmemStack | N>(a, fbs, st)                                             \
		  : (mm3 ? launch_fetch<A, T, kVarMinMax3 | N>(a, fbs, st) : launch_fetch<A, T, N>(a, fbs, st)))
		// the drain split's builds: closest hit, local-memory stack, 2-input min/max
		const bool split = (a.variant & kVarDrainSplit) && !a.any_hit;
		if (split) return a.nodes4 ? launch_fetch<false, false, kVarDrainSplit | kVarNodes4>(a, fbs, st)
						   : a.two_level ? launch_fetch<false, true, kVarDrainSplit>(a, fbs, st)
										 : launch_fetch<false, false, kVarDrainSplit>(a, fbs, st);
		if (a.nodes4) return a.any_hit ? LRX_FETCH(true, false, kVarNodes4) : LRX_FETCH(false, false, kVarNodes4);
		if (a.any_hit) return a.two_level ? LRX_FETCH(true, true, 0u) : LRX_FETCH(true, false, 0u);
		return a.two_level ? LRX_FETCH(false, true, 0u) : LRX_FETCH(false, false, 0u);
#undef LRX_FETCH
	}
	// compile-time variants; the occupancy-bounded build only takes <= 64-thread blocks
	uint32_t cv = a.variant & (kVarMinMax3 | kVarOccupancy);
	if (bs > 64 || a.nodes4) cv &= ~kVarOccupancy;  // (no occupancy-bounded builds for 64-byte records)
	if (smem_stack_bits(a.variant)) cv = smem_stack_bits(a.variant);  // builds of their own (no other compile-time bits)
	if (cnt) cv = 0;
	const size_t smem = sizeof(uint2) * (cv == kVarSmemStack32 ? 32 : cv == kVarSmemStack16 ? 16 : cv == kVarSmemStack ? 8 : 0) * bs;
#define LRX_LAUNCH(A, T, C, V) k_trace<A, T, C, V><<<grid, bs, smem, st>>>(a)
#define LRX_LAUNCH_V(A, T)                                         \
	switch (cv) {                                                  \
	case kVarSmemStack: LRX_LAUNCH(A, T, false, kVarSmemStack); break; \
	case kVarSmemStack16: LRX_LAUNCH(A, T, false, kVarSmemStack16); break; \
	case kVarSmemStack32: LRX_LAUNCH(A, T, false, kVarSmemStack32); break; \
	case kVarMinMax3: LRX_LAUNCH(A, T, false, kVarMinMax3); break; \
	case kVarOccupancy: LRX_LAUNCH(A, T, false, kVarOccupancy); break; \
	case kVarMinMax3 | kVarOccupancy: LRX_LAUNCH(A, T, false, kVarMinMax3 | kVarOccupancy); break; \
	default: LRX_LAUNCH(A, T, false, 0u); break;                   \
	}
#define LRX_LAUNCH_N4(A)                                                        \
	switch (cv) {                                                               \
	case kVarSmemStack: LRX_LAUNCH(A, false, false, kVarSmemStack | kVarNodes4); break; \
	case kVarSmemStack16: LRX_LAUNCH(A, false, false, kVarSmemStack16 | kVarNodes4); break; \
	case kVarSmemStack32: LRX_LAUNCH(A, false, false, kVarSmemStack32 | kVarNodes4); break; \
	case kVarMinMax3: LRX_LAUNCH(A, false, false, kVarMinMax3 | kVarNodes4); break; \
	default: LRX_LAUNCH(A, false, false, kVarNodes4); break;                    \
	}
	if (a.nodes4) {
		if (a.any_hit) { if (cnt) LRX_LAUNCH(true, false, true, kVarNodes4); else LRX_LAUNCH_N4(true); }
		else { if (cnt) LRX_LAUNCH(false, false, true, kVarNodes4); else LRX_LAUNCH_N4(false); }
	} else if (a.any_hit) {
		if (a.two_level) { if (cnt) LRX_LAUNCH(true, true, true, 0u); else LRX_LAUNCH_V(true, true); }
		else { if (cnt) LRX_LAUNCH(true, false, true, 0u); else LRX_LAUNCH_V(true, false); }
	} else {
		if (a.two_level) { if (cnt) LRX_LAUNCH(false, true, true, 0u); else LRX_LAUNCH_V(false, true); }
		else { if (cnt) LRX_LAUNCH(false, false, true, 0u); else LRX_LAUNCH_V(false, false); }
	}
#undef LRX_LAUNCH_N4
#undef LRX_LAUNCH_V
#undef LRX_LAUNCH
	LRX_CUDA(cudaGetLastError());
	k_clear_launch_start<<<1, 1, 0, st>>>(a.launch_id % kQueueSlots);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

}  // namespace lrx
