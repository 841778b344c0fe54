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

__device__ __forceinline__ float u8_to_float(uint32_t b) {
	return __uint_as_float(0x4B000000u | b) - 8388608.f;  // exact for b < 2^23
}

struct NodeHits {
	uint32_t child_base, tri_base, imask;
	uint32_t ihits;  // internal children, bit j = slot (j ^ oct)
	uint32_t tmask;  // leaf triangles, bit k = triangle tri_base + k
};

// Slab test of the 8 quantised child boxes.  t = q * (scale * idir) +
// (origin - o) * idir; NaN plane distances (zero direction components) are
// dropped by fminf/fmaxf, which only ever keeps a child.
__device__ __forceinline__ NodeHits intersect_node(const WideNode *__restrict__ nodes, uint32_t idx,
		const ActiveRay &r, float tmin, float tmax) {
	const uint4 *p = reinterpret_cast<const uint4 *>(nodes + idx);
	const uint4 w0 = __ldg(p), w1 = __ldg(p + 1), w2 = __ldg(p + 2), w3 = __ldg(p + 3), w4 = __ldg(p + 4);
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
	// qlo_x = w2.xy, qlo_y = w2.zw, qlo_z = w3.xy, qhi_x = w3.zw, qhi_y = w4.xy, qhi_z = w4.zw
	const uint32_t nx0 = px ? w2.x : w3.z, nx1 = px ? w2.y : w3.w;
	const uint32_t fx0 = px ? w3.z : w2.x, fx1 = px ? w3.w : w2.y;
	const uint32_t ny0 = py ? w2.z : w4.x, ny1 = py ? w2.w : w4.y;
	const uint32_t fy0 = py ? w4.x : w2.z, fy1 = py ? w4.y : w2.w;
	const uint32_t nz0 = pz ? w3.x : w4.z, nz1 = pz ? w3.y : w4.w;
	const uint32_t fz0 = pz ? w4.z : w3.x, fz1 = pz ? w4.w : w3.y;
	uint32_t ih = 0, tm = 0;
#pragma unroll
	for (int s = 0; s < 8; ++s) {
		const int sh = (s & 3) * 8;
		const uint32_t nxw = s < 4 ? nx0 : nx1, fxw = s < 4 ? fx0 : fx1;
		const uint32_t nyw = s < 4 ? ny0 : ny1, fyw = s < 4 ? fy0 : fy1;
		const uint32_t nzw = s < 4 ? nz0 : nz1, fzw = s < 4 ? fz0 : fz1;
		const uint32_t mw = s < 4 ? w1.z : w1.w;
		const float tnx = fmaf(u8_to_float((nxw >> sh) & 0xffu), ax, bx);
		const float tny = fmaf(u8_to_float((nyw >> sh) & 0xffu), ay, by);
		const float tnz = fmaf(u8_to_float((nzw >> sh) & 0xffu), az, bz);
		const float tfx = fmaf(u8_to_float((fxw >> sh) & 0xffu), ax, bx);
		const float tfy = fmaf(u8_to_float((fyw >> sh) & 0xffu), ay, by);
		const float tfz = fmaf(u8_to_float((fzw >> sh) & 0xffu), az, bz);
		const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
		const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
		const uint32_t m = (mw >> sh) & 0xffu;
		if (tn <= tf && m != 0u) {
			if (h.imask & (1u << s)) ih |= 1u << (s ^ r.oct);
			else tm |= ((m >> 5) & 7u) << (m & 31u);
		}
	}
	h.ihits = ih;
	h.tmask = tm;
	return h;
}

__device__ __forceinline__ bool finite3(float3 v) {
	return isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
}

// Per-lane traversal state, resumable one step at a time so a warp can refill
// lanes whose ray finished while the others keep going.
struct Traversal {
	float3 wo, wd;            // world-space ray
	float mint;
	ActiveRay ray;            // world ray, or the instance-local one
	float best_t, best_b1, best_b2;
	uint32_t best_mesh, best_tri;
	uint2 cur;                // node group being expanded, or an instance group
	int sp, inst_sp;
	uint32_t inst_obj;
	uint32_t visits;
	uint2 stack[kStackSize];
};

struct Counts {
	uint32_t nodes = 0, tris = 0, insts = 0;
};

// Loads ray i.  Returns false for a masked ray (nothing is traced and its
// hit is not written).  Rays that cannot hit anything (empty scene, NaN or
// infinite origin/direction, NaN maxt) get an empty group and finish on the
// first step with a miss.
__device__ __forceinline__ bool trav_init(Traversal &T, const TraceArgs &a, uint32_t i) {
	const float4 *rp = reinterpret_cast<const float4 *>(a.rays) + 3 * (size_t)i;
	const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
	if (__float_as_uint(r2.y) & LRX_RAY_FLAGS_MASKED) return false;  // bvh.cl:243-244
	T.wo = make_float3(r0.x, r0.y, r0.z);
	T.wd = make_float3(r0.w, r1.x, r1.y);
	T.mint = r1.z;
	T.best_t = r1.w;
	T.best_b1 = T.best_b2 = 0.f;
	T.best_mesh = T.best_tri = kNull;
	T.sp = 0;
	T.inst_sp = -1;
	T.inst_obj = kNull;
	T.visits = 0;
	make_active(T.ray, T.wo, T.wd);
	const bool live = a.root != kNull && finite3(T.wo) && finite3(T.wd) && !isnan(r1.w);
	T.cur = live ? make_uint2(a.root, (1u << (24 + T.ray.oct)) | 1u) : make_uint2(0u, 0u);
	return true;
}

__device__ __forceinline__ void write_hit(const TraceArgs &a, uint32_t i, const Traversal &T) {
	uint32_t *hp = reinterpret_cast<uint32_t *>(a.hits) + 5 * (size_t)i;
	hp[0] = __float_as_uint(T.best_t);
	hp[1] = __float_as_uint(T.best_b1);
	hp[2] = __float_as_uint(T.best_b2);
	hp[3] = T.best_mesh;
	hp[4] = T.best_tri;
}

__device__ __forceinline__ bool push(Traversal &T, const TraceArgs &a, uint2 v) {
	if (T.sp >= kStackSize) {
		atomicOr(a.status, kStatusStackOverflow);
		return false;
	}
	T.stack[T.sp++] = v;
	return true;
}

// One traversal step: pops empty groups, then enters one instance or expands
// one node and tests that node's leaf triangles.  Returns true when the ray
// is finished.
template <bool ANY, bool TWO_LEVEL, bool COUNT>
__device__ __forceinline__ bool trav_step(Traversal &T, const TraceArgs &a, Counts &C) {
	for (;;) {
		if (TWO_LEVEL && (T.cur.y & kInstGroup)) break;
		if (T.cur.y >> 24) break;
		if (TWO_LEVEL && T.inst_sp == T.sp) {  // the instance's BLAS is exhausted
			T.inst_sp = -1;
			T.inst_obj = kNull;
			make_active(T.ray, T.wo, T.wd);
		}
		if (T.sp == 0) return true;
		T.cur = T.stack[--T.sp];
	}
	if (TWO_LEVEL && (T.cur.y & kInstGroup)) {
		const uint32_t k = __ffs(T.cur.y & 0xffu) - 1;
		T.cur.y &= ~(1u << k);
		if ((T.cur.y & 0xffu) && !push(T, a, T.cur)) return true;
		const InstRecord *ir = a.insts + T.cur.x + k;
		const uint4 info = __ldg(reinterpret_cast<const uint4 *>(&ir->info));
		if (COUNT) ++C.insts;
		T.inst_obj = info.y;
		if (info.z & kInstIdentity) {
			make_active(T.ray, T.wo, T.wd);
		} else {
			const float4 m0 = __ldg(&ir->r0), m1 = __ldg(&ir->r1), m2 = __ldg(&ir->r2), m3 = __ldg(&ir->r3);
			make_active(T.ray, xform_point(m0, m1, m2, m3, T.wo), xform_vector(m0, m1, m2, T.wd));
		}
		T.inst_sp = T.sp;
		T.cur = info.x == kNull ? make_uint2(0u, 0u) : make_uint2(info.x, (1u << (24 + T.ray.oct)) | 1u);
		return false;
	}
	const uint32_t j = __ffs(T.cur.y >> 24) - 1;
	T.cur.y &= ~(1u << (24 + j));
	const uint32_t s = j ^ T.ray.oct;
	const uint32_t node = T.cur.x + __popc(T.cur.y & ((1u << s) - 1u) & 0xffu);
	if ((T.cur.y >> 24) && !push(T, a, T.cur)) return true;
	if (++T.visits > a.visit_limit) {
		atomicOr(a.status, kStatusVisitLimit);
		return true;
	}
	if (COUNT) ++C.nodes;
	const NodeHits h = intersect_node(a.nodes, node, T.ray, T.mint, T.best_t);
	T.cur = make_uint2(h.child_base, (h.ihits << 24) | h.imask);
	if (!h.tmask) return false;
	if (TWO_LEVEL && T.inst_sp < 0) {
		// top-level leaves are instances, entered one per step
		if ((T.cur.y >> 24) && !push(T, a, T.cur)) return true;
		T.cur = make_uint2(h.tri_base, kInstGroup | h.tmask);
		return false;
	}
	uint32_t tm = h.tmask;
	while (tm) {
		const uint32_t k = __ffs(tm) - 1;
		tm &= tm - 1;
		const float4 *tp = reinterpret_cast<const float4 *>(a.tris + h.tri_base + k);
		const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
		if (COUNT) ++C.tris;
		float t, b1, b2;
		if (tri_intersect(T.ray.o, T.ray.d, T.mint, T.best_t, make_float3(ta.x, ta.y, ta.z),
				make_float3(tb.x, tb.y, tb.z), make_float3(tc.x, tc.y, tc.z), t, b1, b2)) {
			const uint32_t tri = __float_as_uint(ta.w);
			uint32_t mesh = __float_as_uint(tb.w);
			if (TWO_LEVEL && mesh == kNull) mesh = T.inst_obj;
			if (ANY || t < T.best_t || mesh < T.best_mesh || (mesh == T.best_mesh && tri < T.best_tri)) {
				T.best_t = t;
				T.best_b1 = b1;
				T.best_b2 = b2;
				T.best_mesh = mesh;
				T.best_tri = tri;
				if (ANY) return true;
			}
		}
	}
	return false;
}

template <bool COUNT>
__device__ __forceinline__ void flush_counts(const TraceArgs &a, const Counts &C, uint32_t rays) {
	if (!COUNT) return;
	// every lane of the warp reaches this point
	unsigned long long v[4] = {C.nodes, C.tris, C.insts, rays};
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

// One thread per ray: the reference layout of work (bvh.cl:228-260).
template <bool ANY, bool TWO_LEVEL, bool COUNT>
__global__ void __launch_bounds__(128) k_trace(TraceArgs a) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (!COUNT && i >= a.count) return;
	Traversal T;
	Counts C;
	uint32_t traced = 0;
	if (i < a.count && trav_init(T, a, i)) {
		while (!trav_step<ANY, TWO_LEVEL, COUNT>(T, a, C)) {
		}
		write_hit(a, i, T);
		traced = 1;
	}
	flush_counts<COUNT>(a, C, traced);
}

// Persistent blocks with warp-level dynamic ray fetch.  Block b owns rays
// [b*chunk, (b+1)*chunk); its warps claim them from a shared-memory cursor.
// Whenever lanes of a warp are idle (their ray finished), one __ballot_sync
// finds them, one lane claims that many rays with a shared atomic and
// __shfl_sync broadcasts the base, so the warp keeps all lanes on live rays
// until the block's range runs dry.  No global scratch is used.
template <bool ANY, bool TWO_LEVEL, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) k_trace_pt(TraceArgs a, uint32_t chunk, uint32_t refill_min) {
	__shared__ uint32_t s_next;
	const uint32_t begin = blockIdx.x * chunk;
	const uint32_t end = min(begin + chunk, a.count);
	if (threadIdx.x == 0) s_next = begin;
	__syncthreads();
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t lt_mask = (1u << lane) - 1u;
	Traversal T;
	Counts C;
	uint32_t rid = kNull, traced = 0;
	bool exhausted = false;
	for (;;) {
		const uint32_t idle = __ballot_sync(0xffffffffu, rid == kNull);
		if (!exhausted && (__popc(idle) >= refill_min || idle == 0xffffffffu)) {
			const uint32_t nidle = __popc(idle);
			const uint32_t leader = __ffs(idle) - 1;
			uint32_t base = 0;
			if (lane == leader) base = atomicAdd(&s_next, nidle);
			base = __shfl_sync(0xffffffffu, base, leader);
			exhausted = base + nidle >= end;
			if (rid == kNull) {
				const uint32_t idx = base + __popc(idle & lt_mask);
				if (idx < end && trav_init(T, a, idx)) rid = idx;
			}
		}
		const uint32_t busy = __ballot_sync(0xffffffffu, rid != kNull);
		if (busy == 0) {
			if (exhausted) break;
			continue;  // every fetched ray was masked: fetch again
		}
		if (rid != kNull && trav_step<ANY, TWO_LEVEL, COUNT>(T, a, C)) {
			write_hit(a, rid, T);
			rid = kNull;
			++traced;
		}
	}
	flush_counts<COUNT>(a, C, traced);
}

static int g_num_sms = 0;

lrx_status launch_trace(const TraceArgs &a, cudaStream_t st) {
	if (a.count == 0) return LRX_OK;
	if (a.kernel == kKernelSimple) {
		const uint32_t bs = 128;
		const uint32_t grid = (a.count + bs - 1) / bs;
		const bool cnt = a.counters != nullptr;
#define LRX_LAUNCH(A, T, C) k_trace<A, T, C><<<grid, bs, 0, st>>>(a)
		if (a.any_hit) {
			if (a.two_level) { if (cnt) LRX_LAUNCH(true, true, true); else LRX_LAUNCH(true, true, false); }
			else { if (cnt) LRX_LAUNCH(true, false, true); else LRX_LAUNCH(true, false, false); }
		} else {
			if (a.two_level) { if (cnt) LRX_LAUNCH(false, true, true); else LRX_LAUNCH(false, true, false); }
			else { if (cnt) LRX_LAUNCH(false, false, true); else LRX_LAUNCH(false, false, false); }
		}
#undef LRX_LAUNCH
		LRX_CUDA(cudaGetLastError());
		return LRX_OK;
	}
	if (g_num_sms == 0) {
		int dev = 0, n = 0;
		LRX_CUDA(cudaGetDevice(&dev));
		LRX_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
		g_num_sms = n;
	}
	// resident blocks: 152 SMs x blocks_per_sm, each owning an equal ray range
	const uint32_t per_sm = a.blocks_per_sm ? a.blocks_per_sm : 8u;
	const uint32_t max_blocks = (uint32_t)g_num_sms * per_sm;
	const uint32_t min_chunk = 2u * kTraceBlock;
	uint32_t grid = (a.count + min_chunk - 1) / min_chunk;
	if (grid > max_blocks) grid = max_blocks;
	const uint32_t chunk = (a.count + grid - 1) / grid;
	grid = (a.count + chunk - 1) / chunk;
	const uint32_t refill = a.refill_min ? a.refill_min : 1u;
	const bool cnt = a.counters != nullptr;
#define LRX_LAUNCH(A, T, C) k_trace_pt<A, T, C><<<grid, kTraceBlock, 0, st>>>(a, chunk, refill)
	if (a.any_hit) {
		if (a.two_level) { if (cnt) LRX_LAUNCH(true, true, true); else LRX_LAUNCH(true, true, false); }
		else { if (cnt) LRX_LAUNCH(true, false, true); else LRX_LAUNCH(true, false, false); }
	} else {
		if (a.two_level) { if (cnt) LRX_LAUNCH(false, true, true); else LRX_LAUNCH(false, true, false); }
		else { if (cnt) LRX_LAUNCH(false, false, true); else LRX_LAUNCH(false, false, false); }
	}
#undef LRX_LAUNCH
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

}  // namespace lrx
