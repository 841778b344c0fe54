// GPU BVH builder: 63-bit Morton codes -> radix sort -> bottom-up LBVH
// (one thread per leaf climbing with an atomic per internal node, the
// agglomerative formulation of Apetrei 2014 over the Karras 2012 ordering)
// -> optional treelet restructuring -> SAH-optimal top-down collapse into
// 8-wide nodes with outward-rounded 8-bit child boxes (the compressed wide
// BVH of Ylitie, Karras and Laine 2017).
//
// Replaces the reference's CPU builders (src/luxrays/core/bvh/
// bvhclassicbuild.cpp:124-233, bvhembreebuild.cpp:218-357): any correct BVH
// returns the same closest hit, so the tree shape is free; what must hold is
// that every child box contains its primitives' padded boxes, which the
// outward rounding below guarantees.
#include <algorithm>
#include <cstring>

#include <cub/device/device_radix_sort.cuh>

#include "lrx_common.cuh"
#include "lrx_internal.h"

namespace lrx {

constexpr uint32_t kLeafFlag = 0x80000000u;

// counters[] layout (uint32)
enum : int {
	C_BMIN = 0,    // 3: centroid bounds min (ordered uint)
	C_BMAX = 3,    // 3: centroid bounds max
	C_ROOT = 6,    // binary root reference
	C_NODES = 7,   // wide-node allocation counter
	C_TRIS = 8,    // leaf-primitive allocation counter
	C_QA = 9,      // queue A item count
	C_QB = 10,     // queue B item count
	C_ERR = 11,    // nonzero: a capacity guard fired (never expected)
	C_BOX = 12,    // 6 floats: root box lo.xyz, hi.xyz
	C_COUNT = 20
};

// ---------------------------------------------------------------------------
// Morton codes
// ---------------------------------------------------------------------------

__global__ void k_centroid_bounds(uint32_t n, const float4 *__restrict__ lo, const float4 *__restrict__ hi,
		uint32_t *counters) {
	float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float4 a = lo[i], b = hi[i];
		const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			mn[k] = fminf(mn[k], c[k]);
			mx[k] = fmaxf(mx[k], c[k]);
		}
	}
#pragma unroll
	for (int k = 0; k < 3; ++k) {
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) {
			mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
			mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
		}
	}
	if ((threadIdx.x & 31) == 0) {
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			atomicMin(&counters[C_BMIN + k], f2ord(mn[k]));
			atomicMax(&counters[C_BMAX + k], f2ord(mx[k]));
		}
	}
}

__device__ __forceinline__ uint64_t expand21(uint32_t v) {
	uint64_t x = v & 0x1fffffu;
	x = (x | x << 32) & 0x1f00000000ffffull;
	x = (x | x << 16) & 0x1f0000ff0000ffull;
	x = (x | x << 8) & 0x100f00f00f00f00full;
	x = (x | x << 4) & 0x10c30c30c30c30c3ull;
	x = (x | x << 2) & 0x1249249249249249ull;
	return x;
}

__global__ void k_morton(uint32_t n, const float4 *__restrict__ lo, const float4 *__restrict__ hi,
		const uint32_t *__restrict__ counters, uint64_t *keys, uint32_t *vals) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float4 a = lo[i], b = hi[i];
	const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
	uint32_t q[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const float mn = ord2f(counters[C_BMIN + k]), mx = ord2f(counters[C_BMAX + k]);
		const float ext = mx - mn;
		float u = ext > 0.f ? (c[k] - mn) / ext : 0.f;
		u = fminf(fmaxf(u, 0.f), 1.f);
		q[k] = min((uint32_t)(u * 2097152.f), 2097151u);
	}
	keys[i] = (expand21(q[0]) << 2) | (expand21(q[1]) << 1) | expand21(q[2]);
	vals[i] = i;
}

// ---------------------------------------------------------------------------
// Bottom-up binary hierarchy
// ---------------------------------------------------------------------------

// delta(a) < delta(b), delta(i) = (key[i] ^ key[i+1], i ^ (i+1)) compared
// lexicographically: the key bits dominate, the index breaks key ties.
__device__ __forceinline__ bool delta_less(const uint64_t *__restrict__ keys, uint32_t a, uint32_t b) {
	const uint64_t ka = keys[a] ^ keys[a + 1], kb = keys[b] ^ keys[b + 1];
	if (ka != kb) return ka < kb;
	return (a ^ (a + 1)) < (b ^ (b + 1));
}

// Per internal node k of the binary tree: children bchild[2k], bchild[2k+1]
// (kLeafFlag | leaf position in sorted order, or an internal node), box
// bn_lo/bn_hi[k], bmeta[k] = (leaf count, parent; kNull for the root); per
// leaf position i: lparent[i].  The treelet pass rewrites topology, boxes
// and counts in place, so subtrees need not stay contiguous in sorted order.
__global__ void k_hierarchy(uint32_t n, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ sorted,
		const float4 *__restrict__ plo, const float4 *__restrict__ phi, uint32_t *bchild, float4 *bn_lo,
		float4 *bn_hi, uint2 *bmeta, uint32_t *lparent, uint32_t *other, uint32_t *counters) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const uint32_t p = sorted[i];
	float4 lo = plo[p], hi = phi[p];
	if (n == 1) {
		counters[C_ROOT] = kLeafFlag;
		reinterpret_cast<float *>(counters + C_BOX)[0] = lo.x;
		reinterpret_cast<float *>(counters + C_BOX)[1] = lo.y;
		reinterpret_cast<float *>(counters + C_BOX)[2] = lo.z;
		reinterpret_cast<float *>(counters + C_BOX)[3] = hi.x;
		reinterpret_cast<float *>(counters + C_BOX)[4] = hi.y;
		reinterpret_cast<float *>(counters + C_BOX)[5] = hi.z;
		return;
	}
	uint32_t l = i, r = i, cur = kLeafFlag | i;
	// Each climb step moves to a strictly larger range, so the loop ends in
	// at most n steps.
	for (uint32_t step = 0; step < n; ++step) {
		const bool left_child = (l == 0) || (r != n - 1 && delta_less(keys, r, l - 1));
		const uint32_t parent = left_child ? r : l - 1;
		bchild[2 * parent + (left_child ? 0 : 1)] = cur;
		if (cur & kLeafFlag) lparent[cur & ~kLeafFlag] = parent;
		else reinterpret_cast<uint32_t *>(bmeta)[2 * cur + 1] = parent;
		__threadfence();
		const uint32_t prev = atomicExch(&other[parent], left_child ? l : r);
		if (prev == kNull) return;  // the sibling finishes this node
		__threadfence();
		if (left_child) r = prev;
		else l = prev;
		const uint32_t sib = __ldcg(&bchild[2 * parent + (left_child ? 1 : 0)]);
		float4 slo, shi;
		if (sib & kLeafFlag) {
			const uint32_t sp = sorted[sib & ~kLeafFlag];
			slo = plo[sp];
			shi = phi[sp];
		} else {
			slo = __ldcg(&bn_lo[sib]);
			shi = __ldcg(&bn_hi[sib]);
		}
		lo = make_float4(fminf(lo.x, slo.x), fminf(lo.y, slo.y), fminf(lo.z, slo.z), 0.f);
		hi = make_float4(fmaxf(hi.x, shi.x), fmaxf(hi.y, shi.y), fmaxf(hi.z, shi.z), 0.f);
		__stcg(&bn_lo[parent], lo);
		__stcg(&bn_hi[parent], hi);
		__stcg(reinterpret_cast<uint32_t *>(bmeta) + 2 * parent, r - l + 1);
		cur = parent;
		if (l == 0 && r == n - 1) {
			counters[C_ROOT] = parent;
			float *box = reinterpret_cast<float *>(counters + C_BOX);
			box[0] = lo.x; box[1] = lo.y; box[2] = lo.z;
			box[3] = hi.x; box[4] = hi.y; box[5] = hi.z;
			return;
		}
	}
}

// ---------------------------------------------------------------------------
// Treelet restructuring (after Karras and Aila 2013): a bottom-up sweep in
// which the second thread to reach a node owns its whole (finished) subtree.
// At a node with at least `min_prims` primitives it grows a treelet of up to
// 7 leaves -- repeatedly splitting the treelet leaf of largest area -- finds
// the topology of least SAH cost over those leaves by dynamic programming
// over the 127 leaf subsets, and rewrites the treelet's internal nodes in
// place (same node indices, the treelet root keeps its position).  Costs:
// internal node 1.2 x area, leaf-sized subtree (<= leaf_max primitives,
// which the collapse turns into one leaf slot) 1.0 x area x primitives.
// ---------------------------------------------------------------------------

constexpr float kSahNode = 1.2f, kSahTri = 1.0f;
constexpr int kTreeletLeaves = 7;

__device__ __forceinline__ float box_area(float3 lo, float3 hi) {
	const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
	return dx * dy + dx * dz + dy * dz;
}

struct TreeletLeaf {
	uint32_t ref, count;
	float3 lo, hi;
	float cost;
};

__device__ __forceinline__ void treelet_leaf(uint32_t ref, const uint32_t *__restrict__ sorted,
		const float4 *__restrict__ plo, const float4 *__restrict__ phi, const float4 *bn_lo, const float4 *bn_hi,
		const uint2 *bmeta, const float *cost, TreeletLeaf &t) {
	t.ref = ref;
	float4 a, c;
	if (ref & kLeafFlag) {
		const uint32_t p = sorted[ref & ~kLeafFlag];
		a = plo[p];
		c = phi[p];
		t.count = 1;
	} else {
		a = __ldcg(&bn_lo[ref]);
		c = __ldcg(&bn_hi[ref]);
		t.count = __ldcg(reinterpret_cast<const uint32_t *>(bmeta) + 2 * ref);
	}
	t.lo = make_float3(a.x, a.y, a.z);
	t.hi = make_float3(c.x, c.y, c.z);
	t.cost = (ref & kLeafFlag) ? kSahTri * box_area(t.lo, t.hi) : __ldcg(&cost[ref]);
}

__device__ __forceinline__ float subtree_cost(float area, float child_costs, uint32_t count, uint32_t leaf_max) {
	const float c = kSahNode * area + child_costs;
	return count <= leaf_max ? fminf(c, kSahTri * area * (float)count) : c;
}

__global__ void __launch_bounds__(128) k_treelet(uint32_t n, const uint32_t *__restrict__ sorted,
		const float4 *__restrict__ plo, const float4 *__restrict__ phi, uint32_t *bchild, float4 *bn_lo,
		float4 *bn_hi, uint2 *bmeta, uint32_t *lparent, float *cost, uint32_t *visits, uint32_t leaf_max,
		uint32_t min_prims) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	uint32_t *meta = reinterpret_cast<uint32_t *>(bmeta);  // [2k] leaf count, [2k + 1] parent
	uint32_t node = __ldcg(&lparent[i]);
	// each step moves to the parent, so the climb ends within n steps
	for (uint32_t step = 0; step < n && node != kNull; ++step) {
		__threadfence();
		if (atomicAdd(&visits[node], 1u) == 0u) return;  // the sibling subtree's thread continues
		__threadfence();
		const uint32_t count = __ldcg(&meta[2 * node]);
		TreeletLeaf L[kTreeletLeaves];
		treelet_leaf(__ldcg(&bchild[2 * node]), sorted, plo, phi, bn_lo, bn_hi, bmeta, cost, L[0]);
		treelet_leaf(__ldcg(&bchild[2 * node + 1]), sorted, plo, phi, bn_lo, bn_hi, bmeta, cost, L[1]);
		const float4 nlo4 = __ldcg(&bn_lo[node]), nhi4 = __ldcg(&bn_hi[node]);
		const float area = box_area(make_float3(nlo4.x, nlo4.y, nlo4.z), make_float3(nhi4.x, nhi4.y, nhi4.z));
		const float current = subtree_cost(area, L[0].cost + L[1].cost, count, leaf_max);
		float best_cost = current;
		if (count >= min_prims) {
			uint32_t inner[kTreeletLeaves - 1];
			int nl = 2, ni = 1;
			inner[0] = node;
			while (nl < kTreeletLeaves) {  // split the largest-area internal leaf
				int best = -1;
				float ba = -1.f;
				for (int k = 0; k < nl; ++k) {
					if (L[k].ref & kLeafFlag) continue;
					const float a = box_area(L[k].lo, L[k].hi);
					if (a > ba) {
						ba = a;
						best = k;
					}
				}
				if (best < 0) break;
				const uint32_t r = L[best].ref;
				inner[ni++] = r;
				treelet_leaf(__ldcg(&bchild[2 * r]), sorted, plo, phi, bn_lo, bn_hi, bmeta, cost, L[best]);
				treelet_leaf(__ldcg(&bchild[2 * r + 1]), sorted, plo, phi, bn_lo, bn_hi, bmeta, cost, L[nl++]);
			}
			if (nl >= 3) {
				float copt[1 << kTreeletLeaves];
				uint8_t part[1 << kTreeletLeaves];
				const uint32_t full = (1u << nl) - 1u;
				for (uint32_t S = 1; S <= full; ++S) {
					if ((S & (S - 1u)) == 0u) {
						copt[S] = L[__ffs(S) - 1].cost;
						part[S] = 0;
						continue;
					}
					float3 lo = make_float3(INFINITY, INFINITY, INFINITY), hi = make_float3(-INFINITY, -INFINITY, -INFINITY);
					uint32_t c = 0;
					for (int k = 0; k < nl; ++k) {
						if (!((S >> k) & 1u)) continue;
						lo = make_float3(fminf(lo.x, L[k].lo.x), fminf(lo.y, L[k].lo.y), fminf(lo.z, L[k].lo.z));
						hi = make_float3(fmaxf(hi.x, L[k].hi.x), fmaxf(hi.y, L[k].hi.y), fmaxf(hi.z, L[k].hi.z));
						c += L[k].count;
					}
					// two-way splits of S; the part holding S's lowest leaf enumerates each once
					const uint32_t low = S & (0u - S), rest = S ^ low;
					float bc = INFINITY;
					uint32_t bp = low;
					for (uint32_t sub = rest;; sub = (sub - 1u) & rest) {
						const uint32_t P = sub | low;
						if (P != S) {
							const float cc = copt[P] + copt[S ^ P];
							if (cc < bc) {
								bc = cc;
								bp = P;
							}
						}
						if (sub == 0u) break;
					}
					copt[S] = subtree_cost(box_area(lo, hi), bc, c, leaf_max);
					part[S] = (uint8_t)bp;
				}
				if (copt[full] < current * 0.9999f) {
					best_cost = copt[full];
					// rewrite: subsets of the optimal split tree onto the treelet's internal nodes
					uint32_t st_set[kTreeletLeaves], st_node[kTreeletLeaves];
					int sp = 0, next = 1;
					st_set[sp] = full;
					st_node[sp++] = node;
					while (sp > 0) {
						--sp;
						const uint32_t S = st_set[sp], idx = st_node[sp];
						const uint32_t halves[2] = {part[S], S ^ part[S]};
						for (int side = 0; side < 2; ++side) {
							const uint32_t sub = halves[side];
							uint32_t ref;
							if ((sub & (sub - 1u)) == 0u) {
								ref = L[__ffs(sub) - 1].ref;
								if (ref & kLeafFlag) __stcg(&lparent[ref & ~kLeafFlag], idx);
								else __stcg(&meta[2 * ref + 1], idx);
							} else {
								ref = inner[next++];
								__stcg(&meta[2 * ref + 1], idx);
								st_set[sp] = sub;
								st_node[sp++] = ref;
							}
							__stcg(&bchild[2 * idx + side], ref);
						}
						float3 lo = make_float3(INFINITY, INFINITY, INFINITY), hi = make_float3(-INFINITY, -INFINITY, -INFINITY);
						uint32_t c = 0;
						for (int k = 0; k < nl; ++k) {
							if (!((S >> k) & 1u)) continue;
							lo = make_float3(fminf(lo.x, L[k].lo.x), fminf(lo.y, L[k].lo.y), fminf(lo.z, L[k].lo.z));
							hi = make_float3(fmaxf(hi.x, L[k].hi.x), fmaxf(hi.y, L[k].hi.y), fmaxf(hi.z, L[k].hi.z));
							c += L[k].count;
						}
						__stcg(&bn_lo[idx], make_float4(lo.x, lo.y, lo.z, 0.f));
						__stcg(&bn_hi[idx], make_float4(hi.x, hi.y, hi.z, 0.f));
						__stcg(&meta[2 * idx], c);
						__stcg(&cost[idx], copt[S]);
					}
				}
			}
		}
		__stcg(&cost[node], best_cost);
		node = __ldcg(&meta[2 * node + 1]);
	}
}

// ---------------------------------------------------------------------------
// Which binary nodes become wide nodes: the SAH-optimal collapse of Ylitie,
// Karras and Laine 2017 (section 3.1), by dynamic programming bottom-up over
// the binary tree.  C(x, i) is the least cost of covering x's subtree with
// at most i roots -- each root a leaf slot (<= leaf_max primitives) or a wide
// node of its own:
//   C(x, 1) = kWideTri * A(x) * count(x)      if count(x) <= leaf_max
//           = kWideNode * A(x) + D(x, width)  otherwise (x is a wide node)
//   D(x, j) = min over k in [1, j-1] of C(left, k) + C(right, j - k)
//   C(x, i) = min(C(x, 1), D(x, i))           for i >= 2
// and a primitive costs kWideTri * its area for any i.  Per node the pass
// stores C(x, 1..8) and a decision word: byte 0 the k of D(x, width) (how
// a wide node at x spreads its slots over its two subtrees), byte i-1 for
// i >= 2 the k of D(x, i), or 0 when x itself is the cheaper single root.
// A wide node test takes about four times the instructions of a triangle
// test, but runs on about eight times as many lanes of a warp (triangle
// groups are small and ragged): per ray the two cost about the same, and
// weights of 1 : 1 gave the fastest trees on the heightfield's three ray sets
// (1 : 0.25 and 1 : 0.5 left more triangles per leaf and ran 1.4 % and 0.4 %
// slower).
// ---------------------------------------------------------------------------

constexpr float kWideNode = 1.0f, kWideTri = 1.0f;

__device__ __forceinline__ void wide_child_costs(uint32_t ref, const uint32_t *__restrict__ sorted,
		const float4 *__restrict__ plo, const float4 *__restrict__ phi, const float4 *wcost, float c[8]) {
	if (ref & kLeafFlag) {
		const uint32_t p = sorted[ref & ~kLeafFlag];
		const float4 a = plo[p], b = phi[p];
		const float v = kWideTri * box_area(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z));
#pragma unroll
		for (int k = 0; k < 8; ++k) c[k] = v;
	} else {
		const float4 u = __ldcg(&wcost[2 * ref]), w = __ldcg(&wcost[2 * ref + 1]);
		c[0] = u.x; c[1] = u.y; c[2] = u.z; c[3] = u.w;
		c[4] = w.x; c[5] = w.y; c[6] = w.z; c[7] = w.w;
	}
}

__global__ void __launch_bounds__(128) k_wide_cost(uint32_t n, const uint32_t *__restrict__ sorted,
		const float4 *__restrict__ plo, const float4 *__restrict__ phi, const uint32_t *bchild, const float4 *bn_lo,
		const float4 *bn_hi, const uint2 *bmeta, const uint32_t *lparent, uint32_t *visits, uint32_t leaf_max,
		uint32_t width, float4 *wcost, uint2 *wdec) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const uint32_t *meta = reinterpret_cast<const uint32_t *>(bmeta);  // [2k] leaf count, [2k + 1] parent
	uint32_t node = __ldcg(&lparent[i]);
	// each step moves to the parent, so the climb ends within n steps
	for (uint32_t step = 0; step < n && node != kNull; ++step) {
		__threadfence();
		if (atomicAdd(&visits[node], 1u) == 0u) return;  // the sibling subtree's thread continues
		__threadfence();
		float cl[8], cr[8];
		wide_child_costs(__ldcg(&bchild[2 * node]), sorted, plo, phi, wcost, cl);
		wide_child_costs(__ldcg(&bchild[2 * node + 1]), sorted, plo, phi, wcost, cr);
		const float4 lo4 = __ldcg(&bn_lo[node]), hi4 = __ldcg(&bn_hi[node]);
		const float area = box_area(make_float3(lo4.x, lo4.y, lo4.z), make_float3(hi4.x, hi4.y, hi4.z));
		const uint32_t count = __ldcg(&meta[2 * node]);
		float dist[9];
		uint32_t split[9];
		for (uint32_t j = 2; j <= width; ++j) {
			float best = INFINITY;
			uint32_t bk = 1;
			for (uint32_t k = 1; k < j; ++k) {
				const float c = cl[k - 1] + cr[j - k - 1];
				if (c < best) {
					best = c;
					bk = k;
				}
			}
			dist[j] = best;
			split[j] = bk;
		}
		const float c1 = count <= leaf_max ? kWideTri * area * (float)count : kWideNode * area + dist[width];
		float c[8];
		uint32_t dec[8];
		c[0] = c1;
		dec[0] = split[width];
		for (uint32_t k = 2; k <= 8; ++k) {
			const uint32_t j = k <= width ? k : width;
			const bool use = dist[j] < c1;
			c[k - 1] = use ? dist[j] : c1;
			dec[k - 1] = use ? split[j] : 0u;
		}
		__stcg(&wcost[2 * node], make_float4(c[0], c[1], c[2], c[3]));
		__stcg(&wcost[2 * node + 1], make_float4(c[4], c[5], c[6], c[7]));
		__stcg(&wdec[node], make_uint2(dec[0] | dec[1] << 8 | dec[2] << 16 | dec[3] << 24,
				dec[4] | dec[5] << 8 | dec[6] << 16 | dec[7] << 24));
		node = __ldcg(&meta[2 * node + 1]);
	}
}

// ---------------------------------------------------------------------------
// Collapse to 8-wide quantised nodes
// ---------------------------------------------------------------------------

// Smallest biased exponent e (scale 2^(e-127)) with ext * 2^-(e-127) <= 255.
__device__ __forceinline__ uint32_t quant_exponent(float ext) {
	if (!(ext > 0.f)) return 1u;
	const int ex = (int)((__float_as_uint(ext) >> 23) & 0xffu);
	int e = ex - 8;
	if (e < 1) e = 1;
	while (e < 253 && __fmul_ru(ext, __uint_as_float((uint32_t)(254 - e) << 23)) > 255.f) ++e;
	return (uint32_t)e;
}

struct ChildBox {
	float3 lo, hi;
};

__device__ __forceinline__ void load_ref_box(uint32_t ref, const uint32_t *__restrict__ sorted,
		const float4 *__restrict__ plo, const float4 *__restrict__ phi, const float4 *__restrict__ bn_lo,
		const float4 *__restrict__ bn_hi, ChildBox &b) {
	float4 a, c;
	if (ref & kLeafFlag) {
		const uint32_t p = sorted[ref & ~kLeafFlag];
		a = plo[p];
		c = phi[p];
	} else {
		a = bn_lo[ref];
		c = bn_hi[ref];
	}
	b.lo = make_float3(a.x, a.y, a.z);
	b.hi = make_float3(c.x, c.y, c.z);
}

__global__ void __launch_bounds__(128) k_collapse(const uint2 *__restrict__ items, const uint32_t *n_items_ptr,
		uint2 *__restrict__ out_items, uint32_t *n_out, const uint32_t *__restrict__ bchild,
		const float4 *__restrict__ bn_lo, const float4 *__restrict__ bn_hi, const uint2 *__restrict__ bmeta,
		const uint32_t *__restrict__ sorted, const float4 *__restrict__ plo, const float4 *__restrict__ phi,
		uint32_t leaf_max, uint32_t width, WideNode *__restrict__ wnodes, uint32_t *__restrict__ prim_order,
		uint32_t *counters, uint32_t cap, const uint2 *__restrict__ wdec) {
	// wdec: k_wide_cost's decisions, present whenever the tree has an internal node
	// cap = primitive count: bounds the node array, the leaf order and each queue
	const uint32_t n_items = min(*n_items_ptr, cap);
	for (uint32_t it = blockIdx.x * blockDim.x + threadIdx.x; it < n_items; it += gridDim.x * blockDim.x) {
		const uint2 item = items[it];
		uint32_t cref[8];
		ChildBox cb[8];
		int cnt;
		if (item.x & kLeafFlag) {
			cref[0] = item.x;
			load_ref_box(item.x, sorted, plo, phi, bn_lo, bn_hi, cb[0]);
			cnt = 1;
		} else {
			// the SAH-optimal cover of the subtree by at most `width` roots
			// (k_wide_cost's decisions); each split divides a slot budget j
			// into k and j - k, so the roots never exceed `width`
			uint32_t st_ref[8], st_j[8];
			int sp = 0;
			cnt = 0;
			const uint32_t k0 = wdec[item.x].x & 0xffu;
			st_ref[sp] = bchild[2 * item.x + 1];
			st_j[sp++] = width - k0;
			st_ref[sp] = bchild[2 * item.x];
			st_j[sp++] = k0;
			while (sp > 0 && cnt < 8) {
				--sp;
				const uint32_t r = st_ref[sp], j = st_j[sp];
				uint32_t k = 0;
				if (!(r & kLeafFlag) && j >= 2 && j <= 8) {
					const uint2 d = wdec[r];
					k = ((j <= 4 ? d.x : d.y) >> (8 * ((j - 1) & 3))) & 0xffu;
				}
				if (k == 0 || k >= j || sp + 2 > 8) {  // r is one root
					cref[cnt] = r;
					load_ref_box(r, sorted, plo, phi, bn_lo, bn_hi, cb[cnt]);
					++cnt;
				} else {
					st_ref[sp] = bchild[2 * r + 1];
					st_j[sp++] = j - k;
					st_ref[sp] = bchild[2 * r];
					st_j[sp++] = k;
				}
			}
			if (sp > 0 || k0 == 0 || k0 >= width) atomicOr(&counters[C_ERR], 64u);  // never: a cover lost a subtree
		}
		// Child primitive counts and node bounds
		uint32_t ccount[8];
		float3 nlo = cb[0].lo, nhi = cb[0].hi;
		uint32_t n_int = 0, n_tri = 0;
		for (int k = 0; k < cnt; ++k) {
			ccount[k] = (cref[k] & kLeafFlag) ? 1u : bmeta[cref[k]].x;
			if (ccount[k] > leaf_max) ++n_int;
			else n_tri += ccount[k];
			nlo = make_float3(fminf(nlo.x, cb[k].lo.x), fminf(nlo.y, cb[k].lo.y), fminf(nlo.z, cb[k].lo.z));
			nhi = make_float3(fmaxf(nhi.x, cb[k].hi.x), fmaxf(nhi.y, cb[k].hi.y), fmaxf(nhi.z, cb[k].hi.z));
		}
		// Slot assignment: slot s takes the child lying furthest against the
		// direction octant s (sign bit set = negative axis), so a ray of
		// octant o meets children roughly front to back in slot order j ^ o.
		int slot_child[8];
		for (int s = 0; s < 8; ++s) slot_child[s] = -1;
		{
			const float3 pc = make_float3(0.5f * (nlo.x + nhi.x), 0.5f * (nlo.y + nhi.y), 0.5f * (nlo.z + nhi.z));
			float cost[8][8];
			for (int k = 0; k < cnt; ++k) {
				const float cx = 0.5f * (cb[k].lo.x + cb[k].hi.x) - pc.x;
				const float cy = 0.5f * (cb[k].lo.y + cb[k].hi.y) - pc.y;
				const float cz = 0.5f * (cb[k].lo.z + cb[k].hi.z) - pc.z;
				for (int s = 0; s < 8; ++s)
					cost[k][s] = ((s & 1) ? -cx : cx) + ((s & 2) ? -cy : cy) + ((s & 4) ? -cz : cz);
			}
			uint32_t kdone = 0, sdone = 0;
			for (int round = 0; round < cnt; ++round) {
				float bc = INFINITY;
				int bk = -1, bs = -1;
				for (int k = 0; k < cnt; ++k) {
					if (kdone & (1u << k)) continue;
					for (int s = 0; s < 8; ++s) {
						if (sdone & (1u << s)) continue;
						if (bk < 0 || cost[k][s] < bc) {
							bc = cost[k][s];
							bk = k;
							bs = s;
						}
					}
				}
				kdone |= 1u << bk;
				sdone |= 1u << bs;
				slot_child[bs] = bk;
			}
		}
		// Quantisation grid: origin = node min, per-axis power-of-two scale.
		const uint32_t ex = quant_exponent(__fsub_ru(nhi.x, nlo.x));
		const uint32_t ey = quant_exponent(__fsub_ru(nhi.y, nlo.y));
		const uint32_t ez = quant_exponent(__fsub_ru(nhi.z, nlo.z));
		const float ix = __uint_as_float((254u - ex) << 23);
		const float iy = __uint_as_float((254u - ey) << 23);
		const float iz = __uint_as_float((254u - ez) << 23);

		const uint32_t child_base = n_int ? atomicAdd(&counters[C_NODES], n_int) : 0u;
		const uint32_t tri_base = n_tri ? atomicAdd(&counters[C_TRIS], n_tri) : 0u;
		if (child_base + n_int > cap || tri_base + n_tri > cap || item.y >= cap) {
			atomicOr(&counters[C_ERR], 1u);
			continue;
		}

		uint32_t imask = 0, int_rank = 0, tri_off = 0;
		uint32_t meta[2] = {0, 0}, qlx[2] = {0, 0}, qly[2] = {0, 0}, qlz[2] = {0, 0};
		uint32_t qhx[2] = {0, 0}, qhy[2] = {0, 0}, qhz[2] = {0, 0};
		for (int s = 0; s < 8; ++s) {
			const int k = slot_child[s];
			if (k < 0) continue;
			auto qlo = [](float v, float org, float inv) {
				const float q = floorf(__fmul_rd(__fsub_rd(v, org), inv));
				return (uint32_t)fminf(fmaxf(q, 0.f), 255.f);
			};
			auto qhi = [](float v, float org, float inv) {
				const float q = ceilf(__fmul_ru(__fsub_ru(v, org), inv));
				return (uint32_t)fminf(fmaxf(q, 0.f), 255.f);
			};
			const int wsel = s >> 2, sh = (s & 3) * 8;
			qlx[wsel] |= qlo(cb[k].lo.x, nlo.x, ix) << sh;
			qly[wsel] |= qlo(cb[k].lo.y, nlo.y, iy) << sh;
			qlz[wsel] |= qlo(cb[k].lo.z, nlo.z, iz) << sh;
			qhx[wsel] |= qhi(cb[k].hi.x, nlo.x, ix) << sh;
			qhy[wsel] |= qhi(cb[k].hi.y, nlo.y, iy) << sh;
			qhz[wsel] |= qhi(cb[k].hi.z, nlo.z, iz) << sh;
			if (ccount[k] > leaf_max) {
				imask |= 1u << s;
				meta[wsel] |= (kInternalMetaBase + s) << sh;
				const uint32_t slot = atomicAdd(n_out, 1u);
				if (slot < cap) out_items[slot] = make_uint2(cref[k], child_base + int_rank);
				else atomicOr(&counters[C_ERR], 2u);
				++int_rank;
			} else {
				const uint32_t m = (((1u << ccount[k]) - 1u) << 5) | tri_off;
				meta[wsel] |= m << sh;
				// the subtree's (<= leaf_max <= 3) primitives, by a walk of its binary nodes
				uint32_t walk[4], wsp = 0, j = 0;
				walk[wsp++] = cref[k];
				for (int it = 0; it < 16 && wsp && j < ccount[k]; ++it) {  // <= 5 nodes; the cap guards bad input
					const uint32_t r = walk[--wsp];
					if (r & kLeafFlag) {
						prim_order[tri_base + tri_off + j++] = sorted[r & ~kLeafFlag];
					} else if (wsp + 2 <= 4) {
						walk[wsp++] = bchild[2 * r + 1];
						walk[wsp++] = bchild[2 * r];
					}
				}
				if (j != ccount[k]) atomicOr(&counters[C_ERR], 32u);
				tri_off += ccount[k];
			}
		}
		WideNode nd;
		nd.w[0] = make_uint4(__float_as_uint(nlo.x), __float_as_uint(nlo.y), __float_as_uint(nlo.z),
				ex | (ey << 8) | (ez << 16) | (imask << 24));
		nd.w[1] = make_uint4(child_base, tri_base, meta[0], meta[1]);
		nd.w[2] = make_uint4(qlx[0], qlx[1], qly[0], qly[1]);
		nd.w[3] = make_uint4(qlz[0], qlz[1], qhx[0], qhx[1]);
		nd.w[4] = make_uint4(qhy[0], qhy[1], qhz[0], qhz[1]);
		wnodes[item.y] = nd;
	}
}

// Structural check of a finished wide BVH: every node but the root is the
// child of exactly one node, every leaf-order slot is referenced by exactly
// one leaf, and every index is in range.  Counts go to refs[0..n_nodes) and
// refs[n_nodes..n_nodes+n_prims); bad indices set counters[C_ERR].
__global__ void k_validate_refs(const WideNode *__restrict__ nodes, uint32_t n_nodes, uint32_t n_prims,
		uint32_t *refs, uint32_t *counters) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_nodes) return;
	const WideNode nd = nodes[i];
	const uint32_t imask = nd.w[0].w >> 24;
	const uint32_t child_base = nd.w[1].x, tri_base = nd.w[1].y;
	uint32_t rank = 0;
	for (int s = 0; s < 8; ++s) {
		const uint32_t m = ((s < 4 ? nd.w[1].z : nd.w[1].w) >> ((s & 3) * 8)) & 0xffu;
		if (imask & (1u << s)) {
			const uint32_t c = child_base + rank++;
			if (c == 0 || c >= n_nodes) atomicOr(&counters[C_ERR], 4u);
			else atomicAdd(&refs[c], 1u);
		} else if (m) {
			const uint32_t cnt = __popc((m >> 5) & 7u), off = m & 31u;
			for (uint32_t k = 0; k < cnt; ++k) {
				const uint32_t t = tri_base + off + k;
				if (t >= n_prims) atomicOr(&counters[C_ERR], 8u);
				else atomicAdd(&refs[n_nodes + t], 1u);
			}
		}
	}
}

__global__ void k_validate_counts(const uint32_t *refs, uint32_t n_nodes, uint32_t n_prims, uint32_t *counters) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_nodes + n_prims) return;
	const uint32_t want = i == 0 ? 0u : 1u;
	if (refs[i] != want) atomicOr(&counters[C_ERR], 16u);
}

__global__ void k_init_collapse(uint2 *queue, uint32_t *counters) {
	queue[0] = make_uint2(counters[C_ROOT], 0u);
	counters[C_QA] = 1u;
	counters[C_QB] = 0u;
	counters[C_NODES] = 1u;
	counters[C_TRIS] = 0u;
}

__global__ void k_init_counters(uint32_t *counters) {
	const int i = threadIdx.x;
	if (i < C_COUNT) {
		uint32_t v = 0u;
		if (i >= C_BMIN && i < C_BMIN + 3) v = 0xffffffffu;
		if (i >= C_BMAX && i < C_BMAX + 3) v = 0u;
		counters[i] = v;
	}
}

// ---------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------

static inline uint32_t blocks_for(uint64_t n, uint32_t bs) { return (uint32_t)((n + bs - 1) / bs); }

lrx_status build_wide_bvh(uint32_t n, const float4 *d_lo, const float4 *d_hi, uint32_t leaf_max,
		uint32_t node_width, uint32_t treelet_passes, cudaStream_t st, BuildScratch &S, BvhResult *out) {
	if (node_width < 2 || node_width > 8) {
		set_error("node width must be in [2, 8]");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	*out = BvhResult();
	if (n == 0) return LRX_OK;
	if (leaf_max < 1) leaf_max = 1;
	if (leaf_max > 3) leaf_max = 3;
	lrx_status rc;
	const uint32_t ni = n > 1 ? n - 1 : 1;
	if ((rc = S.keys.alloc(sizeof(uint64_t) * n)) != LRX_OK) return rc;
	if ((rc = S.keys_alt.alloc(sizeof(uint64_t) * n)) != LRX_OK) return rc;
	if ((rc = S.vals.alloc(sizeof(uint32_t) * n)) != LRX_OK) return rc;
	if ((rc = S.vals_alt.alloc(sizeof(uint32_t) * n)) != LRX_OK) return rc;
	if ((rc = S.bnodes.alloc((sizeof(float4) * 2 + sizeof(uint32_t) * 2) * ni)) != LRX_OK) return rc;
	if ((rc = S.branges.alloc(sizeof(uint2) * ni)) != LRX_OK) return rc;
	if ((rc = S.treelet_scratch.alloc(sizeof(uint32_t) * ((size_t)n + ni))) != LRX_OK) return rc;
	if ((rc = S.other_bound.alloc(sizeof(uint32_t) * ni)) != LRX_OK) return rc;
	if ((rc = S.wide_nodes.alloc(sizeof(WideNode) * (size_t)n)) != LRX_OK) return rc;
	if ((rc = S.prim_order.alloc(sizeof(uint32_t) * n)) != LRX_OK) return rc;
	if ((rc = S.queue_a.alloc(sizeof(uint2) * n)) != LRX_OK) return rc;
	if ((rc = S.queue_b.alloc(sizeof(uint2) * n)) != LRX_OK) return rc;
	if ((rc = S.counters.alloc(sizeof(uint32_t) * 64)) != LRX_OK) return rc;

	uint32_t *counters = S.counters.as<uint32_t>();
	float4 *bn_lo = S.bnodes.as<float4>();
	float4 *bn_hi = bn_lo + ni;
	uint32_t *bchild = reinterpret_cast<uint32_t *>(bn_hi + ni);
	uint2 *bmeta = S.branges.as<uint2>();
	uint32_t *lparent = S.treelet_scratch.as<uint32_t>();
	float *sah = reinterpret_cast<float *>(lparent + n);

	k_init_counters<<<1, 32, 0, st>>>(counters);
	k_centroid_bounds<<<std::min(blocks_for(n, 256), 1024u), 256, 0, st>>>(n, d_lo, d_hi, counters);
	k_morton<<<blocks_for(n, 256), 256, 0, st>>>(n, d_lo, d_hi, counters, S.keys.as<uint64_t>(), S.vals.as<uint32_t>());
	LRX_CUDA(cudaGetLastError());

	cub::DoubleBuffer<uint64_t> dk(S.keys.as<uint64_t>(), S.keys_alt.as<uint64_t>());
	cub::DoubleBuffer<uint32_t> dv(S.vals.as<uint32_t>(), S.vals_alt.as<uint32_t>());
	size_t temp_bytes = 0;
	LRX_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, dk, dv, (int)n, 0, 63, st));
	if ((rc = S.cub_temp.alloc(temp_bytes)) != LRX_OK) return rc;
	LRX_CUDA(cub::DeviceRadixSort::SortPairs(S.cub_temp.ptr, temp_bytes, dk, dv, (int)n, 0, 63, st));
	const uint64_t *keys = dk.Current();
	const uint32_t *sorted = dv.Current();

	LRX_CUDA(cudaMemsetAsync(S.other_bound.ptr, 0xff, sizeof(uint32_t) * ni, st));
	LRX_CUDA(cudaMemsetAsync(bmeta, 0xff, sizeof(uint2) * ni, st));  // root's parent stays kNull
	k_hierarchy<<<blocks_for(n, 128), 128, 0, st>>>(n, keys, sorted, d_lo, d_hi, bchild, bn_lo, bn_hi, bmeta,
			lparent, S.other_bound.as<uint32_t>(), counters);
	LRX_CUDA(cudaGetLastError());

	// Treelet passes: pass k restructures subtrees of >= 7 * 2^k primitives.
	for (uint32_t pass = 0; n > 2 && pass < treelet_passes; ++pass) {
		LRX_CUDA(cudaMemsetAsync(S.other_bound.ptr, 0, sizeof(uint32_t) * ni, st));  // visit counters
		k_treelet<<<blocks_for(n, 128), 128, 0, st>>>(n, sorted, d_lo, d_hi, bchild, bn_lo, bn_hi, bmeta, lparent,
				sah, S.other_bound.as<uint32_t>(), leaf_max, 7u << std::min(pass, 20u));
		LRX_CUDA(cudaGetLastError());
	}

	// Which binary nodes become wide nodes (the SAH-optimal cover, above);
	// its tables live only for the collapse
	DevBuf wtab;
	const uint2 *wdec = nullptr;
	if (n > 1) {
		if ((rc = wtab.alloc((sizeof(float4) * 2 + sizeof(uint2)) * (size_t)ni)) != LRX_OK) return rc;
		float4 *wcost = wtab.as<float4>();
		uint2 *dec = reinterpret_cast<uint2 *>(wcost + 2 * (size_t)ni);
		LRX_CUDA(cudaMemsetAsync(S.other_bound.ptr, 0, sizeof(uint32_t) * ni, st));  // visit counters
		k_wide_cost<<<blocks_for(n, 128), 128, 0, st>>>(n, sorted, d_lo, d_hi, bchild, bn_lo, bn_hi, bmeta, lparent,
				S.other_bound.as<uint32_t>(), leaf_max, node_width, wcost, dec);
		LRX_CUDA(cudaGetLastError());
		wdec = dec;
	}

	// Level-synchronous collapse
	k_init_collapse<<<1, 1, 0, st>>>(S.queue_a.as<uint2>(), counters);
	LRX_CUDA(cudaGetLastError());
	uint2 *qin = S.queue_a.as<uint2>(), *qout = S.queue_b.as<uint2>();
	int cin = C_QA, cout = C_QB;
	uint32_t depth = 0;
	for (;;) {
		uint32_t n_in = 0;
		LRX_CUDA(cudaMemcpyAsync(&n_in, counters + cin, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
		LRX_CUDA(cudaStreamSynchronize(st));
		if (n_in == 0) break;
		if (n_in > n) {
			set_error("BVH collapse queue overflow");
			return LRX_ERR_BUILD;
		}
		++depth;
		if (depth > (uint32_t)kMaxTreeDepth) {
			// a restructured tree may be deeper than the stack allows: build the plain LBVH instead
			if (treelet_passes > 0) return build_wide_bvh(n, d_lo, d_hi, leaf_max, node_width, 0, st, S, out);
			set_error("BVH deeper than the traversal stack allows");
			return LRX_ERR_BUILD;
		}
		LRX_CUDA(cudaMemsetAsync(counters + cout, 0, sizeof(uint32_t), st));
		k_collapse<<<std::min(blocks_for(n_in, 128), 152u * 16u), 128, 0, st>>>(qin, counters + cin, qout,
				counters + cout, bchild, bn_lo, bn_hi, bmeta, sorted, d_lo, d_hi, leaf_max, node_width,
				S.wide_nodes.as<WideNode>(), S.prim_order.as<uint32_t>(), counters, n, wdec);
		LRX_CUDA(cudaGetLastError());
		std::swap(qin, qout);
		std::swap(cin, cout);
	}
	uint32_t host_counters[C_COUNT];
	LRX_CUDA(cudaMemcpyAsync(host_counters, counters, sizeof(host_counters), cudaMemcpyDeviceToHost, st));
	LRX_CUDA(cudaStreamSynchronize(st));
	if (host_counters[C_ERR] != 0 || host_counters[C_TRIS] != n) {
		set_error("BVH collapse lost primitives");
		return LRX_ERR_BUILD;
	}
	// Validate the structure before anyone traverses it.  The reference
	// counts reuse the (now idle) Morton key buffer.
	{
		const uint32_t n_nodes = host_counters[C_NODES];
		const size_t ref_bytes = sizeof(uint32_t) * ((size_t)n_nodes + n);
		if (ref_bytes > S.keys.bytes) {
			set_error("BVH validation scratch too small");
			return LRX_ERR_BUILD;
		}
		uint32_t *refs = S.keys.as<uint32_t>();
		LRX_CUDA(cudaMemsetAsync(refs, 0, ref_bytes, st));
		k_validate_refs<<<blocks_for(n_nodes, 256), 256, 0, st>>>(S.wide_nodes.as<WideNode>(), n_nodes, n, refs,
				counters);
		k_validate_counts<<<blocks_for((uint64_t)n_nodes + n, 256), 256, 0, st>>>(refs, n_nodes, n, counters);
		LRX_CUDA(cudaGetLastError());
		uint32_t err = 0;
		LRX_CUDA(cudaMemcpyAsync(&err, counters + C_ERR, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
		LRX_CUDA(cudaStreamSynchronize(st));
		if (err != 0) {
			set_error("BVH validation failed (code " + std::to_string(err) + ")");
			return LRX_ERR_BUILD;
		}
	}
	out->node_count = host_counters[C_NODES];
	out->depth = depth;
	std::memcpy(out->lo, &host_counters[C_BOX], 3 * sizeof(float));
	std::memcpy(out->hi, &host_counters[C_BOX + 3], 3 * sizeof(float));
	return LRX_OK;
}

// ---------------------------------------------------------------------------
// Scene assembly kernels
// ---------------------------------------------------------------------------

__global__ void k_triangle_boxes(uint32_t n, const float *__restrict__ v, const uint32_t *__restrict__ idx,
		float4 *__restrict__ lo, float4 *__restrict__ hi) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const uint32_t a = idx[3 * i], b = idx[3 * i + 1], c = idx[3 * i + 2];
	const float3 p0 = make_float3(v[3 * a], v[3 * a + 1], v[3 * a + 2]);
	const float3 p1 = make_float3(v[3 * b], v[3 * b + 1], v[3 * b + 2]);
	const float3 p2 = make_float3(v[3 * c], v[3 * c + 1], v[3 * c + 2]);
	float3 mn = make_float3(fminf(fminf(p0.x, p1.x), p2.x), fminf(fminf(p0.y, p1.y), p2.y), fminf(fminf(p0.z, p1.z), p2.z));
	float3 mx = make_float3(fmaxf(fmaxf(p0.x, p1.x), p2.x), fmaxf(fmaxf(p0.y, p1.y), p2.y), fmaxf(fmaxf(p0.z, p1.z), p2.z));
	// BVHAccel::Init leaf box: Expand(MachineEpsilon::E(bbox)) (bvhaccel.cpp:116-122)
	const float e = fmaxf(fmaxf(machine_eps(mn.x), fmaxf(machine_eps(mn.y), machine_eps(mn.z))),
			fmaxf(machine_eps(mx.x), fmaxf(machine_eps(mx.y), machine_eps(mx.z))));
	lo[i] = make_float4(__fsub_rd(mn.x, e), __fsub_rd(mn.y, e), __fsub_rd(mn.z, e), 0.f);
	hi[i] = make_float4(__fadd_ru(mx.x, e), __fadd_ru(mx.y, e), __fadd_ru(mx.z, e), 0.f);
}

lrx_status launch_triangle_boxes(uint32_t n_tris, const float *d_verts, const uint32_t *d_idx, float4 *d_lo,
		float4 *d_hi, cudaStream_t st) {
	if (!n_tris) return LRX_OK;
	k_triangle_boxes<<<blocks_for(n_tris, 256), 256, 0, st>>>(n_tris, d_verts, d_idx, d_lo, d_hi);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

__global__ void k_relocate(const WideNode *__restrict__ src, WideNode *__restrict__ dst, uint32_t n,
		uint32_t node_off, uint32_t tri_off) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	WideNode nd = src[i];
	nd.w[1].x += node_off;
	nd.w[1].y += tri_off;
	dst[i] = nd;
}

lrx_status launch_relocate_nodes(const WideNode *src, WideNode *dst, uint32_t n, uint32_t node_offset,
		uint32_t tri_offset, cudaStream_t st) {
	if (!n) return LRX_OK;
	k_relocate<<<blocks_for(n, 256), 256, 0, st>>>(src, dst, n, node_offset, tri_offset);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

// 80-byte record -> 64-byte record: the occupied slots (non-zero meta byte)
// in slot order, each with its meta byte and its six quantised planes.  The
// internal children keep their order, so child_base + rank still finds
// them; a node with more than 4 children sets *err.
__global__ void k_pack_nodes4(const WideNode *__restrict__ src, Node4 *__restrict__ dst, uint32_t n, uint32_t *err) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const WideNode nd = src[i];
	// per slot half (slots 0-3, 4-7): meta, then qlo x/y/z and qhi x/y/z
	const uint32_t word[7][2] = {{nd.w[1].z, nd.w[1].w}, {nd.w[2].x, nd.w[2].y}, {nd.w[2].z, nd.w[2].w},
			{nd.w[3].x, nd.w[3].y}, {nd.w[3].z, nd.w[3].w}, {nd.w[4].x, nd.w[4].y}, {nd.w[4].z, nd.w[4].w}};
	uint32_t packed[7] = {0, 0, 0, 0, 0, 0, 0};
	uint32_t p = 0;
	for (int s = 0; s < 8; ++s) {
		const uint32_t sh = (s & 3) * 8;
		if (!((word[0][s >> 2] >> sh) & 0xffu)) continue;  // empty slot
		if (p == 4) {
			atomicOr(err, 1u);
			return;
		}
		for (int k = 0; k < 7; ++k) packed[k] |= ((word[k][s >> 2] >> sh) & 0xffu) << (8 * p);
		++p;
	}
	Node4 o;
	o.w[0] = nd.w[0];
	o.w[1] = make_uint4(nd.w[1].x, nd.w[1].y, packed[0], packed[1]);
	o.w[2] = make_uint4(packed[2], packed[3], packed[4], packed[5]);
	o.w[3] = make_uint4(packed[6], 0u, 0u, 0u);
	dst[i] = o;
}

lrx_status pack_nodes4(const WideNode *src, Node4 *dst, uint32_t n, cudaStream_t st) {
	if (!n) return LRX_OK;
	DevBuf err;
	lrx_status rc;
	if ((rc = err.alloc(sizeof(uint32_t))) != LRX_OK) return rc;
	LRX_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(uint32_t), st));
	k_pack_nodes4<<<blocks_for(n, 256), 256, 0, st>>>(src, dst, n, err.as<uint32_t>());
	LRX_CUDA(cudaGetLastError());
	uint32_t h = 0;
	LRX_CUDA(cudaMemcpyAsync(&h, err.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	LRX_CUDA(cudaStreamSynchronize(st));
	if (h) {
		set_error("64-byte node records hold at most 4 children (build with node_width 4)");
		return LRX_ERR_BUILD;
	}
	return LRX_OK;
}

__global__ void k_triangle_records(uint32_t n, const uint32_t *__restrict__ order, const float *__restrict__ v,
		const uint32_t *__restrict__ idx, const uint32_t *__restrict__ tri_object, uint32_t object_const,
		TriRecord *__restrict__ dst) {
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	const uint32_t t = order[k];
	const uint32_t a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
	const float3 p0 = make_float3(v[3 * a], v[3 * a + 1], v[3 * a + 2]);
	const float3 p1 = make_float3(v[3 * b], v[3 * b + 1], v[3 * b + 2]);
	const float3 p2 = make_float3(v[3 * c], v[3 * c + 1], v[3 * c + 2]);
	const float3 e1 = rn_sub(p1, p0), e2 = rn_sub(p2, p0);
	uint32_t obj = object_const, tri = t;
	if (tri_object) {
		obj = tri_object[2 * t];
		tri = tri_object[2 * t + 1];
	}
	TriRecord r;
	r.a = make_float4(p0.x, p0.y, p0.z, __uint_as_float(tri));
	r.b = make_float4(e1.x, e1.y, e1.z, __uint_as_float(obj));
	r.c = make_float4(e2.x, e2.y, e2.z, 0.f);
	dst[k] = r;
}

lrx_status launch_triangle_records(uint32_t n_tris, const uint32_t *d_prim_order, const float *d_verts,
		const uint32_t *d_idx, const uint32_t *d_tri_object, uint32_t object_const, TriRecord *dst, cudaStream_t st) {
	if (!n_tris) return LRX_OK;
	k_triangle_records<<<blocks_for(n_tris, 256), 256, 0, st>>>(n_tris, d_prim_order, d_verts, d_idx, d_tri_object,
			object_const, dst);
	LRX_CUDA(cudaGetLastError());
	return LRX_OK;
}

}  // namespace lrx
