// CPU oracle for the LuxRays ray-intersection path -- TEST INFRASTRUCTURE.
//
// Restates the reference's CPU accelerators with the same FP32 operation
// order; compile with -O2 -ffp-contract=off (no FMA contraction, no fast
// math) so every product and sum rounds exactly as the reference's do.
// Only tests/, the smoke check and bench.py's CPU-baseline leg use it.
// Citations are file:line in the LuxCore source tree.

#include "lrx_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <pthread.h>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "lrx_oracle_motion.h"

namespace orc {

static const uint32_t NULL_INDEX = 0xffffffffu;

// -- L0 geometry: include/luxrays/core/geometry/{point,vector}.h ------------

struct V3 {
	float x, y, z;
	float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

static inline V3 sub(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 add(const V3 &a, const V3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
// vector.h:151-153
static inline float dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vector.h:159-163
static inline V3 cross(const V3 &a, const V3 &b) {
	return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}

// utils.h:145-161
template <class T> static inline T Max(T a, T b) { return a > b ? a : b; }
template <class T> static inline T Min(T a, T b) { return a < b ? a : b; }
template <class T> static inline T Clamp(T v, T lo, T hi) { return v > lo ? (v < hi ? v : hi) : lo; }

struct Ray {
	V3 o, d;
	float mint, maxt, time;
};

static inline Ray from_orc(const orc_ray &r) {
	Ray ray;
	ray.o = {r.o[0], r.o[1], r.o[2]};
	ray.d = {r.d[0], r.d[1], r.d[2]};
	ray.mint = r.mint;
	ray.maxt = r.maxt;
	ray.time = r.time;
	return ray;
}

// -- MachineEpsilon: include/luxrays/core/epsilon.h:50-94 -------------------

static inline float next_float(float v) {
	uint32_t i;
	std::memcpy(&i, &v, 4);
	i += 0x80u;  // DEFAULT_EPSILON_DISTANCE_FROM_VALUE, epsilon_types.cl:30
	std::memcpy(&v, &i, 4);
	return v;
}
static inline float eps(float v) {
	const float e = std::fabs(next_float(v) - v);
	return Clamp(e, 1e-5f, 1e-1f);  // DEFAULT_EPSILON_MIN/MAX, epsilon_types.cl:21-22
}
static inline float eps(const V3 &p) { return Max(eps(p.x), Max(eps(p.y), eps(p.z))); }

// -- BBox: include/luxrays/core/geometry/bbox.h, src/.../bbox.cpp -----------

struct BBox {
	V3 pMin{INFINITY, INFINITY, INFINITY};
	V3 pMax{-INFINITY, -INFINITY, -INFINITY};
	BBox() {}
	BBox(const V3 &p1, const V3 &p2) {
		pMin = {Min(p1.x, p2.x), Min(p1.y, p2.y), Min(p1.z, p2.z)};
		pMax = {Max(p1.x, p2.x), Max(p1.y, p2.y), Max(p1.z, p2.z)};
	}
	void expand(float delta) {  // bbox.h:80-83
		pMin = sub(pMin, V3{delta, delta, delta});
		pMax = add(pMax, V3{delta, delta, delta});
	}
};

// bbox.cpp:29-49
static inline BBox Union(const BBox &b, const V3 &p) {
	BBox r = b;
	r.pMin = {Min(b.pMin.x, p.x), Min(b.pMin.y, p.y), Min(b.pMin.z, p.z)};
	r.pMax = {Max(b.pMax.x, p.x), Max(b.pMax.y, p.y), Max(b.pMax.z, p.z)};
	return r;
}
static inline BBox Union(const BBox &b, const BBox &b2) {
	BBox r;
	r.pMin = {Min(b.pMin.x, b2.pMin.x), Min(b.pMin.y, b2.pMin.y), Min(b.pMin.z, b2.pMin.z)};
	r.pMax = {Max(b.pMax.x, b2.pMax.x), Max(b.pMax.y, b2.pMax.y), Max(b.pMax.z, b2.pMax.z)};
	return r;
}
static inline float eps(const BBox &b) { return Max(eps(b.pMin), eps(b.pMax)); }

// bbox.cpp:147-165
static inline bool bbox_intersectp(const Ray &ray, const float *pMin, const float *pMax) {
	float t0 = ray.mint, t1 = ray.maxt;
	for (int i = 0; i < 3; ++i) {
		const float invRayDir = 1.f / ray.d[i];
		float tNear = (pMin[i] - ray.o[i]) * invRayDir;
		float tFar = (pMax[i] - ray.o[i]) * invRayDir;
		if (tNear > tFar) std::swap(tNear, tFar);
		t0 = tNear > t0 ? tNear : t0;
		t1 = tFar < t1 ? tFar : t1;
		if (t0 > t1) return false;
	}
	return true;
}

// -- Triangle::Intersect: include/luxrays/core/geometry/triangle.h:55-89 ----

static inline bool tri_intersect(const Ray &ray, const V3 &p0, const V3 &p1, const V3 &p2,
		float *t, float *b1, float *b2) {
	const V3 e1 = sub(p1, p0);
	const V3 e2 = sub(p2, p0);
	const V3 s1 = cross(ray.d, e2);
	const float divisor = dot(s1, e1);
	if (divisor == 0.f) return false;
	const float invDivisor = 1.f / divisor;
	const V3 d = sub(ray.o, p0);
	*b1 = dot(d, s1) * invDivisor;
	if (*b1 < 0.f) return false;
	const V3 s2 = cross(d, e1);
	*b2 = dot(ray.d, s2) * invDivisor;
	if (*b2 < 0.f) return false;
	const float b0 = 1.f - *b1 - *b2;
	if (b0 < 0.f) return false;
	*t = dot(e2, s2) * invDivisor;
	if (*t < ray.mint || *t > ray.maxt) return false;
	return true;
}

// -- Matrix4x4 / Transform --------------------------------------------------

// matrix4x4.cpp:118-170 (Gauss-Jordan with full pivoting)
static bool matrix_inverse(const float m[4][4], float out[4][4]) {
	int indxc[4], indxr[4];
	int ipiv[4] = {0, 0, 0, 0};
	float minv[4][4];
	std::memcpy(minv, m, 16 * sizeof(float));
	for (int i = 0; i < 4; ++i) {
		int irow = -1, icol = -1;
		float big = 0.f;
		for (int j = 0; j < 4; ++j) {
			if (ipiv[j] != 1) {
				for (int k = 0; k < 4; ++k) {
					if (ipiv[k] == 0) {
						if (std::fabs(minv[j][k]) >= big) {
							big = std::fabs(minv[j][k]);
							irow = j;
							icol = k;
						}
					} else if (ipiv[k] > 1)
						return false;
				}
			}
		}
		if (icol < 0) return false;  // NaN entries: no pivot found
		++ipiv[icol];
		if (irow != icol)
			for (int k = 0; k < 4; ++k) std::swap(minv[irow][k], minv[icol][k]);
		indxr[i] = irow;
		indxc[i] = icol;
		if (minv[icol][icol] == 0.f) return false;
		const float pivinv = 1.f / minv[icol][icol];
		minv[icol][icol] = 1.f;
		for (int j = 0; j < 4; ++j) minv[icol][j] *= pivinv;
		for (int j = 0; j < 4; ++j) {
			if (j != icol) {
				const float save = minv[j][icol];
				minv[j][icol] = 0;
				for (int k = 0; k < 4; ++k) minv[j][k] -= minv[icol][k] * save;
			}
		}
	}
	for (int j = 3; j >= 0; --j) {
		if (indxr[j] != indxc[j])
			for (int k = 0; k < 4; ++k) std::swap(minv[k][indxr[j]], minv[k][indxc[j]]);
	}
	std::memcpy(out, minv, 16 * sizeof(float));
	return true;
}

// transform.h:130-142 / 144-156: point with the w divide skipped when w == 1
static inline V3 xform_point(const float m[4][4], const V3 &p) {
	const float x = p.x, y = p.y, z = p.z;
	V3 r{m[0][0] * x + m[0][1] * y + m[0][2] * z + m[0][3],
		m[1][0] * x + m[1][1] * y + m[1][2] * z + m[1][3],
		m[2][0] * x + m[2][1] * y + m[2][2] * z + m[2][3]};
	const float w = m[3][0] * x + m[3][1] * y + m[3][2] * z + m[3][3];
	if (w != 1.f) {
		const float inv = 1.f / w;  // point.h:100-103
		r = {inv * r.x, inv * r.y, inv * r.z};
	}
	return r;
}
// transform.h:186-193
static inline V3 xform_vector(const float m[4][4], const V3 &v) {
	const float x = v.x, y = v.y, z = v.z;
	return {m[0][0] * x + m[0][1] * y + m[0][2] * z,
		m[1][0] * x + m[1][1] * y + m[1][2] * z,
		m[2][0] * x + m[2][1] * y + m[2][2] * z};
}
// transform.h:271-280
static BBox xform_bbox(const float m[4][4], const BBox &b) {
	BBox r(xform_point(m, b.pMin), xform_point(m, b.pMax));
	r = Union(r, xform_point(m, V3{b.pMax.x, b.pMin.y, b.pMin.z}));
	r = Union(r, xform_point(m, V3{b.pMin.x, b.pMax.y, b.pMin.z}));
	r = Union(r, xform_point(m, V3{b.pMin.x, b.pMin.y, b.pMax.z}));
	r = Union(r, xform_point(m, V3{b.pMax.x, b.pMax.y, b.pMin.z}));
	r = Union(r, xform_point(m, V3{b.pMax.x, b.pMin.y, b.pMax.z}));
	r = Union(r, xform_point(m, V3{b.pMin.x, b.pMax.y, b.pMax.z}));
	return r;
}

// -- Classic BVH builder: src/luxrays/core/bvh/bvhclassicbuild.cpp ----------

struct Params {  // bvhaccel.cpp:49-70 defaults
	uint32_t treeType = 4;
	int costSamples = 0, isectCost = 80, traversalCost = 10;
	float emptyBonus = 0.5f;
};

struct TreeNode {  // bvhbuild.h:54-71
	BBox bbox;
	uint32_t a = 0, b = 0, c = 0, d = 0;  // triangleLeaf {meshIndex, triangleIndex} / bvhLeaf {leaf, transform, motion, meshOffset}
	TreeNode *leftChild = nullptr;
	TreeNode *rightSibling = nullptr;
};

static inline float ltf_key(const TreeNode *n, uint32_t axis) {  // bvhclassicbuild.cpp:36-46
	return n->bbox.pMax[axis] + n->bbox.pMin[axis];
}

// bvhclassicbuild.cpp:50-122
static void find_best_split(const Params &params, std::vector<TreeNode *> &list,
		uint32_t begin, uint32_t end, float *splitValue, uint32_t *bestAxis) {
	if (end - begin == 2) {
		*splitValue = (list[begin]->bbox.pMax[0] + list[begin]->bbox.pMin[0] +
				list[end - 1]->bbox.pMax[0] + list[end - 1]->bbox.pMin[0]) / 2;
		*bestAxis = 0;
		return;
	}
	V3 mean2{0, 0, 0}, var{0, 0, 0};
	for (uint32_t i = begin; i < end; i++)
		mean2 = add(mean2, add(list[i]->bbox.pMax, list[i]->bbox.pMin));
	{
		const float inv = 1.f / static_cast<float>(end - begin);  // point.h:105-110
		mean2 = {mean2.x * inv, mean2.y * inv, mean2.z * inv};
	}
	for (uint32_t i = begin; i < end; i++) {
		V3 v = sub(add(list[i]->bbox.pMax, list[i]->bbox.pMin), mean2);
		v.x *= v.x;
		v.y *= v.y;
		v.z *= v.z;
		var = add(var, v);
	}
	if (var.x > var.y && var.x > var.z) *bestAxis = 0;
	else if (var.y > var.z) *bestAxis = 1;
	else *bestAxis = 2;

	if (params.costSamples > 1) {
		BBox nodeBounds;
		for (uint32_t i = begin; i < end; i++) nodeBounds = Union(nodeBounds, list[i]->bbox);
		const V3 d = sub(nodeBounds.pMax, nodeBounds.pMin);
		auto area = [](const BBox &b) {  // bbox.h SurfaceArea
			const V3 e = sub(b.pMax, b.pMin);
			return 2.f * (e.x * e.y + e.x * e.z + e.y * e.z);
		};
		const float invTotalSA = 1.f / area(nodeBounds);
		const float increment = 2 * d[*bestAxis] / (params.costSamples + 1);
		float bestCost = INFINITY;
		for (float splitVal = 2 * nodeBounds.pMin[*bestAxis] + increment;
				splitVal < 2 * nodeBounds.pMax[*bestAxis]; splitVal += increment) {
			int nBelow = 0, nAbove = 0;
			BBox bbBelow, bbAbove;
			for (uint32_t j = begin; j < end; j++) {
				if ((list[j]->bbox.pMax[*bestAxis] + list[j]->bbox.pMin[*bestAxis]) < splitVal) {
					nBelow++;
					bbBelow = Union(bbBelow, list[j]->bbox);
				} else {
					nAbove++;
					bbAbove = Union(bbAbove, list[j]->bbox);
				}
			}
			const float pBelow = area(bbBelow) * invTotalSA;
			const float pAbove = area(bbAbove) * invTotalSA;
			const float eb = (nAbove == 0 || nBelow == 0) ? params.emptyBonus : 0.f;
			const float cost = params.traversalCost + params.isectCost * (1.f - eb) * (pBelow * nBelow + pAbove * nAbove);
			if (cost < bestCost) {
				bestCost = cost;
				*splitValue = splitVal;
			}
		}
	} else {
		*splitValue = mean2[*bestAxis];
	}
}

// bvhclassicbuild.cpp:124-181
static TreeNode *build_bvh(uint32_t *nNodes, const Params &params,
		std::vector<TreeNode *> &leafList, uint32_t begin, uint32_t end, uint32_t axis) {
	uint32_t splitAxis = axis;
	float splitValue = 0.f;

	*nNodes += 1;
	if (end - begin == 1) return new TreeNode(*leafList[begin]);

	TreeNode *parent = new TreeNode();
	std::vector<uint32_t> splits;
	splits.reserve(params.treeType + 1);
	splits.push_back(begin);
	splits.push_back(end);
	for (uint32_t i = 2; i <= params.treeType; i *= 2) {
		for (uint32_t j = 0, offset = 0; j + offset < i && splits.size() > j + 1; j += 2) {
			if (splits[j + 1] - splits[j] < 2) {
				j--;  // unsigned wrap is intended, as in the reference
				offset++;
				continue;
			}
			find_best_split(params, leafList, splits[j], splits[j + 1], &splitValue, &splitAxis);
			const uint32_t ax = splitAxis;
			const float sv = splitValue;
			auto it = std::partition(leafList.begin() + splits[j], leafList.begin() + splits[j + 1],
					[ax, sv](TreeNode *n) { return ltf_key(n, ax) < sv; });
			uint32_t middle = static_cast<uint32_t>(std::distance(leafList.begin(), it));
			middle = Max(splits[j] + 1, Min(splits[j + 1] - 1, middle));
			splits.insert(splits.begin() + j + 1, middle);
		}
	}

	TreeNode *child = build_bvh(nNodes, params, leafList, splits[0], splits[1], splitAxis);
	parent->leftChild = child;
	parent->bbox = child->bbox;
	TreeNode *lastChild = child;
	for (uint32_t i = 1; i < splits.size() - 1; i++) {
		child = build_bvh(nNodes, params, leafList, splits[i], splits[i + 1], splitAxis);
		lastChild->rightSibling = child;
		parent->bbox = Union(parent->bbox, child->bbox);
		lastChild = child;
	}
	return parent;
}

static void free_bvh(TreeNode *node) {
	while (node) {
		TreeNode *next = node->rightSibling;
		free_bvh(node->leftChild);
		delete node;
		node = next;
	}
}

// 32-B BVHArrayNode (bvhbuild_types.cl:21-42)
struct ArrayNode {
	union {
		struct { float bboxMin[3], bboxMax[3]; } bvhNode;
		struct { uint32_t v[3], meshIndex, triangleIndex; } triangleLeaf;
		struct { uint32_t leafIndex, transformIndex, motionIndex, meshOffsetIndex; } bvhLeaf;
	};
	uint32_t nodeData;
	int32_t pad0;
};
static_assert(sizeof(ArrayNode) == 32, "BVHArrayNode is 32 bytes");

struct Mesh {
	const V3 *verts;
	const uint32_t *tris;  // 3 per triangle, mesh-local
	uint32_t nVerts, nTris;
};

// bvhclassicbuild.cpp:183-220
static uint32_t build_bvh_array(const std::vector<const Mesh *> *meshes, TreeNode *node,
		uint32_t offset, ArrayNode *arr) {
	while (node) {
		ArrayNode *an = &arr[offset];
		if (node->leftChild) {
			std::memcpy(&an->bvhNode.bboxMin[0], &node->bbox.pMin, sizeof(float) * 3);
			std::memcpy(&an->bvhNode.bboxMax[0], &node->bbox.pMax, sizeof(float) * 3);
			offset = build_bvh_array(meshes, node->leftChild, offset + 1, arr);
			an->nodeData = offset;
		} else {
			if (meshes) {
				const Mesh *m = (*meshes)[node->a];
				const uint32_t *tri = &m->tris[3 * (size_t)node->b];
				an->triangleLeaf.v[0] = tri[0];
				an->triangleLeaf.v[1] = tri[1];
				an->triangleLeaf.v[2] = tri[2];
				an->triangleLeaf.meshIndex = node->a;
				an->triangleLeaf.triangleIndex = node->b;
			} else {
				an->bvhLeaf.leafIndex = node->a;
				an->bvhLeaf.transformIndex = node->b;
				an->bvhLeaf.motionIndex = node->c;
				an->bvhLeaf.meshOffsetIndex = node->d;
			}
			++offset;
			an->nodeData = offset | 0x80000000u;
		}
		an->pad0 = 0;
		node = node->rightSibling;
	}
	return offset;
}

static std::vector<ArrayNode> build_bvh_nodes(const Params &params,
		const std::vector<const Mesh *> *meshes, std::vector<TreeNode *> &leafList) {
	uint32_t nNodes = 0;
	TreeNode *root = build_bvh(&nNodes, params, leafList, 0, (uint32_t)leafList.size(), 2);
	std::vector<ArrayNode> arr(nNodes);
	build_bvh_array(meshes, root, 0, arr.data());
	free_bvh(root);
	return arr;
}

static inline bool is_leaf(uint32_t nodeData) { return (nodeData & 0x80000000u) != 0; }
static inline uint32_t skip_index(uint32_t nodeData) { return nodeData & 0x7fffffffu; }

// -- BVHAccel: src/luxrays/accelerators/bvhaccel.cpp ------------------------

struct BVHAccel {
	std::vector<const Mesh *> meshes;
	std::vector<ArrayNode> tree;
	uint64_t totalVertexCount = 0;

	// bvhaccel.cpp:72-168
	void init(const std::vector<const Mesh *> &ms, const Params &params) {
		meshes = ms;
		size_t total = 0;
		for (const Mesh *m : meshes) total += m->nTris, totalVertexCount += m->nVerts;
		if (total == 0) return;
		std::vector<TreeNode> bvNodes(total);
		std::vector<TreeNode *> bvList(total, nullptr);
		size_t idx = 0;
		for (uint32_t mi = 0; mi < meshes.size(); ++mi) {
			const Mesh *m = meshes[mi];
			for (uint32_t i = 0; i < m->nTris; ++i, ++idx) {
				TreeNode *node = &bvNodes[idx];
				const uint32_t *t = &m->tris[3 * (size_t)i];
				node->bbox = Union(BBox(m->verts[t[0]], m->verts[t[1]]), m->verts[t[2]]);
				node->bbox.expand(eps(node->bbox));
				node->a = mi;
				node->b = i;
				bvList[idx] = node;
			}
		}
		tree = build_bvh_nodes(params, &meshes, bvList);
	}

	// bvhaccel.cpp:170-260; `stats` counts node and leaf visits
	bool intersect(const Ray &initialRay, orc_hit *hit, uint64_t *nodeVisits = nullptr,
			uint64_t *leafVisits = nullptr) const {
		hit->t = initialRay.maxt;
		hit->meshIndex = NULL_INDEX;
		hit->triangleIndex = NULL_INDEX;
		hit->b1 = hit->b2 = 0.f;
		if (tree.empty()) return false;
		Ray ray = initialRay;
		uint32_t cur = 0;
		const uint32_t stop = skip_index(tree[0].nodeData);
		float t, b1, b2;
		while (cur < stop) {
			const ArrayNode &node = tree[cur];
			if (nodeVisits) ++*nodeVisits;
			const uint32_t nodeData = node.nodeData;
			if (is_leaf(nodeData)) {
				if (leafVisits) ++*leafVisits;
				const Mesh *m = meshes[node.triangleLeaf.meshIndex];
				const V3 p0 = m->verts[node.triangleLeaf.v[0]];
				const V3 p1 = m->verts[node.triangleLeaf.v[1]];
				const V3 p2 = m->verts[node.triangleLeaf.v[2]];
				if (tri_intersect(ray, p0, p1, p2, &t, &b1, &b2)) {
					if (t < hit->t) {
						ray.maxt = t;
						hit->t = t;
						hit->b1 = b1;
						hit->b2 = b2;
						hit->meshIndex = node.triangleLeaf.meshIndex;
						hit->triangleIndex = node.triangleLeaf.triangleIndex;
					}
				}
				++cur;
			} else {
				if (bbox_intersectp(ray, node.bvhNode.bboxMin, node.bvhNode.bboxMax)) ++cur;
				else cur = nodeData;
			}
		}
		return hit->meshIndex != NULL_INDEX;
	}
};

// -- MBVHAccel: src/luxrays/accelerators/mbvhaccel.cpp ----------------------

struct Object {
	uint32_t mesh;
	bool instance;
	float m[4][4], mInv[4][4];
	int motion = -1;  // index of the object's MotionSystem (a MotionTriangleMesh), else -1
};

// MotionSystem::Bound / InterpolatedTransform::Bound (motionsystem.cpp:74-86,
// :356-365) with storingGlobal2Local: every sampled world->local matrix is
// inverted and the box transformed by it.
static BBox motion_bound(const orc_motion::MotionSystem &ms, const BBox &ibox) {
	BBox result;
	for (const orc_motion::InterpolatedTransform &it : ms.interpolatedTransforms) {
		BBox tbox;
		const float N = 1024.f;
		for (float i = 0; i <= N; ++i) {
			const float t = orc_motion::Lerp(i / N, it.startTime, it.endTime);
			float m[4][4], inv[4][4];
			it.Sample(t, m);
			if (!matrix_inverse(m, inv)) throw std::runtime_error("Singular matrix in motion bound");
			tbox = Union(tbox, xform_bbox(inv, ibox));
		}
		result = Union(result, tbox);
	}
	return result;
}

struct MBVHAccel {
	const std::vector<Object> *objects = nullptr;
	const std::vector<Mesh> *meshes = nullptr;
	const std::vector<orc_motion::MotionSystem> *motions = nullptr;
	std::vector<BVHAccel> uniqueLeafs;
	std::vector<std::vector<const Mesh *>> leafMeshLists;
	std::vector<uint32_t> uniqueLeafsTransform;  // object index of each transform
	std::vector<uint32_t> uniqueLeafsMotionSystem;  // object index of each motion system
	std::vector<ArrayNode> root;

	// trianglemesh.cpp:72-83 and :241-248
	BBox object_bbox(const Object &o) const {
		const Mesh &m = (*meshes)[o.mesh];
		BBox b;
		for (uint32_t i = 0; i < m.nVerts; ++i) b = Union(b, m.verts[i]);
		if (o.instance) b = xform_bbox(o.m, b);
		else if (o.motion >= 0) b = motion_bound((*motions)[o.motion], b);  // trianglemesh.cpp:268-275
		return b;
	}

	// mbvhaccel.cpp:58-216
	void init(const std::vector<Object> &objs, const std::vector<Mesh> &ms,
			const std::vector<orc_motion::MotionSystem> &mss, const Params &params) {
		objects = &objs;
		meshes = &ms;
		motions = &mss;
		size_t totalTris = 0;
		for (const Object &o : objs) totalTris += ms[o.mesh].nTris;
		if (totalTris == 0) return;
		const uint32_t nLeafs = (uint32_t)objs.size();
		std::vector<uint32_t> leafsIndex, leafsTransformIndex, leafsMotionSystemIndex;
		std::map<uint32_t, uint32_t> uniqueLeafIndexByMesh;
		uniqueLeafs.reserve(nLeafs);
		leafMeshLists.reserve(nLeafs);
		for (uint32_t i = 0; i < nLeafs; ++i) {
			const Object &o = objs[i];
			if (!o.instance && o.motion < 0) {
				const uint32_t u = (uint32_t)uniqueLeafs.size();
				leafMeshLists.push_back({&ms[o.mesh]});
				uniqueLeafs.emplace_back();
				uniqueLeafs.back().init(leafMeshLists.back(), params);
				uniqueLeafIndexByMesh[o.mesh] = u;
				leafsIndex.push_back(u);
				leafsTransformIndex.push_back(NULL_INDEX);
				leafsMotionSystemIndex.push_back(NULL_INDEX);
			} else {
				auto it = uniqueLeafIndexByMesh.find(o.mesh);
				if (it == uniqueLeafIndexByMesh.end()) {
					const uint32_t u = (uint32_t)uniqueLeafs.size();
					leafMeshLists.push_back({&ms[o.mesh]});
					uniqueLeafs.emplace_back();
					uniqueLeafs.back().init(leafMeshLists.back(), params);
					uniqueLeafIndexByMesh[o.mesh] = u;
					leafsIndex.push_back(u);
				} else {
					leafsIndex.push_back(it->second);
				}
				if (o.instance) {
					leafsTransformIndex.push_back((uint32_t)uniqueLeafsTransform.size());
					uniqueLeafsTransform.push_back(i);
					leafsMotionSystemIndex.push_back(NULL_INDEX);
				} else {
					leafsTransformIndex.push_back(NULL_INDEX);
					leafsMotionSystemIndex.push_back((uint32_t)uniqueLeafsMotionSystem.size());
					uniqueLeafsMotionSystem.push_back(i);
				}
			}
		}
		// leafMeshLists must not reallocate after init() captured pointers
		for (size_t k = 0; k < uniqueLeafs.size(); ++k) uniqueLeafs[k].meshes = leafMeshLists[k];

		std::vector<TreeNode> bvhLeafs(nLeafs);
		std::vector<TreeNode *> bvhLeafsList(nLeafs, nullptr);
		for (uint32_t i = 0; i < nLeafs; ++i) {
			TreeNode *l = &bvhLeafs[i];
			l->bbox = object_bbox(objs[i]);
			l->bbox.expand(eps(l->bbox));
			l->a = leafsIndex[i];
			l->b = leafsTransformIndex[i];
			l->c = leafsMotionSystemIndex[i];
			l->d = i;
			bvhLeafsList[i] = l;
		}
		root = build_bvh_nodes(params, nullptr, bvhLeafsList);
	}

	// transform.h:259-262 via mbvhaccel.cpp:324-327; a motion leaf applies
	// its system's Sample(ray.time) (matrix4x4op.h:80-82)
	Ray local_ray(const Ray &ray, uint32_t transformIndex, uint32_t motionIndex) const {
		Ray r = ray;
		if (transformIndex != NULL_INDEX) {
			const Object &o = (*objects)[uniqueLeafsTransform[transformIndex]];
			r.o = xform_point(o.mInv, ray.o);
			r.d = xform_vector(o.mInv, ray.d);
		} else if (motionIndex != NULL_INDEX) {
			const Object &o = (*objects)[uniqueLeafsMotionSystem[motionIndex]];
			float m[4][4];
			(*motions)[o.motion].Sample(ray.time, m);
			r.o = xform_point(m, ray.o);
			r.d = xform_vector(m, ray.d);
		}
		return r;
	}

	// mbvhaccel.cpp:252-357
	bool intersect(const Ray &ray, orc_hit *hit) const {
		hit->t = ray.maxt;
		hit->meshIndex = NULL_INDEX;
		hit->triangleIndex = NULL_INDEX;
		hit->b1 = hit->b2 = 0.f;
		if (root.empty()) return false;

		bool insideLeafTree = false;
		uint32_t currentRootNode = 0;
		const uint32_t rootStopNode = skip_index(root[0].nodeData);
		uint32_t currentNode = currentRootNode;
		uint32_t currentStopNode = rootStopNode;
		uint32_t currentMeshOffset = 0;
		const ArrayNode *currentTree = root.data();
		const BVHAccel *currentLeaf = nullptr;
		Ray currentRay = ray;

		for (;;) {
			if (currentNode >= currentStopNode) {
				if (insideLeafTree) {
					currentTree = root.data();
					currentNode = currentRootNode;
					currentStopNode = rootStopNode;
					currentRay = ray;
					currentRay.maxt = hit->t;
					insideLeafTree = false;
					if (currentNode >= currentStopNode) break;
				} else {
					break;
				}
			}
			const ArrayNode &node = currentTree[currentNode];
			const uint32_t nodeData = node.nodeData;
			if (is_leaf(nodeData)) {
				if (insideLeafTree) {
					const uint32_t absoluteMeshIndex = node.triangleLeaf.meshIndex + currentMeshOffset;
					const Mesh *m = currentLeaf->meshes[node.triangleLeaf.meshIndex];
					const V3 p0 = m->verts[node.triangleLeaf.v[0]];
					const V3 p1 = m->verts[node.triangleLeaf.v[1]];
					const V3 p2 = m->verts[node.triangleLeaf.v[2]];
					float t, b1, b2;
					if (tri_intersect(currentRay, p0, p1, p2, &t, &b1, &b2)) {
						if (t < hit->t) {
							currentRay.maxt = t;
							hit->t = t;
							hit->b1 = b1;
							hit->b2 = b2;
							hit->meshIndex = absoluteMeshIndex;
							hit->triangleIndex = node.triangleLeaf.triangleIndex;
						}
					}
					++currentNode;
				} else {
					currentLeaf = &uniqueLeafs[node.bvhLeaf.leafIndex];
					currentTree = currentLeaf->tree.data();
					currentRay = local_ray(ray, node.bvhLeaf.transformIndex, node.bvhLeaf.motionIndex);
					currentRay.maxt = hit->t;
					currentMeshOffset = node.bvhLeaf.meshOffsetIndex;
					currentRootNode = currentNode + 1;
					currentNode = 0;
					currentStopNode = currentLeaf->tree.empty() ? 0 : skip_index(currentTree[0].nodeData);
					insideLeafTree = true;
				}
			} else {
				if (bbox_intersectp(currentRay, node.bvhNode.bboxMin, node.bvhNode.bboxMax)) ++currentNode;
				else currentNode = nodeData;
			}
		}
		return hit->meshIndex != NULL_INDEX;
	}
};

// -- Scene wrapper ----------------------------------------------------------

struct Scene {
	std::vector<V3> verts;
	std::vector<uint32_t> tris;
	std::vector<Mesh> meshes;
	std::vector<Object> objects;
	std::vector<orc_motion::MotionSystem> motions;
	int accel = ORC_ACCEL_BVH;
	BVHAccel bvh;
	std::vector<const Mesh *> bvhMeshes;
	MBVHAccel mbvh;
	Params params;

	bool intersect(const Ray &r, orc_hit *h) const {
		return accel == ORC_ACCEL_BVH ? bvh.intersect(r, h) : mbvh.intersect(r, h);
	}

	// Ray in the local space of object `oi`, as MBVHAccel::Intersect forms it
	Ray object_ray(const Ray &r, uint32_t oi) const {
		const Object &o = objects[oi];
		Ray lr = r;
		if (o.instance) {
			lr.o = xform_point(o.mInv, r.o);
			lr.d = xform_vector(o.mInv, r.d);
		} else if (o.motion >= 0) {
			float m[4][4];
			motions[o.motion].Sample(r.time, m);
			lr.o = xform_point(m, r.o);
			lr.d = xform_vector(m, r.d);
		}
		return lr;
	}
};

template <class F>
static void parallel_for(uint64_t n, int nThreads, F fn) {
	if (nThreads <= 0) nThreads = (int)std::max(1u, std::thread::hardware_concurrency());
	if ((uint64_t)nThreads > n) nThreads = (int)std::max<uint64_t>(1, n);
	if (nThreads == 1) {
		fn(0, n);
		return;
	}
	std::vector<std::thread> th;
	const uint64_t chunk = (n + nThreads - 1) / nThreads;
	for (int i = 0; i < nThreads; ++i) {
		const uint64_t b = i * chunk, e = std::min<uint64_t>(n, b + chunk);
		if (b >= e) break;
		th.emplace_back([=]() { fn(b, e); });
	}
	for (auto &t : th) t.join();
}

// Runs `fn` on a thread with a large stack: the classic builder and its
// flattening recurse once per tree level.
template <class F>
static void run_big_stack(F fn) {
	struct Ctx { F *f; std::string err; };
	Ctx ctx{&fn, {}};
	pthread_attr_t attr;
	pthread_attr_init(&attr);
	pthread_attr_setstacksize(&attr, (size_t)1 << 30);
	pthread_t tid;
	auto entry = [](void *p) -> void * {
		Ctx *c = (Ctx *)p;
		try {
			(*c->f)();
		} catch (const std::exception &e) {
			c->err = e.what();
		}
		return nullptr;
	};
	if (pthread_create(&tid, &attr, entry, &ctx) != 0) {
		pthread_attr_destroy(&attr);
		fn();
		return;
	}
	pthread_join(tid, nullptr);
	pthread_attr_destroy(&attr);
	if (!ctx.err.empty()) throw std::runtime_error(ctx.err);
}

}  // namespace orc

using namespace orc;

extern "C" {

void *orc_scene_create(const float *verts, const uint64_t *vert_offsets,
		const uint32_t *tris, const uint64_t *tri_offsets, uint32_t n_meshes,
		const orc_object *objs, uint32_t n_objs, int accel, int tree_type,
		char *err, uint64_t err_len) {
	return orc_scene_create_motion(verts, vert_offsets, tris, tri_offsets, n_meshes, objs, n_objs,
			nullptr, 0, accel, tree_type, err, err_len);
}

void *orc_scene_create_motion(const float *verts, const uint64_t *vert_offsets,
		const uint32_t *tris, const uint64_t *tri_offsets, uint32_t n_meshes,
		const orc_object *objs, uint32_t n_objs, const orc_motion_desc *mds, uint32_t n_motions,
		int accel, int tree_type, char *err, uint64_t err_len) {
	auto fail = [&](const std::string &msg) -> void * {
		if (err && err_len) std::snprintf(err, err_len, "%s", msg.c_str());
		return nullptr;
	};
	try {
		Scene *s = new Scene();
		s->accel = accel;
		s->params.treeType = tree_type <= 2 ? 2 : (tree_type <= 4 ? 4 : 8);  // bvhaccel.cpp:59-62
		const uint64_t nv = vert_offsets[n_meshes], nt = tri_offsets[n_meshes];
		s->verts.resize(nv);
		if (nv) std::memcpy(s->verts.data(), verts, nv * 12);
		s->tris.assign(tris, tris + 3 * nt);
		s->meshes.resize(n_meshes);
		for (uint32_t i = 0; i < n_meshes; ++i) {
			Mesh &m = s->meshes[i];
			m.verts = s->verts.data() + vert_offsets[i];
			m.tris = s->tris.data() + 3 * tri_offsets[i];
			m.nVerts = (uint32_t)(vert_offsets[i + 1] - vert_offsets[i]);
			m.nTris = (uint32_t)(tri_offsets[i + 1] - tri_offsets[i]);
			for (uint64_t k = 0; k < 3ull * m.nTris; ++k)
				if (m.tris[k] >= m.nVerts) { delete s; return fail("vertex index out of range"); }
		}
		const uint32_t no = objs ? n_objs : n_meshes;
		s->objects.resize(no);
		for (uint32_t i = 0; i < no; ++i) {
			Object &o = s->objects[i];
			if (objs) {
				o.mesh = objs[i].mesh;
				o.instance = objs[i].has_transform != 0;
				std::memcpy(o.m, objs[i].m, 64);
			} else {
				o.mesh = i;
				o.instance = false;
			}
			if (o.mesh >= n_meshes) { delete s; return fail("object mesh index out of range"); }
			if (o.instance && !matrix_inverse(o.m, o.mInv)) { delete s; return fail("singular instance transform"); }
		}
		for (uint32_t k = 0; k < n_motions; ++k) {
			const orc_motion_desc &md = mds[k];
			if (md.object >= no || md.count == 0) { delete s; return fail("bad motion object or keyframe count"); }
			Object &o = s->objects[md.object];
			if (o.motion >= 0) { delete s; return fail("object has two motion systems"); }
			std::vector<float> times(md.times, md.times + md.count);
			std::vector<const float (*)[4]> mats;
			for (uint32_t j = 0; j < md.count; ++j) mats.push_back(reinterpret_cast<const float (*)[4]>(md.transforms + 16ull * j));
			s->motions.emplace_back(times, mats);  // throws on a singular keyframe
			o.instance = false;
			o.motion = (int)s->motions.size() - 1;
		}
		run_big_stack([&]() {
			if (accel == ORC_ACCEL_BVH) {
				for (const Object &o : s->objects) {
					if (o.instance || o.motion >= 0) throw std::runtime_error("BVH accelerator does not support instances");
					s->bvhMeshes.push_back(&s->meshes[o.mesh]);
				}
				s->bvh.init(s->bvhMeshes, s->params);
			} else {
				s->mbvh.init(s->objects, s->meshes, s->motions, s->params);
			}
		});
		return s;
	} catch (const std::exception &e) {
		return fail(e.what());
	}
}

void orc_scene_destroy(void *scene) { delete (Scene *)scene; }

double orc_intersect(void *scene, const orc_ray *rays, orc_hit *hits, uint64_t n, int n_threads) {
	const Scene *s = (const Scene *)scene;
	const auto t0 = std::chrono::steady_clock::now();
	parallel_for(n, n_threads, [&](uint64_t b, uint64_t e) {
		for (uint64_t i = b; i < e; ++i) s->intersect(from_orc(rays[i]), &hits[i]);
	});
	return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void orc_brute_force(void *scene, const orc_ray *rays, orc_hit *hits, uint64_t n, int n_threads) {
	const Scene *s = (const Scene *)scene;
	parallel_for(n, n_threads, [&](uint64_t b, uint64_t e) {
		for (uint64_t i = b; i < e; ++i) {
			const Ray r0 = from_orc(rays[i]);
			orc_hit &h = hits[i];
			h.t = r0.maxt;
			h.b1 = h.b2 = 0.f;
			h.meshIndex = h.triangleIndex = NULL_INDEX;
			for (uint32_t oi = 0; oi < s->objects.size(); ++oi) {
				const Mesh &m = s->meshes[s->objects[oi].mesh];
				Ray r = s->object_ray(r0, oi);
				for (uint32_t ti = 0; ti < m.nTris; ++ti) {
					const uint32_t *t3 = &m.tris[3 * (size_t)ti];
					r.maxt = h.t;
					float t, b1, b2;
					if (tri_intersect(r, m.verts[t3[0]], m.verts[t3[1]], m.verts[t3[2]], &t, &b1, &b2) && t < h.t) {
						h.t = t;
						h.b1 = b1;
						h.b2 = b2;
						h.meshIndex = oi;
						h.triangleIndex = ti;
					}
				}
			}
		}
	});
}

int orc_triangle_hit(void *scene, const orc_ray *ray, uint32_t meshIndex,
		uint32_t triangleIndex, float *t, float *b1, float *b2) {
	const Scene *s = (const Scene *)scene;
	if (meshIndex >= s->objects.size()) return 0;
	const Mesh &m = s->meshes[s->objects[meshIndex].mesh];
	if (triangleIndex >= m.nTris) return 0;
	const Ray r = s->object_ray(from_orc(*ray), meshIndex);
	const uint32_t *t3 = &m.tris[3 * (size_t)triangleIndex];
	return tri_intersect(r, m.verts[t3[0]], m.verts[t3[1]], m.verts[t3[2]], t, b1, b2) ? 1 : 0;
}

uint64_t orc_bvh_node_count(void *scene) {
	const Scene *s = (const Scene *)scene;
	return s->accel == ORC_ACCEL_BVH ? s->bvh.tree.size() : 0;
}

void orc_bvh_nodes(void *scene, orc_bvh_node *out) {
	const Scene *s = (const Scene *)scene;
	if (s->accel != ORC_ACCEL_BVH) return;
	// bvhaccelhw.cpp:45-160: vertex indices rebased onto the concatenated vertex array
	std::vector<uint32_t> vbase(s->bvhMeshes.size());
	uint32_t acc = 0;
	for (size_t i = 0; i < s->bvhMeshes.size(); ++i) vbase[i] = acc, acc += s->bvhMeshes[i]->nVerts;
	for (size_t i = 0; i < s->bvh.tree.size(); ++i) {
		ArrayNode n = s->bvh.tree[i];
		if (is_leaf(n.nodeData))
			for (int k = 0; k < 3; ++k) n.triangleLeaf.v[k] += vbase[n.triangleLeaf.meshIndex];
		std::memcpy(&out[i], &n, 32);
	}
}

int orc_mbvh_export(void *scene, uint64_t counts[4], orc_bvh_node *nodes, float *verts, float *mats,
		uint32_t *motion_ranges, orc_interval *intervals) {
	const Scene *s = (const Scene *)scene;
	if (s->accel != ORC_ACCEL_MBVH) return 0;
	const MBVHAccel &mb = s->mbvh;
	// mbvhaccelhw.cpp:64-128 / :308-440 (one page): root nodes, then every
	// unique leaf's nodes; leaf-tree vertex indices rebased onto the
	// concatenated vertex array, skip indices and root leaf references onto
	// the concatenated node array
	std::vector<uint32_t> leafNodeOffset, leafVertOffset;
	uint64_t nn = mb.root.size(), nv = 0;
	for (const BVHAccel &l : mb.uniqueLeafs) {
		leafNodeOffset.push_back((uint32_t)nn);
		leafVertOffset.push_back((uint32_t)nv);
		nn += l.tree.size();
		for (const Mesh *m : l.meshes) nv += m->nVerts;
	}
	uint64_t nits = 0;
	for (uint32_t oi : mb.uniqueLeafsMotionSystem)
		nits += (*mb.motions)[(*mb.objects)[oi].motion].interpolatedTransforms.size();
	const uint64_t want[4] = {nn, nv, mb.uniqueLeafsTransform.size(), mb.uniqueLeafsMotionSystem.size()};
	if (!nodes) {
		std::memcpy(counts, want, sizeof(want));
		counts[3] |= nits << 32;
		return 1;
	}
	uint64_t k = 0;
	for (ArrayNode n : mb.root) {
		if (is_leaf(n.nodeData)) n.bvhLeaf.leafIndex = leafNodeOffset[n.bvhLeaf.leafIndex];
		std::memcpy(&nodes[k++], &n, 32);
	}
	for (size_t li = 0; li < mb.uniqueLeafs.size(); ++li) {
		const BVHAccel &l = mb.uniqueLeafs[li];
		for (ArrayNode n : l.tree) {
			if (is_leaf(n.nodeData)) {
				uint32_t vb = leafVertOffset[li];
				for (uint32_t mi = 0; mi < n.triangleLeaf.meshIndex; ++mi) vb += l.meshes[mi]->nVerts;
				for (int j = 0; j < 3; ++j) n.triangleLeaf.v[j] += vb;
			} else {
				n.nodeData = skip_index(n.nodeData) + leafNodeOffset[li];
			}
			std::memcpy(&nodes[k++], &n, 32);
		}
		for (const Mesh *m : l.meshes) {
			std::memcpy(verts, m->verts, 12ull * m->nVerts);
			verts += 3ull * m->nVerts;
		}
	}
	// mbvhaccelhw.cpp:142-151: each transform leaf gets Transform::mInv
	for (uint32_t oi : mb.uniqueLeafsTransform) {
		std::memcpy(mats, (*mb.objects)[oi].mInv, 64);
		mats += 16;
	}
	// mbvhaccelhw.cpp:154-191: every InterpolatedTransform of each motion system
	uint32_t first = 0;
	for (uint32_t oi : mb.uniqueLeafsMotionSystem) {
		const orc_motion::MotionSystem &ms = (*mb.motions)[(*mb.objects)[oi].motion];
		*motion_ranges++ = first;
		*motion_ranges++ = first + (uint32_t)ms.interpolatedTransforms.size() - 1;
		first += (uint32_t)ms.interpolatedTransforms.size();
		for (const orc_motion::InterpolatedTransform &it : ms.interpolatedTransforms) {
			orc_interval &o = *intervals++;
			std::memset(&o, 0, sizeof(o));
			o.startTime = it.startTime;
			o.endTime = it.endTime;
			std::memcpy(o.start, it.start, 64);
			std::memcpy(o.end, it.end, 64);
			const orc_motion::Decomposed *d[2] = {&it.startT, &it.endT};
			for (int e = 0; e < 2; ++e) {
				std::memcpy(o.R[e], d[e]->R, 64);
				const float st[6] = {d[e]->Sx, d[e]->Sy, d[e]->Sz, d[e]->Tx, d[e]->Ty, d[e]->Tz};
				std::memcpy(o.ST[e], st, sizeof(st));
			}
			const orc_motion::Quaternion *q[2] = {&it.startQ, &it.endQ};
			for (int e = 0; e < 2; ++e) {
				const float wq[4] = {q[e]->w, q[e]->v.x, q[e]->v.y, q[e]->v.z};
				std::memcpy(o.Q[e], wq, 16);
			}
			o.has[0] = it.hasRotation;
			o.has[1] = it.hasTranslation;
			o.has[2] = it.hasScale;
			o.has[3] = it.hasTranslationX;
			o.has[4] = it.hasTranslationY;
			o.has[5] = it.hasTranslationZ;
			o.has[6] = it.hasScaleX;
			o.has[7] = it.hasScaleY;
			o.has[8] = it.hasScaleZ;
			o.has[9] = it.isActive;
		}
	}
	return 1;
}

void orc_visit_stats(void *scene, const orc_ray *rays, uint64_t n,
		double *nodes_per_ray, double *leaves_per_ray) {
	const Scene *s = (const Scene *)scene;
	uint64_t nodes = 0, leaves = 0;
	if (s->accel == ORC_ACCEL_BVH) {
		for (uint64_t i = 0; i < n; ++i) {
			orc_hit h;
			s->bvh.intersect(from_orc(rays[i]), &h, &nodes, &leaves);
		}
	}
	*nodes_per_ray = n ? (double)nodes / n : 0.0;
	*leaves_per_ray = n ? (double)leaves / n : 0.0;
}

int orc_matrix_inverse(const float *m, float *out) {
	float a[4][4], r[4][4];
	std::memcpy(a, m, 64);
	if (!matrix_inverse(a, r)) return 0;
	std::memcpy(out, r, 64);
	return 1;
}

float orc_machine_epsilon(float v) { return eps(v); }

}  // extern "C"
