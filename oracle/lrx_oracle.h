/*
 * CPU oracle for the LuxRays ray-intersection path -- TEST INFRASTRUCTURE.
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check in __graft_entry__.py and the CPU-baseline leg of bench.py load it.
 * It restates, in plain C++ with FP32 arithmetic and no FMA contraction, the
 * reference's own CPU accelerators:
 *   - Triangle::Intersect        include/luxrays/core/geometry/triangle.h:55-89
 *   - BBox::IntersectP           src/luxrays/core/geometry/bbox.cpp:147-165
 *   - MachineEpsilon::E          include/luxrays/core/epsilon.h:50-94
 *   - classic BVH builder        src/luxrays/core/bvh/bvhclassicbuild.cpp:51-233
 *   - BVHAccel::Init/Intersect   src/luxrays/accelerators/bvhaccel.cpp:72-260
 *   - MBVHAccel::Init/Intersect  src/luxrays/accelerators/mbvhaccel.cpp:58-357
 *   - Matrix4x4::Inverse         src/luxrays/core/geometry/matrix4x4.cpp:118-170
 *   - Transform * Point/Vector/Ray/BBox  include/luxrays/core/geometry/transform.h:144-290
 *   - TriangleMesh/InstanceTriangleMesh::GetBBox  src/luxrays/core/trianglemesh.cpp:72-83,241-248
 *
 * Parity pin: the restated triangle test and skip-list walk are checked
 * against the reference's own OpenCL kernel text (bvh.cl, triangle_funcs.cl,
 * bbox_funcs.cl) compiled for the CPU by oracle/build_ref.sh into
 * oracle/_ref/; the golden vectors under tests/golden/ were produced by that
 * compiled reference code (tests/golden/make_golden.py).
 */
#ifndef LRX_ORACLE_H
#define LRX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* luxrays::Ray (48 B) and luxrays::RayHit (20 B), ray_types.cl:24-36 */
typedef struct {
	float o[3], d[3];
	float mint, maxt, time;
	uint32_t flags;
	float pad[2];
} orc_ray;

typedef struct {
	float t, b1, b2;
	uint32_t meshIndex, triangleIndex;
} orc_hit;

/* One DataSet entry: a plain TriangleMesh (has_transform == 0) or an
 * InstanceTriangleMesh of mesh `mesh` with local-to-world matrix m
 * (row-major Matrix4x4). */
typedef struct {
	uint32_t mesh;
	uint32_t has_transform;
	float m[16];
} orc_object;

/* 32-B BVHArrayNode, bvhbuild_types.cl:21-42 */
typedef struct {
	uint32_t w[6];
	uint32_t nodeData;
	int32_t pad0;
} orc_bvh_node;

enum { ORC_ACCEL_BVH = 0, ORC_ACCEL_MBVH = 1 };

/* Build a scene. verts: all meshes' xyz concatenated; vert_offsets /
 * tri_offsets: n_meshes+1 prefix offsets (in vertices / triangles);
 * tris: per-mesh-local vertex indices. objs == NULL means one plain object
 * per mesh. Returns NULL and fills err on failure. */
void *orc_scene_create(const float *verts, const uint64_t *vert_offsets,
		const uint32_t *tris, const uint64_t *tri_offsets, uint32_t n_meshes,
		const orc_object *objs, uint32_t n_objs, int accel, int tree_type,
		char *err, uint64_t err_len);
/* As orc_scene_create, with motion systems: motion k makes object
 * mds[k].object a MotionTriangleMesh of its mesh whose MotionSystem has
 * mds[k].count keyframes (times, row-major world->local matrices, 16 floats
 * each). The object's has_transform is ignored. */
typedef struct {
	uint32_t object, count;
	const float *times;
	const float *transforms;
} orc_motion_desc;
void *orc_scene_create_motion(const float *verts, const uint64_t *vert_offsets,
		const uint32_t *tris, const uint64_t *tri_offsets, uint32_t n_meshes,
		const orc_object *objs, uint32_t n_objs, const orc_motion_desc *mds, uint32_t n_motions,
		int accel, int tree_type, char *err, uint64_t err_len);
void orc_scene_destroy(void *scene);

/* Accelerator::Intersect over a ray array, split across n_threads
 * std::threads (0 = hardware concurrency). Returns the elapsed seconds. */
double orc_intersect(void *scene, const orc_ray *rays, orc_hit *hits,
		uint64_t n, int n_threads);

/* Closest hit by testing every triangle of every object with the same
 * Triangle::Intersect (ties: lowest (meshIndex, triangleIndex)). */
void orc_brute_force(void *scene, const orc_ray *rays, orc_hit *hits,
		uint64_t n, int n_threads);

/* Triangle::Intersect of one ray against one (meshIndex, triangleIndex) of
 * the DataSet, in that object's local space (instances: ray transformed by
 * the inverse transform exactly as MBVHAccel::Intersect does). Returns 1 on a
 * hit inside [mint, maxt]. */
int orc_triangle_hit(void *scene, const orc_ray *ray, uint32_t meshIndex,
		uint32_t triangleIndex, float *t, float *b1, float *b2);

/* Node count and a copy of the flattened BVHArrayNode[] of a BVH scene (the
 * layout the reference's GPU kernel reads; vertex indices are rebased to the
 * concatenated vertex array as bvhaccelhw.cpp:45-160 does). */
uint64_t orc_bvh_node_count(void *scene);
void orc_bvh_nodes(void *scene, orc_bvh_node *out);

/* One InterpolatedTransform of a motion system, as the oracle decomposed it
 * (motionsystem.cpp:36-72): times, start/end matrices, per end the rotation
 * matrix R, scales and translations (Sx Sy Sz Tx Ty Tz) and the quaternion
 * (w x y z), then the flags hasRotation, hasTranslation, hasScale,
 * hasTranslationX/Y/Z, hasScaleX/Y/Z, isActive. */
typedef struct {
	float startTime, endTime;
	float start[16], end[16];
	float R[2][16];
	float ST[2][6];
	float Q[2][4];
	int32_t has[10];
} orc_interval;

/* An MBVH scene in the layout MBVHKernel uploads (mbvhaccelhw.cpp:64-191,
 * :308-440, one page): nodes (root tree then every unique leaf's tree,
 * rebased), the concatenated vertices, one world->local matrix per
 * transform leaf, [first, last] interval indices per motion leaf, and the
 * intervals.  With nodes == NULL fills counts = {nodes, vertices,
 * matrices, motion systems | intervals << 32}.  Returns 0 for a BVH scene. */
int orc_mbvh_export(void *scene, uint64_t counts[4], orc_bvh_node *nodes, float *verts, float *mats,
		uint32_t *motion_ranges, orc_interval *intervals);

/* Mean number of BVHArrayNode visits per ray of BVHAccel::Intersect, and of
 * leaf (triangle) visits, over the given rays (the reference-layout byte
 * accounting). */
void orc_visit_stats(void *scene, const orc_ray *rays, uint64_t n,
		double *nodes_per_ray, double *leaves_per_ray);

/* Matrix4x4::Inverse of a row-major 4x4; returns 0 if singular. */
int orc_matrix_inverse(const float *m, float *out);

/* MachineEpsilon::E(float) */
float orc_machine_epsilon(float v);

#ifdef __cplusplus
}
#endif

#endif
