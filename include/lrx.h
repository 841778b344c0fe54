/*
 * lrx -- GB300 ray-intersection engine for the LuxRays data-parallel path.
 *
 * C ABI of liblrx.so: plain pointers, sizes and status codes; no C++ or
 * CUDA types cross it (a CUDA stream is passed as `void *`, a device buffer
 * as a `void *` device address).  Every entry point is thread-safe per
 * scene, returns an lrx_status and never throws.
 *
 * Data formats are LuxRays' own:
 *   lrx_ray  == luxrays::Ray    (48 B)  include/luxrays/core/geometry/ray.h:35-103,
 *                                       ray_types.cl:24-31
 *   lrx_hit  == luxrays::RayHit (20 B)  ray.h:93-103, ray_types.cl:33-36
 * A miss is meshIndex == LRX_NULL_INDEX with t = the ray's maxt
 * (bvh.cl:219-223); rays with LRX_RAY_FLAGS_MASKED set are skipped and their
 * hit is not written (bvh.cl:243-244).
 */
#ifndef LRX_H
#define LRX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LRX_ABI_VERSION 4u
#define LRX_NULL_INDEX 0xffffffffu      /* luxrays_types.cl:21 */
#define LRX_RAY_FLAGS_MASKED 0x1u       /* ray_types.cl:22 */

typedef struct lrx_ray {
	float o[3], d[3];
	float mint, maxt, time;
	uint32_t flags;
	float pad[2];
} lrx_ray;

typedef struct lrx_hit {
	float t, b1, b2;
	uint32_t meshIndex, triangleIndex;
} lrx_hit;

typedef enum lrx_status {
	LRX_OK = 0,
	LRX_ERR_INVALID_ARGUMENT = 1,  /* bad pointer, size, alignment or index */
	LRX_ERR_CUDA = 2,              /* a CUDA runtime call failed */
	LRX_ERR_OUT_OF_MEMORY = 3,     /* device allocation failed */
	LRX_ERR_BUILD = 4,             /* BVH build failed (e.g. depth limit) */
	LRX_ERR_DEVICE = 5,            /* a kernel reported a fault in the status word */
	LRX_ERR_NOT_SUPPORTED = 6,     /* e.g. no sm_103 device */
	LRX_ERR_BUDGET = 7,            /* serving: request exceeds the HBM budget */
	LRX_ERR_BUSY = 8,              /* serving: queue full */
	LRX_ERR_TIMEOUT = 9            /* host wait limit reached */
} lrx_status;

/* Trace modes (lrx_trace `mode`). */
#define LRX_TRACE_CLOSEST 0u  /* closest hit, ties broken by lowest (meshIndex, triangleIndex) */
#define LRX_TRACE_ANY 1u      /* any hit in [mint, maxt] (shadow rays) */

/* One TriangleMesh: FP32 xyz vertices and u32 vertex-index triples, host
 * memory owned by the caller (trianglemesh.h:79-201).  The library copies
 * them to the device during lrx_scene_create. */
typedef struct lrx_mesh_desc {
	const float *vertices;
	const uint32_t *triangles;
	uint32_t vertex_count;
	uint32_t triangle_count;
} lrx_mesh_desc;

#define LRX_OBJECT_INSTANCE 0x1u     /* InstanceTriangleMesh: use transform */
#define LRX_OBJECT_HAS_INVERSE 0x2u  /* inverse supplied (Transform::mInv) */

/* One DataSet entry (dataset.cpp:66-81).  Its position in the object array
 * is the meshIndex reported in hits.  A plain object (flags == 0) is the
 * mesh in world space; an instance (trianglemesh.h:203-305) is the mesh under
 * the row-major local-to-world `transform` (Transform::m).  Without
 * LRX_OBJECT_HAS_INVERSE the inverse is Matrix4x4::Inverse of `transform`
 * (matrix4x4.cpp:118-170), as Transform's constructor computes it. */
typedef struct lrx_object_desc {
	uint32_t mesh;
	uint32_t flags;
	float transform[16];
	float inverse[16];
} lrx_object_desc;

typedef struct lrx_build_opts {
	uint32_t struct_size;    /* sizeof(lrx_build_opts) */
	uint32_t leaf_max;       /* triangles per leaf, 1..3 (default 3) */
	uint32_t treelet_passes; /* treelet SAH restructuring passes (default 2, 0 = plain LBVH) */
	uint32_t node_width;     /* children per wide node, 4..8 (0 = 8); narrower nodes give deeper
	                            trees, by default in the same 80-byte node record */
	/* Added in ABI 4 (a caller passing the 16-byte struct of ABI 1-3 gets
	   LRX_NODES_WIDE8): */
	uint32_t node_layout;    /* LRX_NODES_* -- the node record the scene's tree is stored in */
} lrx_build_opts;

/* Node records (lrx_build_opts.node_layout).  The 80-byte record holds up to
   8 children; the 64-byte record up to 4 -- a quarter less to fetch per
   visit and half the slab tests, for trees of node_width 4 over flat scenes
   (a scene with objects, two-level, keeps the 80-byte record and is
   rejected with LRX_ERR_NOT_SUPPORTED).  lrx_scene_create_autotuned times
   both on its sample. */
#define LRX_NODES_WIDE8 0u
#define LRX_NODES_COMPACT4 1u

typedef struct lrx_scene lrx_scene;

typedef struct lrx_scene_info {
	uint64_t triangle_count;       /* effective triangles (instances counted per instance) */
	uint64_t unique_triangle_count;
	uint32_t object_count;
	uint32_t instance_count;
	uint32_t blas_count;
	uint32_t two_level;
	uint64_t node_count;           /* wide nodes, all levels */
	uint64_t device_bytes;         /* device memory held by the scene */
	uint32_t max_depth;            /* deepest wide-node path */
	uint32_t node_bytes;           /* bytes per node record: 80, or 64 (LRX_NODES_COMPACT4; ABI 4) */
	double build_ms;               /* device build time (excludes host->device copy) */
} lrx_scene_info;

/* ABI version of the loaded library (LRX_ABI_VERSION). */
uint32_t lrx_abi_version(void);

/* Last error message of the calling thread ("" if none). */
const char *lrx_last_error(void);

/* Builds a scene on the current CUDA device: uploads the meshes and builds
 * one BVH per unique mesh plus, when instances are present, a top-level BVH
 * over the objects.  objects == NULL means one plain object per mesh.
 * Replaces: luxrays::Accelerator::Init (include/luxrays/core/accelerator.h:51)
 * together with the device upload in the BVHKernel / MBVHKernel constructors
 * (src/luxrays/accelerators/bvhaccelhw.cpp:38-240,
 * src/luxrays/accelerators/mbvhaccelhw.cpp:41-440). */
lrx_status lrx_scene_create(const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count,
		const lrx_build_opts *opts, void *stream, lrx_scene **out_scene);

/* The motion system of one motion-blurred instance: `count` keyframes with
 * strictly increasing times and row-major 4x4 matrices in the convention of
 * the reference's MotionTriangleMesh -- the motion system MBVHAccel samples
 * at the ray's time and applies to the ray (world to the mesh's local
 * space, mbvhaccel.cpp:326-327).  The object it names must be an instance;
 * its `transform` is then not used. */
typedef struct lrx_motion_desc {
	uint32_t object;          /* index into the objects array */
	uint32_t count;           /* keyframes, >= 1 */
	const float *times;       /* count times */
	const float *transforms;  /* count x 16 floats */
} lrx_motion_desc;

/* lrx_scene_create with motion-blurred instances: each ray is traced against
 * the instance transform interpolated at its `time` (translation and scale
 * lerped, rotation slerped between decomposed keyframes), and the instance's
 * box in the top-level BVH is its swept bound.
 * Replaces: MBVHAccel::Init / Intersect with MotionTriangleMesh leaves
 * (mbvhaccel.cpp:145-172, 323-328) and MotionSystem / InterpolatedTransform
 * (src/luxrays/core/geometry/motionsystem.cpp:33-345). */
lrx_status lrx_scene_create_motion(const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count,
		const lrx_motion_desc *motions, uint32_t motion_count,
		const lrx_build_opts *opts, void *stream, lrx_scene **out_scene);

/* Frees the scene's device memory (Accelerator destructor). */
lrx_status lrx_scene_destroy(lrx_scene *scene);

/* Re-reads the instance transforms of an existing scene (same object list,
 * same meshes) and rebuilds only the top-level BVH.
 * Replaces: luxrays::Accelerator::Update (accelerator.h:52-53),
 * MBVHAccel::Update (mbvhaccel.cpp:237-250) and
 * HardwareIntersectionKernel::Update (hardwareintersectiondevice.h:66),
 * MBVHKernel::Update (mbvhaccelhw.cpp:442-466). */
lrx_status lrx_scene_update_instances(lrx_scene *scene,
		const lrx_object_desc *objects, uint32_t object_count, void *stream);

lrx_status lrx_scene_get_info(const lrx_scene *scene, lrx_scene_info *info);

/* Traces `count` rays already resident in device memory (16-B aligned
 * lrx_ray array) into a device lrx_hit array, asynchronously on `stream`
 * (NULL = legacy default stream, as the reference's cuLaunchKernel on
 * stream 0).
 * Replaces: HardwareIntersectionKernel::EnqueueTraceRayBuffer
 * (include/luxrays/core/hardwareintersectiondevice.h:67-68), i.e.
 * BVHKernel / MBVHKernel::EnqueueTraceRayBuffer
 * (bvhaccelhw.cpp:259-268, mbvhaccelhw.cpp:468-477). */
lrx_status lrx_trace(lrx_scene *scene, const void *d_rays, void *d_hits,
		uint32_t count, uint32_t mode, void *stream);

/* Same as lrx_trace for rays and hits in HOST memory: copies the rays in,
 * traces, copies the hits out and synchronises `stream`.  Staging buffers
 * are allocated on first use and kept by the scene.  Batches of more than
 * 524,288 rays go through lrx_trace_host_batches (chunks whose copies
 * overlap each other's traces).
 * Replaces: the serial IntersectionDevice::TraceRay loop
 * (include/luxrays/core/intersectiondevice.h:65-68) for batches. */
lrx_status lrx_trace_host(lrx_scene *scene, const lrx_ray *h_rays, lrx_hit *h_hits,
		uint32_t count, uint32_t mode, void *stream);

/* One batch of lrx_trace_host_batches: host rays and hits, as lrx_trace_host. */
typedef struct lrx_host_batch {
	lrx_scene *scene;
	const lrx_ray *h_rays;
	lrx_hit *h_hits;
	uint32_t count;
	uint32_t mode;     /* LRX_TRACE_CLOSEST or LRX_TRACE_ANY */
} lrx_host_batch;

/* lrx_trace_host over several batches whose copies and traces overlap: the
 * batches, largest first, are cut into chunks of at most 524,288 rays, and each chunk is
 * copied in, traced (its scene's lrx_trace path, except that a configuration
 * with LRX_VARIANT_SORT_RAYS runs persistent warps on the chunk instead: the
 * chunks are traced side by side, and a sort of each gains less than it
 * costs) and copied out on a side stream (up to 4, round robin, forked from
 * `stream`), so one chunk's copies run while another is traced.  Returns once every hit is in host memory
 * (`stream` synchronised).  Page-locked host buffers let the copies run
 * asynchronously.  Masked rays keep the caller's hit contents: a mapped
 * (page-locked) hit buffer is not copied in -- only its masked slots are
 * read back after the trace -- while other hit buffers are copied in first.
 * Staging comes from a stream-ordered pool (allocated on first use, kept).
 * Replaces: a sequence of IntersectionDevice::TraceRay-style host batches
 * (include/luxrays/core/intersectiondevice.h:65-68) -- no reference counterpart
 * overlaps them. */
lrx_status lrx_trace_host_batches(const lrx_host_batch *batches, uint32_t batch_count, void *stream);

/* Traversal launch configuration of a scene (what the autotuner chooses). */
typedef struct lrx_trace_config {
	uint32_t struct_size;     /* sizeof(lrx_trace_config) */
	uint32_t block_size;      /* threads per block: a multiple of 32 in [32, 512] (0 = 128) */
	uint32_t postpone;        /* leaf triangles are tested only while at least this many lanes
	                             of the warp test triangles; otherwise they are deferred while
	                             node work remains (0 = never defer) */
	uint32_t variant;         /* LRX_VARIANT_* bits */
	uint32_t modes;           /* set: which trace modes take this config (bit 0 closest,
	                             bit 1 any-hit; 0 = both).  get: bit 1 set reads the any-hit one */
	uint32_t refill;          /* with LRX_VARIANT_PERSISTENT: idle lanes of a warp that trigger
	                             its next ray claim, 1-32 (0 = 16).  Added in ABI 2: a caller
	                             passing the 20-byte ABI 1 struct gets 0 */
	/* Failure bounds (added in ABI 3; a caller passing an older, shorter
	 * struct gets 0 for both).  A ray that reaches either is abandoned: its
	 * hit is not written and the scene's status word records why
	 * (lrx_scene_device_status). */
	uint32_t max_visits;      /* node visits per ray.  0 = the scene's own bound, which no
	                             valid tree reaches: the node count of its top-level tree
	                             (the whole BVH of a flat scene), plus the node count of the
	                             largest instanced BVH at each instance entry */
	uint32_t deadline_us;     /* launch deadline in microseconds, from the launch's first
	                             block: rays not yet started when it has passed are abandoned.
	                             0 = 10 s plus 0.1 us per ray of the launch */
} lrx_trace_config;
#define LRX_VARIANT_MINMAX3 0x1u       /* 3-input min/max in the slab tests */
#define LRX_VARIANT_SCENE_L2_KEEP 0x2u /* node/triangle loads marked evict-last in L2 */
#define LRX_VARIANT_STREAM_RAYS 0x4u   /* ray loads / hit stores marked evict-first */
#define LRX_VARIANT_OCCUPANCY 0x8u     /* register budget for 20 blocks of 64 threads per SM (blocks <= 64) */
#define LRX_VARIANT_SORT_RAYS 0x10u    /* reorder batches of >= 32768 rays by direction octant and
                                          origin before tracing (hits stay in caller order) */
#define LRX_VARIANT_SORT_OCTANT 0x20u  /* with SORT_RAYS: key on the direction octant only
                                          (one radix pass, caller order kept within an octant) */
#define LRX_VARIANT_PERSISTENT 0x40u   /* persistent warps claim rays from a device counter
                                          (ballot + shuffle) and refill idle lanes; blocks <= 128 */
#define LRX_VARIANT_SMEM_STACK 0x80u   /* top 8 traversal-stack entries per ray in shared memory
                                          (deeper entries in local memory) */
#define LRX_VARIANT_COMPACT 0x100u     /* with PERSISTENT: compact the indices of the unmasked rays
                                          first (stable) and trace only those -- for wavefront
                                          buffers where finished paths leave masked rays */
#define LRX_VARIANT_SMEM_STACK16 0x400u /* the top 16 traversal-stack entries in shared memory
                                          (ABI 3; blocks <= 256) */
#define LRX_VARIANT_SMEM_STACK32 0x800u /* the top 32 entries in shared memory (ABI 3; blocks <= 128);
                                          with either, deeper entries stay in local memory */
#define LRX_VARIANT_DRAIN_SPLIT 0x2000u /* with PERSISTENT, closest hit (not on scenes with
                                          motion instances): once the launch's rays are all
                                          claimed, a warp's idle lanes take pending subtrees of
                                          its remaining rays and merge their hits back (results
                                          unchanged; the stack stays in local memory and MINMAX3
                                          is not used; ABI 4) */

/* Sets / reads the launch configuration lrx_trace uses for this scene.
 * No reference counterpart (the reference fixes 32-thread blocks,
 * bvhaccelhw.cpp:259-268). */
lrx_status lrx_scene_set_trace_config(lrx_scene *scene, const lrx_trace_config *config);
lrx_status lrx_scene_get_trace_config(const lrx_scene *scene, lrx_trace_config *config);

/* Autotuner: traces the sample batch (device rays) under each candidate
 * launch configuration -- block size {32, 64, 128} x postpone {0, 8} x
 * variant {none, streaming ray access, ray sort, persistent (refill 8),
 * persistent + streaming, persistent + shared-memory stack top, persistent +
 * L2-resident scene}, and for closest hit the persistent shapes with a
 * local-memory stack also with the drain split -- keeps the fastest for
 * `mode` in the scene and returns it in `chosen` (nullable).  Synchronises
 * `stream`; do not trace the same scene from other threads meanwhile.
 * No reference counterpart (the reference fixes its launch shape). */
lrx_status lrx_scene_autotune(lrx_scene *scene, const void *d_sample_rays, uint32_t count, uint32_t mode,
		void *stream, lrx_trace_config *chosen);

/* Builds the scene under each candidate build -- node width {8, 4} x
 * triangles per leaf {3, 2}, and for flat scenes also the 4-wide trees in
 * the 64-byte node record (LRX_NODES_COMPACT4), with opts' treelet passes
 * (opts nullable: 2) -- autotunes each candidate's launch configuration for
 * `mode` on the sample rays (lrx_scene_autotune), and keeps the candidate
 * whose tuned configuration traces the sample fastest; the others are
 * destroyed.  chosen_opts / chosen_config (nullable) receive the kept build
 * options (as many bytes as chosen_opts->struct_size holds, at least the
 * 16 bytes of ABI 1-3) and launch configuration.  Synchronises `stream`.
 * Closest-hit results do not depend on the choice (ties go to the lowest
 * index in every tree).
 * No reference counterpart (the reference builds one fixed tree). */
lrx_status lrx_scene_create_autotuned(const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count, const lrx_build_opts *opts,
		const void *d_sample_rays, uint32_t sample_count, uint32_t mode, void *stream,
		lrx_scene **out_scene, lrx_build_opts *chosen_opts, lrx_trace_config *chosen_config);

/* One ray batch of a multi-batch call (device buffers, as for lrx_trace). */
typedef struct lrx_batch {
	lrx_scene *scene;
	const void *d_rays;
	void *d_hits;
	uint32_t count;
	uint32_t mode;     /* LRX_TRACE_CLOSEST or LRX_TRACE_ANY */
} lrx_batch;

/* Traces many ray batches -- any mix of scenes (on one device) and modes --
 * with one launch of a persistent queue kernel per 384 batches, so small and
 * uneven batches share the GPU instead of each paying a launch and a tail.
 * When any batch's scene config for its mode has LRX_VARIANT_PERSISTENT (the
 * closest-hit default), the batches form one ray index space and persistent
 * warps claim rays from it with ballot/shuffle, refilling idle lanes (a
 * warp's lanes may then hold rays of different batches); otherwise 64-thread
 * blocks claim 64-ray tiles.  Batches whose scene config has
 * LRX_VARIANT_SORT_RAYS and at least 32,768 rays are reordered first (one
 * radix sort per launch).  When a call holds at most 4 batches of 131,072
 * rays or more (a wavefront's camera, bounce and shadow buffers), those --
 * and any batch on a scene with motion-blurred instances -- are traced by
 * launches of their own (the scene's lrx_trace path) on side streams forked
 * from `stream` and joined back into it, so they run beside each other and
 * beside the queue launch (the side streams are the calling thread's own,
 * created by its first such call, which belongs outside a graph capture).  Results
 * equal lrx_trace on each batch.  Asynchronous on `stream`; graph-capturable (no host synchronisation; the
 * sort scratch is stream-ordered pool memory).
 * Replaces: a sequence of HardwareIntersectionKernel::EnqueueTraceRayBuffer
 * calls (hardwareintersectiondevice.h:67-68), one per RayBuffer. */
lrx_status lrx_trace_batches(const lrx_batch *batches, uint32_t batch_count, void *stream);

/* lrx_trace_batches with a completion notice per batch: d_done_flags[k] is
 * set to 1 (after the batch's hits are written and fenced system-wide) as
 * soon as batch k is finished, while other batches of the launch may still
 * run -- the flags may live in host-mapped memory and be polled by the host.
 * The caller zeroes the flags; d_tile_counters (batch_count words of device
 * memory) is scratch -- per-batch progress -- that the call zeroes on `stream`.  Flags of empty batches
 * are not written.  No reference counterpart. */
lrx_status lrx_trace_batches_ex(const lrx_batch *batches, uint32_t batch_count, void *stream,
		uint32_t *d_tile_counters, uint32_t *d_done_flags);

/* ------------------------------------------------------------------------
 * Serving: many render sessions submit ray batches against registered scenes;
 * one server per device keeps scenes resident under an HBM budget (least
 * recently used scenes with no work in flight are evicted and rebuilt on
 * demand) and runs a continuous-batching loop: whenever one of its streams
 * is free, every admitted pending request is launched together through the
 * queue kernel, so requests arriving while others run overlap them on the
 * device.  No reference counterpart (the reference traces one RayBuffer per
 * call on stream 0, pathoclopenclthread.cpp:185).
 * ------------------------------------------------------------------------ */
typedef struct lrx_server lrx_server;

#define LRX_SERVE_BATCHED 0u  /* continuous batching over `streams` streams (default) */
#define LRX_SERVE_PLAIN 1u    /* one lrx_trace per request, FIFO on one stream (comparison) */

typedef struct lrx_server_opts {
	uint32_t struct_size;      /* sizeof(lrx_server_opts) */
	uint32_t policy;           /* LRX_SERVE_* */
	uint64_t budget_bytes;     /* device memory for resident scenes (0 = unlimited) */
	uint32_t streams;          /* concurrent launches in flight (0 = 4) */
	uint32_t max_requests_per_launch;  /* (0 = 384) */
	uint64_t host_cache_bytes; /* host memory for blobs of evicted scenes, reloaded instead of rebuilt
	                              (0 = 16 GiB; UINT64_MAX = no cache).  Added in ABI 2: the 24-byte
	                              ABI 1 struct is accepted and gets the default */
	uint64_t max_rays_per_launch; /* batched policy: a launch takes pending requests (oldest first)
	                              until their rays reach this many; a single larger request still
	                              gets a launch of its own (0 = 2,097,152; UINT64_MAX = no cap).
	                              Bounds the work queued ahead of a launch's last request when
	                              requests arrive faster than they are served.  Added in ABI 4:
	                              the 32-byte struct of ABI 2-3 is accepted and gets the default */
} lrx_server_opts;

typedef struct lrx_server_stats {
	uint64_t requests_done, rays_done;
	uint64_t requests_failed;
	uint64_t scene_builds, scene_evictions;
	uint64_t resident_bytes, peak_resident_bytes;
	uint64_t launches;
	double latency_p50_us, latency_p99_us, latency_mean_us, latency_max_us;
	double busy_seconds;       /* wall time from the first submit to the last completion */
	uint64_t scene_reloads;    /* admissions served from the blob cache instead of a build (ABI 2) */
	uint64_t host_cache_bytes; /* blobs held (ABI 2) */
} lrx_server_stats;

lrx_status lrx_server_create(const lrx_server_opts *opts, lrx_server **out_server);
/* Waits for in-flight work, frees every resident scene and stops the worker. */
lrx_status lrx_server_destroy(lrx_server *server);
/* Registers a scene (arguments as lrx_scene_create); the server keeps a host
 * copy so it can rebuild the scene after an eviction.  Not built until used. */
lrx_status lrx_server_add_scene(lrx_server *server, const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count, uint32_t *out_scene_id);
/* Queues a ray batch (device buffers that stay valid until the request
 * completes); returns at once with a ticket. */
lrx_status lrx_server_submit(lrx_server *server, uint32_t scene_id, const void *d_rays, void *d_hits,
		uint32_t count, uint32_t mode, uint64_t *out_ticket);
/* Waits up to timeout_ms for a ticket: LRX_OK when its hits are written,
 * LRX_ERR_TIMEOUT if still running, or the error that failed it. */
lrx_status lrx_server_wait(lrx_server *server, uint64_t ticket, uint32_t timeout_ms);
lrx_status lrx_server_get_stats(lrx_server *server, lrx_server_stats *stats);
lrx_status lrx_server_reset_stats(lrx_server *server);

/* Largest batch lrx_trace_host_noalloc accepts (its fixed staging area). */
#define LRX_NOALLOC_MAX_RAYS 131072u

/* lrx_trace_host without any device allocation.  This entry point has no
 * counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc or cudaFree.  One example is
 * a host loop that shares the GPU with other work in flight: cudaFree can
 * synchronise the whole device and stall that work, and lrx_trace_host grows
 * its staging buffers with cudaMalloc/cudaFree when a larger batch arrives.
 * Another is an application that owns all device memory through its own
 * fixed pool or budget and allows no allocation outside it.
 *
 * Instead of allocating, the rays, the hits and the launch's scratch (the ray
 * sort's keys, indices and temporary storage for any-hit batches of 32,768
 * rays or more, or the index list of a compacting configuration) live in one
 * array that the library reserves statically on every GPU that loads it:
 * room for LRX_NOALLOC_MAX_RAYS rays and hits plus 4 MiB of scratch
 * (12.5 MiB), held until the process exits.  A batch larger than
 * LRX_NOALLOC_MAX_RAYS is rejected with LRX_ERR_INVALID_ARGUMENT.  The scene's
 * launch configuration for the mode applies unchanged, so results are the
 * same as lrx_trace_host's for the same scene and rays.
 *
 * The first call on a device looks up the array's device address (one
 * cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  Every call on a device shares the array and it
 * keeps the last call's contents; nothing in it needs to start at zero:
 * each call copies its rays and the caller's hit buffer in before the kernel
 * runs, the sort writes its keys and indices before reading them, and the
 * sort's temporary storage is initialised by the sort itself.  Calls whose
 * GPU work overlapped would race on the array, so the library serialises
 * these calls per device, and each one synchronises `stream` before it
 * returns, on success and on failure alike. */
lrx_status lrx_trace_host_noalloc(lrx_scene *scene, const lrx_ray *h_rays, lrx_hit *h_hits,
		uint32_t count, uint32_t mode, void *stream);

/* Like lrx_trace, and also accumulates per-ray traversal counters into
 * d_counters[4] (u64: wide nodes fetched, triangles tested, instances
 * entered, rays traced) -- the byte accounting of the roofline. */
lrx_status lrx_trace_counted(lrx_scene *scene, const void *d_rays, void *d_hits,
		uint32_t count, uint32_t mode, uint64_t *d_counters, void *stream);

/* Synchronises `stream` and returns (then clears) the scene's device status
 * word: 0 = no fault; bit 0 = traversal stack limit; bit 1 = visit limit;
 * bit 2 = launch deadline.  Each bit means some rays of some launch since the
 * last call were abandoned, their hits not written; the call then returns
 * LRX_ERR_DEVICE. */
lrx_status lrx_scene_device_status(lrx_scene *scene, uint32_t *status, void *stream);

/* ---- Scene ingestion and the BVH blob cache ---------------------------- */

/* A triangle mesh read from a file; vertices xyz per vertex, three indices
 * per triangle -- directly usable as an lrx_mesh_desc.  Owned by the
 * library until lrx_ply_free. */
typedef struct lrx_ply_mesh {
	float *vertices;
	uint32_t *triangles;
	uint32_t vertex_count;
	uint32_t triangle_count;
} lrx_ply_mesh;

/* Reads the geometry of an ascii / binary little-endian / binary big-endian
 * PLY file: vertex x, y, z (any numeric type, stored as float) and the face
 * list "vertex_indices" -- triangles kept, quads split into (0,1,2) and
 * (0,2,3), other polygons dropped.  No host CUDA call.
 * Replaces: the geometry part of ExtTriangleMesh::LoadPly
 * (src/luxrays/core/exttrianglemeshfile.cpp:207-290). */
lrx_status lrx_ply_load(const char *path, lrx_ply_mesh *mesh);
void lrx_ply_free(lrx_ply_mesh *mesh);

/* 64-bit content key of a scene's inputs (geometry, objects, build options)
 * for caching built scenes: equal inputs give equal keys.  No CUDA call. */
lrx_status lrx_scene_key(const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count,
		const lrx_build_opts *opts, uint64_t *key);

/* Serialises a built scene -- its device node, triangle and instance arrays
 * and the host metadata instance updates need -- into host memory.  Call
 * with blob NULL to get the size in *bytes; then with a buffer of that size.
 * Synchronises `stream`.  No reference counterpart (the reference rebuilds
 * its accelerators). */
lrx_status lrx_scene_save(const lrx_scene *scene, void *blob, size_t *bytes, void *stream);

/* Creates a scene on the current device from a blob written by
 * lrx_scene_save (checked: magic, version, sizes, checksum) without
 * building: the arrays are uploaded as they are.  Traces equal the saved
 * scene's bit for bit. */
lrx_status lrx_scene_load(const void *blob, size_t bytes, void *stream, lrx_scene **out_scene);

#ifdef __cplusplus
}
#endif

#endif /* LRX_H */
