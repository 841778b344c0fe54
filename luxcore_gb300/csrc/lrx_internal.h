// Host-side internals shared by the C-ABI layer, the builder and the
// traversal launchers.  Not part of the public ABI.
#pragma once

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/lrx.h"

namespace lrx {

struct WideNode;
struct Node4;
struct TriRecord;
struct InstRecord;

// Error reporting: the thread-local message behind lrx_last_error().
void set_error(const std::string &msg);
lrx_status cuda_fail(cudaError_t e, const char *what);

#define LRX_CUDA(call)                                                         \
	do {                                                                       \
		cudaError_t _e = (call);                                               \
		if (_e != cudaSuccess) return ::lrx::cuda_fail(_e, #call);             \
	} while (0)

// Device buffer owned by the library (freed on destruction).
struct DevBuf {
	void *ptr = nullptr;
	size_t bytes = 0;
	DevBuf() = default;
	DevBuf(const DevBuf &) = delete;
	DevBuf &operator=(const DevBuf &) = delete;
	DevBuf(DevBuf &&o) noexcept : ptr(o.ptr), bytes(o.bytes) {
		o.ptr = nullptr;
		o.bytes = 0;
	}
	DevBuf &operator=(DevBuf &&o) noexcept {
		if (this != &o) {
			release();
			ptr = o.ptr;
			bytes = o.bytes;
			o.ptr = nullptr;
			o.bytes = 0;
		}
		return *this;
	}
	~DevBuf() { release(); }
	lrx_status alloc(size_t n);   // no-op if already >= n
	void release();
	template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// Scratch memory for one BVH build (grown on demand, reused across builds).
struct BuildScratch {
	DevBuf keys, keys_alt, vals, vals_alt, cub_temp;
	DevBuf bnodes, branges, other_bound;
	DevBuf wide_nodes, prim_order;
	DevBuf queue_a, queue_b;
	DevBuf counters;   // uint32 counters + bounds (small)
	DevBuf treelet_scratch;
};

struct BvhResult {
	uint32_t node_count = 0;  // wide nodes written to scratch.wide_nodes
	uint32_t depth = 0;       // wide-node levels
	float lo[3] = {0, 0, 0};  // root box (union of the padded primitive boxes)
	float hi[3] = {0, 0, 0};
};

// Builds an 8-wide compressed BVH over n primitive boxes (lo/hi as float4,
// xyz used).  On return scratch.wide_nodes holds node_count nodes whose
// child_base / tri_base are relative to 0, and scratch.prim_order holds the
// n primitive indices in leaf order.  Synchronises `stream`.
lrx_status build_wide_bvh(uint32_t n, const float4 *d_lo, const float4 *d_hi,
		uint32_t leaf_max, uint32_t node_width, uint32_t treelet_passes, cudaStream_t stream,
		BuildScratch &scratch, BvhResult *out);

// Per-triangle padded boxes (Union(BBox(p0,p1),p2) expanded by
// MachineEpsilon::E, bvhaccel.cpp:116-122) for one mesh.
lrx_status launch_triangle_boxes(uint32_t n_tris, const float *d_verts, const uint32_t *d_idx,
		float4 *d_lo, float4 *d_hi, cudaStream_t stream);

// Copies nodes into the scene array, offsetting child/tri bases.
lrx_status launch_relocate_nodes(const WideNode *src, WideNode *dst, uint32_t n,
		uint32_t node_offset, uint32_t tri_offset, cudaStream_t stream);

// Repacks a tree of at most 4 children per node from 80-byte records into
// 64-byte ones (LRX_NODES_COMPACT4).  Synchronises `stream`; LRX_ERR_BUILD
// if a node holds more than 4 children.
lrx_status pack_nodes4(const WideNode *src, Node4 *dst, uint32_t n, cudaStream_t stream);

// Writes triangle records for one mesh in leaf order.  d_tri_object, when
// not null, holds (object index, triangle index) per triangle of a merged
// mesh; otherwise every record gets object_const and its own index.
lrx_status launch_triangle_records(uint32_t n_tris, const uint32_t *d_prim_order,
		const float *d_verts, const uint32_t *d_idx, const uint32_t *d_tri_object,
		uint32_t object_const, TriRecord *dst, cudaStream_t stream);

struct TraceArgs {
	const WideNode *nodes;
	const TriRecord *tris;
	const InstRecord *insts;
	uint32_t root;          // root node of the flat BVH or of the TLAS; kNull = empty
	uint32_t two_level;
	const void *rays;
	void *hits;
	uint32_t count;
	uint32_t any_hit;
	uint32_t *status;
	unsigned long long *counters;  // nullptr unless counting
	uint32_t block_size = 0;       // threads per block (0 = kTraceBlock)
	uint32_t postpone = 0;         // min lanes testing triangles before deferring (0 = never)
	uint32_t variant = 0;          // lrx_trace_config.variant bits
	// Node-visit budget of a ray: visit_limit at its start, plus blas_visits
	// at every instance entry; a ray that exhausts it is abandoned (status
	// bit 1, hit not written).  The scene's own bound -- its top-level tree's
	// node count, plus the largest BLAS's at each entry -- is never reached
	// by a valid tree, since a walk expands each node of a tree at most once
	// per entry into that tree.
	uint32_t visit_limit = 1u << 24;
	uint32_t blas_visits = 0;
	// Launch deadline in %globaltimer ticks of 1,024 ns (0 = none), from the
	// start of each persistent warp or of each block of the one-ray-per-thread
	// kernel: once it has passed, rays not yet started are abandoned (status
	// bit 2, hits not written).  launch_id picks the persistent kernels'
	// counter slot (next_launch_id).
	uint32_t deadline_ticks = 0;
	uint32_t launch_id = 0;
	const uint32_t *order = nullptr;  // thread i traces ray order[i] (sorted launches)
	uint32_t refill = 0;           // persistent fetch: idle lanes that trigger a warp's claim (0 = 16)
	const uint32_t *count_dev = nullptr;  // persistent fetch: rays to claim, read on the device (<= count)
	uint32_t motion = 0;           // two-level scene with motion instances: the kVarMotion builds trace it
	uint32_t nodes4 = 0;           // flat scene in 64-byte node records: the kVarNodes4 builds trace it
};
constexpr uint32_t kTraceBlock = 128;
constexpr uint32_t kVarSortRays = 0x10u;   // reorder rays by octant + origin before tracing
constexpr uint32_t kVarSortOctantOnly = 0x20u;  // ... by direction octant only (one radix pass)
constexpr uint32_t kVarPersistent = 0x40u;  // persistent warps with warp-level ray fetch
constexpr uint32_t kVarSmemStack = 0x80u;  // top of the traversal stack in shared memory
constexpr uint32_t kVarCompact = 0x100u;   // with kVarPersistent: trace only the unmasked rays, compacted first
constexpr uint32_t kVarMotion = 0x200u;    // internal build bit: instance entry samples motion systems
constexpr uint32_t kVarSmemStack16 = 0x400u;  // the top 16 stack entries in shared memory
constexpr uint32_t kVarSmemStack32 = 0x800u;  // the top 32 stack entries in shared memory
constexpr uint32_t kVarNodes4 = 0x1000u;   // internal build bit: the scene's nodes are 64-byte records
constexpr uint32_t kVarDrainSplit = 0x2000u;  // with kVarPersistent, closest hit (no motion): idle lanes take subtrees at the drain
constexpr uint32_t kVarAll = 0x2dffu;      // every public variant bit
// The shared-memory stack bit of a variant (the deepest one asked for), or 0.
constexpr uint32_t smem_stack_bits(uint32_t v) {
	return (v & kVarSmemStack32) ? kVarSmemStack32 : (v & kVarSmemStack16) ? kVarSmemStack16 : (v & kVarSmemStack);
}
// Stack entries per thread in shared memory for a compile-time variant.
constexpr int smem_stack_depth(uint32_t v) {
	return (v & kVarSmemStack32) ? 32 : (v & kVarSmemStack16) ? 16 : (v & kVarSmemStack) ? 8 : 0;
}
constexpr uint32_t kSortMinRays = 32768;   // smaller batches are traced in caller order

lrx_status launch_trace(const TraceArgs &a, cudaStream_t stream);

// Launch deadline in timer ticks for a launch of `rays` rays under a config
// deadline of `deadline_us` microseconds (0: 10 s plus 0.1 us per ray).
inline uint32_t deadline_ticks(uint32_t deadline_us, uint64_t rays) {
	const uint64_t us = deadline_us ? deadline_us : 10000000ull + rays / 10u;
	return (uint32_t)std::min<uint64_t>((us * 1000u + 1023u) / 1024u, 0x7fffffffull);
}

// Id of the next launch: its persistent counter slot is id % kQueueSlots
// (a slot is reused only kQueueSlots launches later).
uint32_t next_launch_id();

// One batch of a multi-batch queue launch (kernel parameter space).
struct QueueBatch {
	const WideNode *nodes;
	const TriRecord *tris;
	const InstRecord *insts;
	const void *rays;
	void *hits;
	uint32_t *status;
	uint32_t root, count;
	uint32_t tile_begin;   // first 64-ray tile of this batch in the launch (tile kernel)
	uint32_t ray_begin;    // first ray of this batch in the launch's ray index space (fetch kernel)
	uint32_t flags;        // bit 0 any-hit, bit 1 two-level, bits 8-15 postpone, bits 16-23 variant,
	                       // bits 24-28 f: each instance entry adds 2^f node visits to the budget (f = 0: none)
	uint32_t visit_limit;
	uint32_t user_index;   // the caller's index of this batch (completion flags)
	uint32_t order_begin;  // sorted batch: its permutation at QueueParams::order + order_begin; else kNull
};
constexpr uint32_t kTileRays = 64;
constexpr uint32_t kMaxQueueBatches = 384;  // keeps the parameter block under 32 KB
constexpr uint32_t kQueueSlots = 4096;      // concurrent queue launches per device
// Rays per fetch-kernel launch: claims overshoot the count by at most one
// claim per resident warp (< 2^20 rays), so they stay below 2^31 and bit 31 of
// a broadcast claim base is free to carry the deadline flag.
constexpr uint32_t kMaxFetchRays = 0x7f000000u;
constexpr uint32_t kDirectBatchRays = 131072;  // lrx_trace_batches: batches this large get launches of their own
constexpr uint32_t kMaxDirectBatches = 4;      // ... when a call holds at most this many of them
constexpr uint32_t kSideStreams = 6;           // side streams per thread and device
// lrx_trace_host_batches: rays per copy-in/trace/copy-out chunk.  512 k rays
// (24 MB in, 10 MB out): on the heightfield step, batches largest first,
// 2,801 Mrays/s end to end, against 2,733 at 384 k, 2,660 at 256 k, 2,640 at
// 640 k, 2,656 at 768 k and 2,552 at 1 M.
constexpr uint32_t kHostChunkRays = 524288u;
struct QueueParams {
	uint32_t n, total_tiles, slot;  // slot = launch_id % kQueueSlots
	uint32_t fetch;         // 1: warp-level ray fetch (k_trace_queue_fetch), 0: 64-ray tiles per block
	uint32_t total_rays;    // fetch kernel: rays in the launch (<= kMaxFetchRays)
	uint32_t refill;        // fetch kernel: idle lanes that trigger a warp's claim, 1-32
	uint32_t *tiles_done;   // per batch progress (tiles, or rays with `fetch`), zeroed before the launch (nullable)
	uint32_t *done_flags;   // per batch, set to 1 when its last ray is written (nullable, may be host-mapped)
	const uint32_t *order;  // permutations of the sorted batches, concatenated (nullable)
	// batches are ordered by ray class (0 closest flat, 1 closest two-level, 2 any flat,
	// 3 any two-level); class c is batches [class_batch[c], class_batch[c + 1])
	uint32_t class_batch[5];
	uint32_t deadline_ticks;  // as TraceArgs::deadline_ticks, for the whole launch
	uint32_t launch_id;
	QueueBatch b[kMaxQueueBatches];
};
static_assert(sizeof(QueueParams) <= 32000, "kernel parameter limit");

// Library-owned stream-ordered memory pool of a device (freed blocks are
// kept for reuse); for per-call scratch that must not synchronise the device.
lrx_status stream_pool(int dev, cudaMemPool_t *out);

// Sets *flag to 1 in stream order, after a fence that orders every earlier
// write of the stream's kernels before it (host-mapped flags allowed).
lrx_status launch_set_flag(uint32_t *flag, cudaStream_t stream);

// d_hits[i] = src[i] for the masked rays of d_rays[0, n); src is a device
// view of the caller's (mapped host) hit buffer.
lrx_status launch_restore_masked_hits(const void *d_rays, uint32_t n, const void *src, void *d_hits,
		cudaStream_t stream);

// One launch of the persistent queue kernel over p.n batches.
lrx_status launch_trace_queue(const QueueParams &p, cudaStream_t stream);

// A device region the caller already owns, lent to one sorted or compacted
// launch for its scratch in place of the stream-ordered pool (the
// no-allocation entry point passes its static array).  The launch fails with
// LRX_ERR_NOT_SUPPORTED if the region is too small; nothing is allocated.
struct FixedScratch {
	void *base = nullptr;   // 256-byte aligned
	size_t bytes = 0;
};
// Scratch bytes a sorted launch of n rays needs besides the sort's own
// temporary storage: keys and indices, double-buffered.
inline size_t sorted_scratch_arrays(uint32_t n) {
	return 4 * (((sizeof(uint32_t) * (size_t)n + 255) / 256) * 256);
}

// Sorts the rays (octant, origin Morton code in [lo, hi]) and traces them in
// that order; scratch from a stream-ordered pool, or from `fixed` when given.
// Hits land in caller order.
lrx_status launch_trace_sorted(const TraceArgs &a, const float lo[3], const float hi[3], cudaStream_t stream,
		const FixedScratch *fixed = nullptr);

// Compacts the indices of the rays without RAY_FLAGS_MASKED (stable) into
// pool scratch (or `fixed` when given) and traces them with the persistent
// kernel, which reads the compacted count on the device.  Masked rays are
// neither read by the traversal nor written.
lrx_status launch_trace_compacted(const TraceArgs &a, cudaStream_t stream, const FixedScratch *fixed = nullptr);

// One batch of a queue launch to reorder: its rays, count, the scene box and
// the offset of its permutation in the launch's concatenated order array.
struct SortBatch {
	const void *rays;
	uint32_t count, offset;
	float lo[3], hi[3];
	bool octant_only;
};
// Computes every listed batch's permutation with one radix sort (batch index
// above the ray key) into pool scratch; *order gets the concatenated
// permutations, *scratch what to release (cudaFreeAsync on `stream`) after
// the launch that reads them.
lrx_status sort_queue_batches(const std::vector<SortBatch> &batches, uint32_t total, cudaStream_t stream,
		const uint32_t **order, void **scratch);

// CUDA device a scene was built on.
int scene_device(const lrx_scene *scene);

// Matrix4x4::Inverse (row-major 4x4, FP32); false for a singular matrix.
bool host_matrix_inverse(const float in[16], float out[16]);

struct MotionInterval;
// A motion system's intervals from `count` keyframes (strictly increasing
// times, row-major matrices): count + 1 records, of which the traversal
// samples the first count (lrx_motion.cpp).
lrx_status motion_intervals(const float *times, const float *mats, uint32_t count,
		std::vector<MotionInterval> &out);
// Swept world box of a local box under a motion system of world->local
// keyframes (MotionSystem::Bound with storingGlobal2Local).
lrx_status motion_bound(const std::vector<MotionInterval> &its, const float lo[3], const float hi[3], float olo[3],
		float ohi[3]);

// lrx_scene_load without the checksum pass, for blobs the library wrote and
// kept in its own memory (the server's cache of evicted scenes).
lrx_status scene_load_trusted(const void *blob, size_t bytes, cudaStream_t stream, lrx_scene **out_scene);

}  // namespace lrx
