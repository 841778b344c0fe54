// The scene record behind the opaque lrx_scene handle, shared by the C-ABI
// translation units: scene assembly (lrx_api.cpp), built-scene blobs
// (lrx_blob.cpp) and the tracing entry points (lrx_launch.cpp).  Not part of
// the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <vector>

#include "lrx_common.cuh"
#include "lrx_internal.h"

namespace lrx {

struct Blas {
	uint32_t mesh = kNull;        // instanced mesh, or kNull for the merged plain BLAS
	uint32_t tri_count = 0;
	uint32_t root = kNull;        // absolute node index
	float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

// Children per wide node of a scene's builds (0 in blobs written before the
// option existed: the 8-wide default).
inline uint32_t node_width(const lrx_build_opts &o) {
	return o.node_width ? o.node_width : 8u;
}

// Size of lrx_build_opts in ABI 1-3 (it ended after node_width).
constexpr uint32_t kBuildOptsAbi3Size = (uint32_t)offsetof(lrx_build_opts, node_layout);

// The build options a caller's struct (nullable) asks for, over the library
// defaults -- 3 triangles per leaf, 2 treelet passes, 8-wide nodes in the
// 80-byte record; fields beyond the caller's struct_size keep their
// defaults, and a struct smaller than the ABI 1-3 one is ignored.
inline lrx_build_opts read_build_opts(const lrx_build_opts *in) {
	lrx_build_opts o{};
	o.struct_size = sizeof(lrx_build_opts);
	o.leaf_max = 3;
	o.treelet_passes = 2;
	o.node_width = 8;
	o.node_layout = LRX_NODES_WIDE8;
	if (in && in->struct_size >= kBuildOptsAbi3Size) {
		if (in->leaf_max) o.leaf_max = in->leaf_max < 3u ? in->leaf_max : 3u;
		o.treelet_passes = in->treelet_passes;
		if (in->node_width) o.node_width = in->node_width;
		if (in->struct_size >= sizeof(lrx_build_opts)) o.node_layout = in->node_layout;
	}
	return o;
}

// Bytes per node record of a scene's tree.
inline uint32_t node_record_bytes(const lrx_build_opts &o) {
	return o.node_layout == LRX_NODES_COMPACT4 ? (uint32_t)sizeof(Node4) : (uint32_t)sizeof(WideNode);
}

// Makes `dev` current for the guard's lifetime.
struct DeviceGuard {
	int prev = -1;
	explicit DeviceGuard(int dev) {
		if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
		else prev = -1;
	}
	~DeviceGuard() {
		if (prev >= 0) cudaSetDevice(prev);
	}
};

}  // namespace lrx

struct lrx_scene {
	int device = 0;
	bool two_level = false;
	uint32_t root = lrx::kNull;
	lrx::DevBuf nodes, tris, insts, status, stage_rays, stage_hits;
	std::vector<lrx::Blas> blas;
	std::vector<uint32_t> obj_blas;     // per object: BLAS index, kNull if empty
	std::vector<uint32_t> obj_flags;
	uint32_t mesh_count = 0;
	uint32_t plain_blas = lrx::kNull;  // index of the merged plain BLAS
	uint32_t tlas_node_offset = 0;
	uint32_t tlas_capacity = 0;
	uint32_t blas_node_total = 0;
	lrx_build_opts opts{};
	// default launch per mode (closest, any-hit): 64-thread blocks (best of a
	// block-size x postpone sweep on the heightfield ray sets).  Closest-hit
	// batches run on persistent warps that refill once 8 lanes are idle (+28 %
	// on incoherent bounce rays there, -4 % on coherent primary rays) and test
	// triangles as they come: on SAH-optimally collapsed trees deferring them
	// no longer pays (postpone 8 against 0: primary +2.2 %, bounce +1.4 %
	// launch time).  Any-hit batches are reordered by octant + origin first
	// (+20 % on shadow rays; the sort costs more than it saves on closest-hit
	// rays, and persistent warps add nothing after it); any hit never defers.
	// Once a closest-hit launch's rays are all claimed, idle lanes take
	// subtrees of their warp's last rays (the drain split: primary -4.6 %,
	// bounce -4.0 % launch time on 1 M rays, neutral on 8 M).
	lrx_trace_config tcfg[2] = {{sizeof(lrx_trace_config), 64, 0, lrx::kVarPersistent | lrx::kVarDrainSplit, 1, 8},
			{sizeof(lrx_trace_config), 64, 8, lrx::kVarSortRays, 2, 0}};
	lrx_scene_info info{};
	lrx::BuildScratch scratch;
	std::mutex mu;
	float bounds_lo[3] = {0, 0, 0}, bounds_hi[3] = {0, 0, 0};  // world box of the root
	// motion-blurred instances: per object an index into motions (kNull: none)
	struct Motion {
		std::vector<lrx::MotionInterval> its;  // keyframes + 1 intervals (the device gets the first keyframes)
		uint32_t offset16 = 0;            // device copy, in 16-byte units from the instance array's base
		bool have_box = false;
		float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // swept world box, padded
	};
	std::vector<uint32_t> obj_motion;
	std::vector<Motion> motions;
};

namespace lrx {

// The node-visit budget of one ray in scene s at its start, and what each
// instance entry adds to it (a correct walk never spends it).
uint32_t scene_visit_limit(const lrx_scene *s);
uint32_t scene_blas_visits(const lrx_scene *s);

// One trace launch of `count` rays with the scene's configuration for `mode`,
// validating every argument (the body of lrx_trace and lrx_trace_counted).
// `fixed`, when given, is the scratch of sorted and compacted launches
// instead of the stream-ordered pool.  `pipeline_chunk`: a chunk of the
// host-buffer pipeline, traced beside others -- a configuration that sorts
// rays takes persistent warps instead (refill 8 unless set).
lrx_status trace_common(lrx_scene *s, const void *d_rays, void *d_hits, uint32_t count, uint32_t mode,
		uint64_t *d_counters, cudaStream_t st, const FixedScratch *fixed = nullptr, bool pipeline_chunk = false);

}  // namespace lrx
