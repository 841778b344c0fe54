// Tracing entry points of liblrx.so over device and host ray buffers:
// lrx_trace, lrx_trace_counted, lrx_trace_batches (one queue launch, or a
// few large launches side by side on forked streams) and the host-buffer
// forms lrx_trace_host and lrx_trace_host_batches (copies overlapped with
// traces).  Declarations are in include/lrx.h.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "lrx_common.cuh"
#include "lrx_internal.h"
#include "lrx_scene.h"

using namespace lrx;

extern "C" {

lrx_status lrx_trace(lrx_scene *s, const void *d_rays, void *d_hits, uint32_t count, uint32_t mode, void *stream) {
	return trace_common(s, d_rays, d_hits, count, mode, nullptr, (cudaStream_t)stream);
}

lrx_status lrx_trace_batches(const lrx_batch *batches, uint32_t n_batches, void *stream) {
	return lrx_trace_batches_ex(batches, n_batches, stream, nullptr, nullptr);
}

// Streams and events of the calling thread on one device for the batches
// lrx_trace_batches launches on their own (created on first use, never
// shared with another thread, so a graph capture on one thread cannot catch
// another thread's work).
struct SideStreams {
	int dev = -1;
	cudaStream_t s[kSideStreams] = {};
	cudaEvent_t fork = nullptr, join[kSideStreams] = {};
	SideStreams() = default;
	SideStreams(const SideStreams &) = delete;
	SideStreams &operator=(const SideStreams &) = delete;
	~SideStreams() {  // at thread exit; errors (a context already torn down) are ignored
		for (uint32_t k = 0; k < kSideStreams; ++k) {
			if (s[k]) cudaStreamDestroy(s[k]);
			if (join[k]) cudaEventDestroy(join[k]);
		}
		if (fork) cudaEventDestroy(fork);
	}
};

static lrx_status side_streams(int dev, SideStreams **out) {
	thread_local std::vector<std::unique_ptr<SideStreams>> per_dev;
	for (auto &p : per_dev)
		if (p->dev == dev) {
			*out = p.get();
			return LRX_OK;
		}
	std::unique_ptr<SideStreams> ss(new SideStreams());
	ss->dev = dev;
	for (uint32_t k = 0; k < kSideStreams; ++k) {
		LRX_CUDA(cudaStreamCreateWithFlags(&ss->s[k], cudaStreamNonBlocking));
		LRX_CUDA(cudaEventCreateWithFlags(&ss->join[k], cudaEventDisableTiming));
	}
	LRX_CUDA(cudaEventCreateWithFlags(&ss->fork, cudaEventDisableTiming));
	*out = ss.get();
	per_dev.push_back(std::move(ss));
	return LRX_OK;
}

// A batch traced by a launch of its own rather than in the queue launch:
// one on a scene with motion instances or with 64-byte node records (the
// queue kernels trace neither), or -- when the call holds at most
// kMaxDirectBatches batches of kDirectBatchRays rays or more -- one of those.
static bool direct_batch(const lrx_batch &b, bool big_direct) {
	return b.count != 0 && ((big_direct && b.count >= kDirectBatchRays) || !b.scene->motions.empty() ||
			b.scene->opts.node_layout == LRX_NODES_COMPACT4);
}

lrx_status lrx_trace_batches_ex(const lrx_batch *batches, uint32_t n_batches, void *stream,
		uint32_t *d_tile_counters, uint32_t *d_done_flags) {
	if (n_batches && !batches) {
		set_error("lrx_trace_batches: null batch array");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if ((d_tile_counters == nullptr) != (d_done_flags == nullptr)) {
		set_error("lrx_trace_batches_ex: give both the tile counters and the done flags, or neither");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	int dev = 0;
	for (uint32_t k = 0; k < n_batches; ++k) {
		const lrx_batch &b = batches[k];
		if (!b.scene || b.mode > LRX_TRACE_ANY) {
			set_error("lrx_trace_batches: batch " + std::to_string(k) + ": null scene or unknown mode");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		if (b.count && (!b.d_rays || !b.d_hits || ((uintptr_t)b.d_rays & 15u) || ((uintptr_t)b.d_hits & 3u))) {
			set_error("lrx_trace_batches: batch " + std::to_string(k) + ": null or misaligned ray/hit buffer");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		if (k == 0) dev = b.scene->device;
		if (b.scene->device != dev) {
			set_error("lrx_trace_batches: all scenes of one call must live on one device");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	}
	if (n_batches == 0) return LRX_OK;
	DeviceGuard g(dev);
	thread_local std::unique_ptr<QueueParams> params;
	if (!params) params.reset(new QueueParams());
	QueueParams &p = *params;
	cudaStream_t st = (cudaStream_t)stream;
	// Warp-level ray fetch when any batch's scene asks for persistent warps in
	// its mode (refill from the first such config) and every batch fits one
	// fetch launch; otherwise 64-ray tiles per block.
	uint32_t n_big = 0;
	for (uint32_t k = 0; k < n_batches; ++k) n_big += batches[k].count >= kDirectBatchRays ? 1u : 0u;
	const bool big_direct = n_big <= kMaxDirectBatches;
	uint32_t fetch = 0, refill = 16;
	for (uint32_t k = 0; k < n_batches; ++k) {
		if (direct_batch(batches[k], big_direct)) continue;
		if (batches[k].count > kMaxFetchRays) {
			fetch = 0;
			break;
		}
		const lrx_trace_config &cfg = batches[k].scene->tcfg[batches[k].mode == LRX_TRACE_ANY ? 1 : 0];
		if (!fetch && (cfg.variant & kVarPersistent)) {
			fetch = 1;
			if (cfg.refill) refill = std::min(32u, cfg.refill);
		}
	}
	p.fetch = fetch;
	p.refill = refill;
	p.tiles_done = d_tile_counters;
	p.done_flags = d_done_flags;
	if (d_tile_counters) LRX_CUDA(cudaMemsetAsync(d_tile_counters, 0, sizeof(uint32_t) * n_batches, st));
	// The batches of one launch are gathered first, then laid out by ray class
	// (closest/any x flat/two-level) so each class is one contiguous range.
	struct Entry {
		uint32_t k, cls;
		bool sort;  // scene config sorts rays and the batch has >= kSortMinRays
	};
	std::vector<Entry> pending;
	uint64_t pend_tiles = 0, pend_rays = 0, pend_sorted = 0;
	std::vector<SortBatch> sorted;
	uint32_t launch_deadline_us = 0;  // the smallest deadline the launch's batches' configs set (0: none set)
	auto flush = [&]() -> lrx_status {
		if (pending.empty()) return LRX_OK;
		std::stable_sort(pending.begin(), pending.end(), [](const Entry &a, const Entry &b) { return a.cls < b.cls; });
		p.n = 0;
		p.total_tiles = 0;
		p.total_rays = 0;
		p.order = nullptr;
		sorted.clear();
		uint32_t sorted_rays = 0;
		for (uint32_t c = 0; c <= 4; ++c) p.class_batch[c] = (uint32_t)pending.size();
		for (const Entry &e : pending) {
			const lrx_batch &b = batches[e.k];
			lrx_scene *s = b.scene;
			const lrx_trace_config &cfg = s->tcfg[b.mode == LRX_TRACE_ANY ? 1 : 0];
			if (p.class_batch[e.cls] == pending.size()) p.class_batch[e.cls] = p.n;
			QueueBatch &q = p.b[p.n++];
			q.nodes = s->nodes.as<WideNode>();
			q.tris = s->tris.as<TriRecord>();
			q.insts = s->insts.as<InstRecord>();
			q.rays = b.d_rays;
			q.hits = b.d_hits;
			q.status = s->status.as<uint32_t>();
			q.root = s->root;
			q.count = b.count;
			q.tile_begin = p.total_tiles;
			q.ray_begin = p.total_rays;
			// runtime-selectable variants only (cache hints); sorting is done before the launch
			const uint32_t var = cfg.variant & (LRX_VARIANT_SCENE_L2_KEEP | LRX_VARIANT_STREAM_RAYS);
			// the visit budget's per-instance-entry part, as a power of two (bits 24-28)
			uint32_t f = 0;
			if (!cfg.max_visits)
				while (f < 31u && (1u << f) < scene_blas_visits(s)) ++f;
			if (f && !s->two_level) f = 0;
			q.flags = (b.mode == LRX_TRACE_ANY ? 1u : 0u) | (s->two_level ? 2u : 0u) |
					((cfg.postpone & 0xffu) << 8) | (var << 16) | (f << 24);
			q.visit_limit = cfg.max_visits ? cfg.max_visits : scene_visit_limit(s);
			if (cfg.deadline_us) launch_deadline_us = launch_deadline_us ? std::min(launch_deadline_us, cfg.deadline_us)
					: cfg.deadline_us;
			q.user_index = e.k;
			q.order_begin = kNull;
			if (e.sort) {
				SortBatch sb;
				sb.rays = b.d_rays;
				sb.count = b.count;
				sb.offset = sorted_rays;
				for (int c = 0; c < 3; ++c) {
					sb.lo[c] = s->bounds_lo[c];
					sb.hi[c] = s->bounds_hi[c];
				}
				sb.octant_only = (cfg.variant & kVarSortOctantOnly) != 0;
				sorted.push_back(sb);
				q.order_begin = sorted_rays;
				sorted_rays += b.count;
			}
			p.total_tiles += (b.count + kTileRays - 1) / kTileRays;
			p.total_rays += fetch ? b.count : 0u;
		}
		// a class with no batches starts where the next non-empty one does
		for (int c = 3; c >= 0; --c) p.class_batch[c] = std::min(p.class_batch[c], p.class_batch[c + 1]);
		p.launch_id = next_launch_id();
		p.slot = p.launch_id % kQueueSlots;
		p.deadline_ticks = deadline_ticks(launch_deadline_us, fetch ? p.total_rays : (uint64_t)p.total_tiles * kTileRays);
		launch_deadline_us = 0;
		void *scratch = nullptr;
		lrx_status rc = sort_queue_batches(sorted, sorted_rays, st, &p.order, &scratch);
		if (rc == LRX_OK) rc = launch_trace_queue(p, st);
		if (scratch) cudaFreeAsync(scratch, st);  // ordered after the launch that reads it
		pending.clear();
		pend_tiles = pend_rays = pend_sorted = 0;
		return rc;
	};
	// A few large batches (at most kMaxDirectBatches of at least kDirectBatchRays
	// rays -- a wavefront's camera, bounce and shadow buffers), and batches on
	// scenes with motion instances (the queue kernels carry no motion code),
	// are traced by launches of their own -- the scene's plain path -- on side
	// streams forked from `stream` and joined back into it, so their launches
	// run beside each other and beside the queue launch of the other batches:
	// one launch's drain (its last, longest rays) overlaps the others' work.
	// Many large batches stay in the queue launch, which drains once for all
	// of them.  A direct batch's completion flag follows its launch on its
	// side stream.
	SideStreams *side = nullptr;
	auto trace_all = [&]() -> lrx_status {
		// largest first: the longest launch starts first, and the others fill in
		// beside it (the heightfield step 1.7261 against 1.7310 ms)
		uint32_t n_direct = 0;
		std::vector<uint32_t> direct;
		for (uint32_t k = 0; k < n_batches; ++k)
			if (direct_batch(batches[k], big_direct)) direct.push_back(k);
		std::stable_sort(direct.begin(), direct.end(),
				[&](uint32_t x, uint32_t y) { return batches[x].count > batches[y].count; });
		for (uint32_t k : direct) {
			const lrx_batch &b = batches[k];
			if (!side) {
				lrx_status rc = side_streams(dev, &side);
				if (rc != LRX_OK) return rc;
				LRX_CUDA(cudaEventRecord(side->fork, st));
				for (uint32_t j = 0; j < kSideStreams; ++j) LRX_CUDA(cudaStreamWaitEvent(side->s[j], side->fork, 0));
			}
			cudaStream_t ss = side->s[n_direct++ % kSideStreams];
			lrx_status rc = trace_common(b.scene, b.d_rays, b.d_hits, b.count, b.mode, nullptr, ss);
			if (rc == LRX_OK && d_done_flags) rc = launch_set_flag(d_done_flags + k, ss);
			if (rc != LRX_OK) return rc;
		}
		for (uint32_t k = 0; k < n_batches; ++k) {
			const lrx_batch &b = batches[k];
			if (b.count == 0 || direct_batch(b, big_direct)) continue;
			lrx_scene *s = b.scene;
			const uint32_t tiles = (b.count + kTileRays - 1) / kTileRays;
			const lrx_trace_config &cfg = s->tcfg[b.mode == LRX_TRACE_ANY ? 1 : 0];
			const bool sort = (cfg.variant & kVarSortRays) && b.count >= kSortMinRays && s->root != kNull;
			if (pending.size() == kMaxQueueBatches || pend_tiles + tiles > 0xffffffffull ||
					(fetch && pend_rays + b.count > kMaxFetchRays) || (sort && pend_sorted + b.count > kMaxFetchRays)) {
				lrx_status rc = flush();
				if (rc != LRX_OK) return rc;
			}
			pending.push_back({k, (b.mode == LRX_TRACE_ANY ? 2u : 0u) | (s->two_level ? 1u : 0u), sort});
			pend_tiles += tiles;
			pend_rays += b.count;
			pend_sorted += sort ? b.count : 0u;
		}
		return flush();
	};
	const lrx_status rc = trace_all();
	if (side) {  // join every side stream back, also after an error (a capture must not stay forked)
		for (uint32_t j = 0; j < kSideStreams; ++j) {
			cudaEventRecord(side->join[j], side->s[j]);
			cudaStreamWaitEvent(st, side->join[j], 0);
		}
	}
	return rc;
}

lrx_status lrx_trace_counted(lrx_scene *s, const void *d_rays, void *d_hits, uint32_t count, uint32_t mode,
		uint64_t *d_counters, void *stream) {
	if (!d_counters) {
		set_error("lrx_trace_counted: null counters");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	return trace_common(s, d_rays, d_hits, count, mode, d_counters, (cudaStream_t)stream);
}

lrx_status lrx_trace_host(lrx_scene *s, const lrx_ray *h_rays, lrx_hit *h_hits, uint32_t count, uint32_t mode,
		void *stream) {
	if (!s) {
		set_error("lrx_trace_host: null scene");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (count == 0) return LRX_OK;
	if (!h_rays || !h_hits) {
		set_error("lrx_trace_host: null ray or hit buffer");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (count > kHostChunkRays) {  // chunks whose copies overlap each other's traces
		const lrx_host_batch b{s, h_rays, h_hits, count, mode};
		return lrx_trace_host_batches(&b, 1, stream);
	}
	std::lock_guard<std::mutex> lk(s->mu);
	DeviceGuard g(s->device);
	lrx_status rc;
	if ((rc = s->stage_rays.alloc(sizeof(lrx_ray) * (size_t)count)) != LRX_OK) return rc;
	if ((rc = s->stage_hits.alloc(sizeof(lrx_hit) * (size_t)count)) != LRX_OK) return rc;
	cudaStream_t st = (cudaStream_t)stream;
	LRX_CUDA(cudaMemcpyAsync(s->stage_rays.ptr, h_rays, sizeof(lrx_ray) * (size_t)count, cudaMemcpyHostToDevice, st));
	// masked rays keep the caller's hit contents: stage them first
	LRX_CUDA(cudaMemcpyAsync(s->stage_hits.ptr, h_hits, sizeof(lrx_hit) * (size_t)count, cudaMemcpyHostToDevice, st));
	if ((rc = trace_common(s, s->stage_rays.ptr, s->stage_hits.ptr, count, mode, nullptr, st)) != LRX_OK) return rc;
	LRX_CUDA(cudaMemcpyAsync(h_hits, s->stage_hits.ptr, sizeof(lrx_hit) * (size_t)count, cudaMemcpyDeviceToHost, st));
	LRX_CUDA(cudaStreamSynchronize(st));
	return LRX_OK;
}

// Device view of host memory the device can reach directly -- pinned and
// mapped (cudaHostAlloc, cudaHostRegister) under unified addressing -- for
// the `bytes` bytes at h: both ends must resolve, to device addresses
// `bytes - 1` apart.  Pageable memory (cudaMemoryTypeUnregistered) and device
// memory give false.
static bool mapped_host_range(const void *h, size_t bytes, void **d) {
	cudaPointerAttributes a0, a1;
	if (cudaPointerGetAttributes(&a0, h) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	const void *last = static_cast<const char *>(h) + (bytes - 1);
	if (cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
		return false;
	if (static_cast<const char *>(a1.devicePointer) - static_cast<const char *>(a0.devicePointer) !=
			(std::ptrdiff_t)(bytes - 1))
		return false;
	*d = a0.devicePointer;
	return true;
}

lrx_status lrx_trace_host_batches(const lrx_host_batch *batches, uint32_t n_batches, void *stream) {
	if (n_batches && !batches) {
		set_error("lrx_trace_host_batches: null batch array");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	int dev = -1;
	for (uint32_t k = 0; k < n_batches; ++k) {
		const lrx_host_batch &b = batches[k];
		if (!b.scene || b.mode > LRX_TRACE_ANY || (b.count && (!b.h_rays || !b.h_hits))) {
			set_error("lrx_trace_host_batches: batch " + std::to_string(k) + ": null scene or buffer, or unknown mode");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		if (dev < 0) dev = b.scene->device;
		if (b.scene->device != dev) {
			set_error("lrx_trace_host_batches: all scenes of one call must live on one device");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	}
	if (dev < 0) return LRX_OK;
	DeviceGuard g(dev);
	cudaStream_t st = (cudaStream_t)stream;
	SideStreams *side = nullptr;
	lrx_status rc = side_streams(dev, &side);
	if (rc != LRX_OK) return rc;
	cudaMemPool_t pool;
	if ((rc = stream_pool(dev, &pool)) != LRX_OK) return rc;
	LRX_CUDA(cudaEventRecord(side->fork, st));
	for (uint32_t j = 0; j < kSideStreams; ++j) LRX_CUDA(cudaStreamWaitEvent(side->s[j], side->fork, 0));
	// Batches are cut into chunks of at most kHostChunkRays rays and run as a
	// three-stage pipeline: every chunk's copy in on the first side stream,
	// back to back, so the host-to-device copies never wait behind a trace or
	// a copy out; its trace on one of the middle side streams (round robin, so
	// the launches' drains overlap each other); its copy out on the last side
	// stream.  Events order each chunk's stages.  Staging comes from the
	// stream-ordered pool and is freed on the copy-out stream.  Masked rays
	// keep the caller's hit contents: when the hit buffer is mapped host
	// memory, only the masked slots are read back from it after the trace;
	// otherwise the chunk's hits are copied in first.
	static_assert(kSideStreams >= 3, "copy-in, trace and copy-out side streams");
	auto run = [&]() -> lrx_status {
		cudaStream_t s_in = side->s[0], s_out = side->s[kSideStreams - 1];
		uint32_t chunk = 0;
		// largest batch first: its chunks' copies and traces start first, and the
		// smaller batches' chunks fill in behind them (heightfield step end to end
		// with 384 k-ray chunks: 2,745 against 2,662 Mrays/s in call order)
		std::vector<uint32_t> order(n_batches);
		for (uint32_t k = 0; k < n_batches; ++k) order[k] = k;
		std::stable_sort(order.begin(), order.end(),
				[&](uint32_t x, uint32_t y) { return batches[x].count > batches[y].count; });
		for (uint32_t k : order) {
			const lrx_host_batch &b = batches[k];
			void *mapped_hits = nullptr;
			const bool mapped = b.count && mapped_host_range(b.h_hits, sizeof(lrx_hit) * (size_t)b.count, &mapped_hits);
			for (uint32_t c0 = 0; c0 < b.count; c0 += kHostChunkRays, ++chunk) {
				const uint32_t n = std::min(kHostChunkRays, b.count - c0);
				cudaStream_t s_tr = side->s[1 + chunk % (kSideStreams - 2)];
				const size_t rb = sizeof(lrx_ray) * (size_t)n, hb = sizeof(lrx_hit) * (size_t)n;
				const lrx_ray *hr = b.h_rays + c0;
				lrx_hit *hh = b.h_hits + c0;
				cudaEvent_t in_done = nullptr, tr_done = nullptr;
				LRX_CUDA(cudaEventCreateWithFlags(&in_done, cudaEventDisableTiming));
				if (cudaEventCreateWithFlags(&tr_done, cudaEventDisableTiming) != cudaSuccess) {
					cudaEventDestroy(in_done);
					return cuda_fail(cudaGetLastError(), "cudaEventCreateWithFlags");
				}
				auto stages = [&]() -> lrx_status {
					void *d_rays = nullptr, *d_hits = nullptr;
					LRX_CUDA(cudaMallocFromPoolAsync(&d_rays, rb, pool, s_in));
					const cudaError_t ea = cudaMallocFromPoolAsync(&d_hits, hb, pool, s_in);
					if (ea != cudaSuccess) {
						cudaFreeAsync(d_rays, s_in);
						return cuda_fail(ea, "cudaMallocFromPoolAsync");
					}
					bool ordered = false;  // the copy-out stream waits for the chunk's trace
					const lrx_status r = [&]() -> lrx_status {
						LRX_CUDA(cudaMemcpyAsync(d_rays, hr, rb, cudaMemcpyHostToDevice, s_in));
						if (!mapped) LRX_CUDA(cudaMemcpyAsync(d_hits, hh, hb, cudaMemcpyHostToDevice, s_in));
						LRX_CUDA(cudaEventRecord(in_done, s_in));
						LRX_CUDA(cudaStreamWaitEvent(s_tr, in_done, 0));
						lrx_status t = trace_common(b.scene, d_rays, d_hits, n, b.mode, nullptr, s_tr, nullptr, true);
						if (t == LRX_OK && mapped)
							t = launch_restore_masked_hits(d_rays, n, static_cast<const lrx_hit *>(mapped_hits) + c0,
									d_hits, s_tr);
						LRX_CUDA(cudaEventRecord(tr_done, s_tr));
						LRX_CUDA(cudaStreamWaitEvent(s_out, tr_done, 0));
						ordered = true;
						if (t == LRX_OK) LRX_CUDA(cudaMemcpyAsync(hh, d_hits, hb, cudaMemcpyDeviceToHost, s_out));
						return t;
					}();
					if (!ordered) {
						// a stage failed before the copy-out stream was ordered after
						// the chunk's work: wait for that work before the buffers go
						cudaStreamSynchronize(s_tr);
						cudaStreamSynchronize(s_in);
					}
					cudaFreeAsync(d_rays, ordered ? s_out : s_in);
					cudaFreeAsync(d_hits, ordered ? s_out : s_in);
					return r;
				};
				const lrx_status r = stages();
				cudaEventDestroy(in_done);  // released once the recorded work completes
				cudaEventDestroy(tr_done);
				if (r != LRX_OK) return r;
			}
		}
		return LRX_OK;
	};
	rc = run();
	for (uint32_t j = 0; j < kSideStreams; ++j) {
		cudaEventRecord(side->join[j], side->s[j]);
		cudaStreamWaitEvent(st, side->join[j], 0);
	}
	if (rc != LRX_OK) return rc;
	LRX_CUDA(cudaStreamSynchronize(st));
	return LRX_OK;
}

}  // extern "C"
