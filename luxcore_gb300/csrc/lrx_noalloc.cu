// lrx_trace_host_noalloc: host-buffer tracing that allocates no device
// memory.  The rays, the hits and the scratch of the launch (the ray sort's
// keys, indices and temporary storage, or the compaction's index list) all
// live in one file-scope static device array instead of buffers obtained
// from cudaMalloc or a memory pool, for callers that cannot allocate (see
// include/lrx.h).  The traversal kernels are the ones lrx_trace launches,
// with the scene's configuration for the mode, so results are the same.
#include <mutex>
#include <string>

#include "lrx_common.cuh"
#include "lrx_internal.h"
#include "lrx_scene.h"

namespace lrx {

namespace {

constexpr size_t kRayBytes = sizeof(lrx_ray);
constexpr size_t kHitBytes = sizeof(lrx_hit);
// Layout: rays, then hits, then the launch scratch; every part 256-byte aligned.
constexpr size_t kHitsOffset = (size_t)LRX_NOALLOC_MAX_RAYS * kRayBytes;
constexpr size_t kScratchOffset = kHitsOffset + (size_t)LRX_NOALLOC_MAX_RAYS * kHitBytes;
// The sort of LRX_NOALLOC_MAX_RAYS rays takes 2 MiB of keys and indices plus
// the radix sort's temporary storage (tens of KiB at this size); 4 MiB covers
// both with room to spare.  A launch that needed more would fail with
// LRX_ERR_NOT_SUPPORTED instead of allocating.
constexpr size_t kScratchBytes = 4u << 20;
constexpr size_t kStageBytes = kScratchOffset + kScratchBytes;
static_assert(kHitsOffset % 256 == 0 && kScratchOffset % 256 == 0, "staging parts must stay aligned");
static_assert(LRX_NOALLOC_MAX_RAYS * 4ull * 4 <= kScratchBytes / 2, "sort arrays must leave room for the sort temp");

// The staging area: one copy per GPU that loads the library, for the life of
// the process.  In host code this name is only a handle for the runtime; the
// device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_stage[kStageBytes];

constexpr int kMaxDevices = 64;
std::mutex g_dev_mutex[kMaxDevices];
void *g_stage_ptr[kMaxDevices] = {};

// Device address of g_stage on `dev`, looked up once per device with that
// device current (the caller holds g_dev_mutex[dev]).
lrx_status stage_address(int dev, void **out) {
	if (!g_stage_ptr[dev]) {
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_stage);
		if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(staging area)");
		g_stage_ptr[dev] = p;
	}
	*out = g_stage_ptr[dev];
	return LRX_OK;
}

struct CurrentDevice {
	int prev = -1;
	lrx_status rc = LRX_OK;
	explicit CurrentDevice(int dev) {
		int cur = 0;
		cudaError_t e = cudaGetDevice(&cur);
		if (e == cudaSuccess && cur != dev) {
			e = cudaSetDevice(dev);
			if (e == cudaSuccess) prev = cur;
		}
		if (e != cudaSuccess) rc = cuda_fail(e, "cudaSetDevice");
	}
	~CurrentDevice() {
		if (prev >= 0) cudaSetDevice(prev);
	}
};

// The copies in, the trace and the copy out of one call, enqueued on `st`.
lrx_status enqueue_call(lrx_scene *scene, unsigned char *stage, const lrx_ray *h_rays, lrx_hit *h_hits,
		uint32_t count, uint32_t mode, cudaStream_t st) {
	unsigned char *d_rays = stage;
	unsigned char *d_hits = stage + kHitsOffset;
	const FixedScratch scratch{stage + kScratchOffset, kScratchBytes};
	LRX_CUDA(cudaMemcpyAsync(d_rays, h_rays, kRayBytes * count, cudaMemcpyHostToDevice, st));
	// masked rays keep the caller's previous hit, as with lrx_trace_host
	LRX_CUDA(cudaMemcpyAsync(d_hits, h_hits, kHitBytes * count, cudaMemcpyHostToDevice, st));
	const lrx_status rc = trace_common(scene, d_rays, d_hits, count, mode, nullptr, st, &scratch);
	if (rc != LRX_OK) return rc;
	LRX_CUDA(cudaMemcpyAsync(h_hits, d_hits, kHitBytes * count, cudaMemcpyDeviceToHost, st));
	return LRX_OK;
}

}  // namespace

}  // namespace lrx

using namespace lrx;

extern "C" lrx_status lrx_trace_host_noalloc(lrx_scene *scene, const lrx_ray *h_rays, lrx_hit *h_hits,
		uint32_t count, uint32_t mode, void *stream) {
	if (!scene) {
		set_error("lrx_trace_host_noalloc: null scene");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (mode > LRX_TRACE_ANY) {
		set_error("lrx_trace_host_noalloc: unknown mode");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (count == 0) return LRX_OK;
	if (!h_rays || !h_hits) {
		set_error("lrx_trace_host_noalloc: null ray or hit buffer");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (count > LRX_NOALLOC_MAX_RAYS) {
		set_error("lrx_trace_host_noalloc: " + std::to_string(count) + " rays exceed the " +
				std::to_string(LRX_NOALLOC_MAX_RAYS) + "-ray limit of the static staging area; "
				"split the batch or use lrx_trace_host");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	const int dev = scene_device(scene);
	if (dev < 0 || dev >= kMaxDevices) {
		set_error("lrx_trace_host_noalloc: device index out of range");
		return LRX_ERR_NOT_SUPPORTED;
	}
	std::lock_guard<std::mutex> lk(g_dev_mutex[dev]);
	CurrentDevice cd(dev);
	if (cd.rc != LRX_OK) return cd.rc;
	void *stage = nullptr;
	lrx_status rc = stage_address(dev, &stage);
	if (rc != LRX_OK) return rc;
	cudaStream_t st = (cudaStream_t)stream;
	rc = enqueue_call(scene, static_cast<unsigned char *>(stage), h_rays, h_hits, count, mode, st);
	// One exit, with the lock still held: whatever was enqueued -- copies into
	// the staging area or the caller's hit buffer, the trace -- has finished
	// before the next call may reuse the array or the caller reads its hits.
	const cudaError_t e = cudaStreamSynchronize(st);
	if (rc != LRX_OK) return rc;
	if (e != cudaSuccess) return cuda_fail(e, "lrx_trace_host_noalloc: cudaStreamSynchronize");
	return LRX_OK;
}
