// Ray reordering before traversal.  Rays are keyed by direction octant and
// the Morton code of their origin inside the scene box, radix-sorted (stable),
// and traced through the resulting index list; hits are written back to each
// ray's own slot, so the caller sees the same order as without sorting.
// Rays in one warp then share a direction octant (the same child order in
// every node) and start close together, which keeps lanes on similar paths.
//
// Scratch (keys, indices, sort temp) comes from a library-owned stream-ordered
// memory pool: allocation and release are ordered on the caller's stream, so
// concurrent calls on one scene do not share scratch and nothing synchronises
// the device.  A caller may lend a region of its own instead (FixedScratch),
// and then nothing is allocated.
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "lrx_common.cuh"
#include "lrx_internal.h"

namespace lrx {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

}  // namespace

lrx_status stream_pool(int dev, cudaMemPool_t *out) {
	if (dev < 0 || dev >= kMaxDevices) {
		set_error("device index out of range");
		return LRX_ERR_NOT_SUPPORTED;
	}
	std::lock_guard<std::mutex> lk(g_pool_mu);
	if (!g_pool[dev]) {
		cudaMemPoolProps props = {};
		props.allocType = cudaMemAllocationTypePinned;
		props.location.type = cudaMemLocationTypeDevice;
		props.location.id = dev;
		cudaMemPool_t p;
		LRX_CUDA(cudaMemPoolCreate(&p, &props));
		uint64_t keep = UINT64_MAX;  // keep freed blocks for the next call
		LRX_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
		g_pool[dev] = p;
	}
	*out = g_pool[dev];
	return LRX_OK;
}

namespace {

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
	v &= 0x3ffu;
	v = (v | (v << 16)) & 0x030000ffu;
	v = (v | (v << 8)) & 0x0300f00fu;
	v = (v | (v << 4)) & 0x030c30c3u;
	v = (v | (v << 2)) & 0x09249249u;
	return v;
}

// key = octant (3 bits) << 27 | Morton code of the origin (9 bits per axis)
__global__ void k_ray_keys(const float4 *__restrict__ rays, uint32_t n, float3 lo, float3 inv_ext,
		uint32_t *__restrict__ keys, uint32_t *__restrict__ idx) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float4 r0 = __ldcs(rays + 3 * (size_t)i), r1 = __ldcs(rays + 3 * (size_t)i + 1);
	const uint32_t oct = (__float_as_uint(r0.w) >> 31) | ((__float_as_uint(r1.x) >> 31) << 1) |
			((__float_as_uint(r1.y) >> 31) << 2);
	auto q = [](float v, float l, float s) {
		const float u = (v - l) * s;
		return u > 0.f ? (u < 511.f ? (uint32_t)u : 511u) : 0u;  // NaN -> 0
	};
	const uint32_t m = (spread10(q(r0.x, lo.x, inv_ext.x)) << 2) | (spread10(q(r0.y, lo.y, inv_ext.y)) << 1) |
			spread10(q(r0.z, lo.z, inv_ext.z));
	keys[i] = (oct << 27) | (m & 0x07ffffffu);
	idx[i] = i;
}

// Queue-launch keys: batch index j above the 30-bit ray key, so one stable
// sort leaves each batch's permutation at its own offset.
__global__ void k_ray_keys_batch(const float4 *__restrict__ rays, uint32_t n, float3 lo, float3 inv_ext,
		uint64_t j, uint32_t key_mask, uint64_t *__restrict__ keys, uint32_t *__restrict__ idx) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float4 r0 = __ldcs(rays + 3 * (size_t)i), r1 = __ldcs(rays + 3 * (size_t)i + 1);
	const uint32_t oct = (__float_as_uint(r0.w) >> 31) | ((__float_as_uint(r1.x) >> 31) << 1) |
			((__float_as_uint(r1.y) >> 31) << 2);
	auto q = [](float v, float l, float s) {
		const float u = (v - l) * s;
		return u > 0.f ? (u < 511.f ? (uint32_t)u : 511u) : 0u;  // NaN -> 0
	};
	const uint32_t m = (spread10(q(r0.x, lo.x, inv_ext.x)) << 2) | (spread10(q(r0.y, lo.y, inv_ext.y)) << 1) |
			spread10(q(r0.z, lo.z, inv_ext.z));
	keys[i] = (j << 30) | (((oct << 27) | (m & 0x07ffffffu)) & key_mask);
	idx[i] = i;
}

float3 key_scale(const float lo[3], const float hi[3]) {
	return make_float3(hi[0] > lo[0] ? 512.f / (hi[0] - lo[0]) : 0.f, hi[1] > lo[1] ? 512.f / (hi[1] - lo[1]) : 0.f,
			hi[2] > lo[2] ? 512.f / (hi[2] - lo[2]) : 0.f);
}

}  // namespace

lrx_status sort_queue_batches(const std::vector<SortBatch> &batches, uint32_t total, cudaStream_t st,
		const uint32_t **order, void **scratch) {
	*order = nullptr;
	*scratch = nullptr;
	if (batches.empty() || total == 0) return LRX_OK;
	int dev = 0;
	LRX_CUDA(cudaGetDevice(&dev));
	cudaMemPool_t pool;
	lrx_status rc = stream_pool(dev, &pool);
	if (rc != LRX_OK) return rc;
	int end_bit = 30;
	while ((1ull << (end_bit - 30)) < batches.size()) ++end_bit;
	size_t temp_bytes = 0;
	{
		cub::DoubleBuffer<uint64_t> dk(nullptr, nullptr);
		cub::DoubleBuffer<uint32_t> dv(nullptr, nullptr);
		LRX_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, dk, dv, (int)total, 0, end_bit, st));
	}
	auto round = [](size_t b) { return ((b + 255) / 256) * 256; };
	const size_t k_arr = round(sizeof(uint64_t) * (size_t)total), v_arr = round(sizeof(uint32_t) * (size_t)total);
	void *base = nullptr;
	LRX_CUDA(cudaMallocFromPoolAsync(&base, 2 * k_arr + 2 * v_arr + temp_bytes, pool, st));
	unsigned char *p = static_cast<unsigned char *>(base);
	uint64_t *k0 = reinterpret_cast<uint64_t *>(p), *k1 = reinterpret_cast<uint64_t *>(p + k_arr);
	uint32_t *v0 = reinterpret_cast<uint32_t *>(p + 2 * k_arr), *v1 = reinterpret_cast<uint32_t *>(p + 2 * k_arr + v_arr);
	void *temp = p + 2 * k_arr + 2 * v_arr;
	cudaError_t e = cudaSuccess;
	for (size_t j = 0; j < batches.size() && e == cudaSuccess; ++j) {
		const SortBatch &b = batches[j];
		const float3 l = make_float3(b.lo[0], b.lo[1], b.lo[2]);
		k_ray_keys_batch<<<(b.count + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float4 *>(b.rays), b.count, l,
				key_scale(b.lo, b.hi), (uint64_t)j, b.octant_only ? 0x38000000u : 0x3fffffffu, k0 + b.offset,
				v0 + b.offset);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) {
		cub::DoubleBuffer<uint64_t> dk(k0, k1);
		cub::DoubleBuffer<uint32_t> dv(v0, v1);
		e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, dk, dv, (int)total, 0, end_bit, st);
		if (e == cudaSuccess) *order = dv.Current();
	}
	if (e != cudaSuccess) {
		cudaFreeAsync(base, st);
		return cuda_fail(e, "queue ray sort");
	}
	*scratch = base;
	return LRX_OK;
}

// Stable selection predicate: ray i is traced unless RAY_FLAGS_MASKED is set
// (its flags word is the 10th of the 12-word record).
struct RayUnmasked {
	const uint32_t *words;
	__device__ __forceinline__ bool operator()(uint32_t i) const {
		return (__ldg(words + 12 * (size_t)i + 9) & LRX_RAY_FLAGS_MASKED) == 0u;
	}
};

lrx_status launch_trace_compacted(const TraceArgs &a_in, cudaStream_t st, const FixedScratch *fixed) {
	TraceArgs a = a_in;
	const uint32_t n = a.count;
	const RayUnmasked pred{static_cast<const uint32_t *>(a.rays)};
	thrust::counting_iterator<uint32_t> first(0u);
	size_t temp_bytes = 0;
	LRX_CUDA(cub::DeviceSelect::If(nullptr, temp_bytes, first, static_cast<uint32_t *>(nullptr),
			static_cast<uint32_t *>(nullptr), (int)n, pred, st));
	const size_t idx_bytes = ((sizeof(uint32_t) * (size_t)n + 255) / 256) * 256;
	const size_t total = idx_bytes + 256 + temp_bytes;
	void *base = nullptr;
	if (fixed) {
		if (total > fixed->bytes) {
			set_error("ray compaction: " + std::to_string(total) + " scratch bytes needed, " +
					std::to_string(fixed->bytes) + " lent");
			return LRX_ERR_NOT_SUPPORTED;
		}
		base = fixed->base;
	} else {
		int dev = 0;
		LRX_CUDA(cudaGetDevice(&dev));
		cudaMemPool_t pool;
		lrx_status prc = stream_pool(dev, &pool);
		if (prc != LRX_OK) return prc;
		LRX_CUDA(cudaMallocFromPoolAsync(&base, total, pool, st));
	}
	unsigned char *p = static_cast<unsigned char *>(base);
	uint32_t *idx = reinterpret_cast<uint32_t *>(p);
	uint32_t *n_sel = reinterpret_cast<uint32_t *>(p + idx_bytes);
	lrx_status rc = LRX_OK;
	cudaError_t e = cub::DeviceSelect::If(p + idx_bytes + 256, temp_bytes, first, idx, n_sel, (int)n, pred, st);
	if (e == cudaSuccess) {
		a.order = idx;
		a.count_dev = n_sel;
		rc = launch_trace(a, st);
	}
	if (!fixed) cudaFreeAsync(base, st);  // ordered after the trace on the same stream
	if (e != cudaSuccess) return cuda_fail(e, "ray compaction");
	return rc;
}

lrx_status launch_trace_sorted(const TraceArgs &a_in, const float lo[3], const float hi[3], cudaStream_t st,
		const FixedScratch *fixed) {
	TraceArgs a = a_in;
	const uint32_t n = a.count;

	// octant-only keys sort in one pass and keep caller order inside an octant
	const int begin_bit = (a.variant & kVarSortOctantOnly) ? 27 : 0;
	size_t temp_bytes = 0;
	{
		cub::DoubleBuffer<uint32_t> dk(nullptr, nullptr), dv(nullptr, nullptr);
		LRX_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, dk, dv, (int)n, begin_bit, 30, st));
	}
	const size_t arr = sorted_scratch_arrays(n) / 4;
	const size_t total = 4 * arr + temp_bytes;
	void *base = nullptr;
	if (fixed) {
		if (total > fixed->bytes) {
			set_error("ray sort: " + std::to_string(total) + " scratch bytes needed, " +
					std::to_string(fixed->bytes) + " lent");
			return LRX_ERR_NOT_SUPPORTED;
		}
		base = fixed->base;
	} else {
		int dev = 0;
		LRX_CUDA(cudaGetDevice(&dev));
		if (dev < 0 || dev >= kMaxDevices) return launch_trace(a, st);
		cudaMemPool_t pool;
		lrx_status prc = stream_pool(dev, &pool);
		if (prc != LRX_OK) return prc;
		LRX_CUDA(cudaMallocFromPoolAsync(&base, total, pool, st));
	}
	unsigned char *p = static_cast<unsigned char *>(base);
	uint32_t *k0 = reinterpret_cast<uint32_t *>(p), *k1 = reinterpret_cast<uint32_t *>(p + arr);
	uint32_t *v0 = reinterpret_cast<uint32_t *>(p + 2 * arr), *v1 = reinterpret_cast<uint32_t *>(p + 3 * arr);
	void *temp = p + 4 * arr;

	lrx_status rc = LRX_OK;
	float3 l = make_float3(lo[0], lo[1], lo[2]);
	float3 s = key_scale(lo, hi);
	k_ray_keys<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float4 *>(a.rays), n, l, s, k0, v0);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) {
		cub::DoubleBuffer<uint32_t> dk(k0, k1), dv(v0, v1);
		e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, dk, dv, (int)n, begin_bit, 30, st);
		if (e == cudaSuccess) {
			a.order = dv.Current();
			rc = launch_trace(a, st);
		}
	}
	if (!fixed) cudaFreeAsync(base, st);  // ordered after the trace on the same stream
	if (e != cudaSuccess) return cuda_fail(e, "ray sort");
	return rc;
}

}  // namespace lrx
