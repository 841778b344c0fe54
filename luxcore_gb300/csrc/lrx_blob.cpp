// Scene content keys and built-scene blobs of liblrx.so: lrx_scene_key,
// lrx_scene_save and lrx_scene_load (declared in include/lrx.h).  A blob
// holds a built scene's device arrays and host metadata, so a cache of built
// scenes can skip the BVH build.
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

extern "C++" {
namespace {

// 64-bit mixing hash over bytes, 8 at a time (a cache key, not a checksum
// against adversaries).
struct Hash64 {
	uint64_t h = 0x6a09e667f3bcc909ull;
	void words(const void *p, size_t n) {
		const unsigned char *b = static_cast<const unsigned char *>(p);
		size_t i = 0;
		for (; i + 8 <= n; i += 8) {
			uint64_t w;
			std::memcpy(&w, b + i, 8);
			mix(w);
		}
		uint64_t tail = 0;
		std::memcpy(&tail, b + i, n - i);
		mix(tail ^ ((uint64_t)(n - i) << 56));
	}
	template <class T> void value(const T &v) { words(&v, sizeof(v)); }
	void mix(uint64_t w) {
		h ^= w + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
		h *= 0xff51afd7ed558ccdull;
		h ^= h >> 33;
	}
};

constexpr char kBlobMagic[8] = {'L', 'R', 'X', 'S', 'C', 'E', 'N', 'E'};
constexpr uint32_t kBlobVersion = 4;  // 3: the trace configs carry the failure bounds; 4: the node record

struct BlobWriter {
	unsigned char *p;  // null: only count
	size_t n = 0;
	void bytes(const void *src, size_t k) {
		if (p) std::memcpy(p + n, src, k);
		n += k;
	}
	template <class T> void value(const T &v) { bytes(&v, sizeof(v)); }
	template <class T> void vec(const std::vector<T> &v) {
		value((uint64_t)v.size());
		if (!v.empty()) bytes(v.data(), sizeof(T) * v.size());
	}
};

struct BlobReader {
	const unsigned char *p;
	size_t size, n = 0;
	bool ok = true;
	const unsigned char *take(size_t k) {
		if (!ok || k > size - n) {
			ok = false;
			return nullptr;
		}
		const unsigned char *q = p + n;
		n += k;
		return q;
	}
	template <class T> T value() {
		T v{};
		const unsigned char *q = take(sizeof(T));
		if (q) std::memcpy(&v, q, sizeof(T));
		return v;
	}
	template <class T> bool vec(std::vector<T> &v, uint64_t max_items) {
		const uint64_t k = value<uint64_t>();
		if (!ok || k > max_items) return ok = false;
		v.resize(k);
		const unsigned char *q = take(sizeof(T) * k);
		if (q && k) std::memcpy(v.data(), q, sizeof(T) * k);
		return ok;
	}
};

}  // namespace
}  // extern "C++"

lrx_status lrx_scene_key(const lrx_mesh_desc *meshes, uint32_t mesh_count, const lrx_object_desc *objects,
		uint32_t object_count, const lrx_build_opts *opts, uint64_t *key) {
	if (!key || (mesh_count && !meshes) || (object_count && !objects)) {
		set_error("lrx_scene_key: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	Hash64 h;
	h.value(mesh_count);
	for (uint32_t i = 0; i < mesh_count; ++i) {
		const lrx_mesh_desc &m = meshes[i];
		if ((m.vertex_count && !m.vertices) || (m.triangle_count && !m.triangles)) {
			set_error("lrx_scene_key: mesh " + std::to_string(i) + " has null arrays");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		h.value(m.vertex_count);
		h.value(m.triangle_count);
		h.words(m.vertices, sizeof(float) * 3 * (size_t)m.vertex_count);
		h.words(m.triangles, sizeof(uint32_t) * 3 * (size_t)m.triangle_count);
	}
	h.value(objects ? object_count : mesh_count);
	for (uint32_t i = 0; objects && i < object_count; ++i) {
		const lrx_object_desc &o = objects[i];
		h.value(o.mesh);
		h.value(o.flags);
		if (o.flags & LRX_OBJECT_INSTANCE) h.words(o.transform, sizeof(o.transform));
		if ((o.flags & LRX_OBJECT_INSTANCE) && (o.flags & LRX_OBJECT_HAS_INVERSE)) h.words(o.inverse, sizeof(o.inverse));
	}
	const lrx_build_opts o = read_build_opts(opts);  // over the lrx_scene_create defaults
	h.value(o.leaf_max);
	h.value(o.treelet_passes);
	if (o.node_width != 8) h.value(o.node_width);  // keys of default-width scenes as before
	if (o.node_layout != LRX_NODES_WIDE8) h.value(o.node_layout);  // and of 80-byte-record scenes
	*key = h.h;
	return LRX_OK;
}

// Blob layout: magic, version, checksum of everything after it, the host
// metadata, then the node, triangle and instance arrays (each a u64 byte
// count and the bytes), copied straight between the blob and device memory.
extern "C++" {
static void write_meta(const lrx_scene *s, BlobWriter &w) {
	w.value((uint32_t)(s->two_level ? 1u : 0u));
	w.value(s->root);
	w.vec(s->blas);
	w.vec(s->obj_blas);
	w.vec(s->obj_flags);
	w.value(s->mesh_count);
	w.value(s->plain_blas);
	w.value(s->tlas_node_offset);
	w.value(s->tlas_capacity);
	w.value(s->blas_node_total);
	w.value(s->opts);
	w.value(s->tcfg[0]);
	w.value(s->tcfg[1]);
	w.value(s->info);
	w.value(s->bounds_lo);
	w.value(s->bounds_hi);
	w.vec(s->obj_motion);
	w.value((uint64_t)s->motions.size());
	for (const lrx_scene::Motion &mo : s->motions) {
		w.value(mo.offset16);
		w.value((uint32_t)(mo.have_box ? 1u : 0u));
		w.value(mo.lo);
		w.value(mo.hi);
		w.vec(mo.its);
	}
}
}  // extern "C++"

static size_t blob_size(const lrx_scene *s) {
	BlobWriter w{nullptr};
	write_meta(s, w);
	return 20 + w.n + 3 * 8 + s->nodes.bytes + s->tris.bytes + s->insts.bytes;
}

lrx_status lrx_scene_save(const lrx_scene *s_, void *blob, size_t *bytes, void *stream) {
	if (!s_ || !bytes) {
		set_error("lrx_scene_save: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	lrx_scene *s = const_cast<lrx_scene *>(s_);
	std::lock_guard<std::mutex> lk(s->mu);
	const size_t need = blob_size(s);
	if (!blob) {
		*bytes = need;
		return LRX_OK;
	}
	if (*bytes < need) {
		set_error("lrx_scene_save: buffer too small (" + std::to_string(need) + " bytes needed)");
		*bytes = need;
		return LRX_ERR_INVALID_ARGUMENT;
	}
	DeviceGuard g(s->device);
	cudaStream_t st = (cudaStream_t)stream;
	unsigned char *out = static_cast<unsigned char *>(blob);
	BlobWriter w{out};
	w.bytes(kBlobMagic, 8);
	w.value(kBlobVersion);
	w.value((uint64_t)0);  // checksum, below
	write_meta(s, w);
	for (const DevBuf *d : {&s->nodes, &s->tris, &s->insts}) {
		w.value((uint64_t)d->bytes);
		if (d->bytes) LRX_CUDA(cudaMemcpyAsync(out + w.n, d->ptr, d->bytes, cudaMemcpyDeviceToHost, st));
		w.n += d->bytes;
	}
	LRX_CUDA(cudaStreamSynchronize(st));
	Hash64 h;
	h.words(out + 20, w.n - 20);
	std::memcpy(out + 12, &h.h, 8);
	*bytes = w.n;
	return LRX_OK;
}

// Creates a scene from a blob; verify = false skips the checksum (the
// server's own cache of blobs it wrote).
static lrx_status scene_from_blob(const void *blob, size_t bytes, cudaStream_t st, bool verify, lrx_scene **out_scene) {
	*out_scene = nullptr;
	const unsigned char *b = static_cast<const unsigned char *>(blob);
	if (bytes < 20 || std::memcmp(b, kBlobMagic, 8) != 0) {
		set_error("lrx_scene_load: not a scene blob");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	uint32_t version;
	uint64_t sum;
	std::memcpy(&version, b + 8, 4);
	std::memcpy(&sum, b + 12, 8);
	if (version != kBlobVersion) {
		set_error("lrx_scene_load: blob version " + std::to_string(version) + " is not supported");
		return LRX_ERR_NOT_SUPPORTED;
	}
	if (verify) {
		Hash64 h;
		h.words(b + 20, bytes - 20);
		if (h.h != sum) {
			set_error("lrx_scene_load: checksum mismatch (corrupt or truncated blob)");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	}
	int dev = 0;
	LRX_CUDA(cudaGetDevice(&dev));
	try {
		lrx_scene *s = new lrx_scene();
		std::unique_ptr<lrx_scene> guard(s);
		s->device = dev;
		BlobReader r{b + 20, bytes - 20};
		const uint64_t lim = bytes;  // no vector can hold more items than the blob has bytes
		s->two_level = r.value<uint32_t>() != 0;
		s->root = r.value<uint32_t>();
		r.vec(s->blas, lim);
		r.vec(s->obj_blas, lim);
		r.vec(s->obj_flags, lim);
		s->mesh_count = r.value<uint32_t>();
		s->plain_blas = r.value<uint32_t>();
		s->tlas_node_offset = r.value<uint32_t>();
		s->tlas_capacity = r.value<uint32_t>();
		s->blas_node_total = r.value<uint32_t>();
		s->opts = r.value<lrx_build_opts>();
		s->tcfg[0] = r.value<lrx_trace_config>();
		s->tcfg[1] = r.value<lrx_trace_config>();
		s->info = r.value<lrx_scene_info>();
		for (int c = 0; c < 3; ++c) s->bounds_lo[c] = r.value<float>();
		for (int c = 0; c < 3; ++c) s->bounds_hi[c] = r.value<float>();
		r.vec(s->obj_motion, lim);
		const uint64_t n_motion = r.value<uint64_t>();
		if (n_motion > lim) r.ok = false;
		for (uint64_t k = 0; r.ok && k < n_motion; ++k) {
			lrx_scene::Motion mo;
			mo.offset16 = r.value<uint32_t>();
			mo.have_box = r.value<uint32_t>() != 0;
			for (int c = 0; c < 3; ++c) mo.lo[c] = r.value<float>();
			for (int c = 0; c < 3; ++c) mo.hi[c] = r.value<float>();
			r.vec(mo.its, lim);
			if (mo.its.size() < 2) r.ok = false;
			s->motions.push_back(std::move(mo));
		}
		const unsigned char *arr[3];
		uint64_t len[3];
		for (int k = 0; k < 3; ++k) {
			len[k] = r.value<uint64_t>();
			arr[k] = r.take(len[k]);
		}
		const uint64_t nb = node_record_bytes(s->opts);
		if (!r.ok || r.n != r.size || s->opts.node_layout > LRX_NODES_COMPACT4 ||
				(s->opts.node_layout == LRX_NODES_COMPACT4 && s->two_level) || len[0] % nb ||
				len[1] % sizeof(TriRecord) || len[2] % 16 || s->obj_blas.size() != s->obj_flags.size() ||
				s->obj_motion.size() != s->obj_flags.size() || (s->root != kNull && (uint64_t)s->root * nb >= len[0])) {
			set_error("lrx_scene_load: malformed blob");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		lrx_status rc;
		if ((rc = s->nodes.alloc(std::max<size_t>(len[0], nb))) != LRX_OK) return rc;
		if ((rc = s->tris.alloc(std::max<size_t>(len[1], sizeof(TriRecord)))) != LRX_OK) return rc;
		if (len[2] && (rc = s->insts.alloc(len[2])) != LRX_OK) return rc;
		if ((rc = s->status.alloc(64)) != LRX_OK) return rc;
		LRX_CUDA(cudaMemsetAsync(s->status.ptr, 0, 64, st));
		DevBuf *dst[3] = {&s->nodes, &s->tris, &s->insts};
		for (int k = 0; k < 3; ++k)
			if (len[k]) LRX_CUDA(cudaMemcpyAsync(dst[k]->ptr, arr[k], len[k], cudaMemcpyHostToDevice, st));
		LRX_CUDA(cudaStreamSynchronize(st));
		s->info.device_bytes = s->nodes.bytes + s->tris.bytes + s->insts.bytes + s->status.bytes;
		*out_scene = guard.release();
		return LRX_OK;
	} catch (const std::bad_alloc &) {
		set_error("lrx_scene_load: host allocation failed");
		return LRX_ERR_OUT_OF_MEMORY;
	}
}

lrx_status lrx_scene_load(const void *blob, size_t bytes, void *stream, lrx_scene **out_scene) {
	if (!blob || !out_scene) {
		set_error("lrx_scene_load: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	return scene_from_blob(blob, bytes, (cudaStream_t)stream, true, out_scene);
}

extern "C++" lrx_status lrx::scene_load_trusted(const void *blob, size_t bytes, cudaStream_t stream,
		lrx_scene **out_scene) {
	return scene_from_blob(blob, bytes, stream, false, out_scene);
}

}  // extern "C"
