// C-ABI layer of liblrx.so: scene assembly on the device, instance
// transforms, tracing entry points and error reporting.  Declarations and
// the reference interfaces each entry point replaces are in include/lrx.h.
//
// Compiled with -ffp-contract=off so the host-side FP32 arithmetic below
// (Matrix4x4::Inverse, instance boxes) rounds exactly as the reference's.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "lrx_common.cuh"
#include "lrx_internal.h"

namespace lrx {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

lrx_status cuda_fail(cudaError_t e, const char *what) {
	set_error(std::string(what) + ": " + cudaGetErrorString(e));
	cudaGetLastError();  // clear a non-sticky error
	return e == cudaErrorMemoryAllocation ? LRX_ERR_OUT_OF_MEMORY : LRX_ERR_CUDA;
}

lrx_status DevBuf::alloc(size_t n) {
	if (n <= bytes && ptr) return LRX_OK;
	release();
	if (n == 0) return LRX_OK;
	void *p = nullptr;
	const cudaError_t e = cudaMalloc(&p, n);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
	ptr = p;
	bytes = n;
	return LRX_OK;
}

void DevBuf::release() {
	if (ptr) cudaFree(ptr);
	ptr = nullptr;
	bytes = 0;
}

// Matrix4x4::Inverse (src/luxrays/core/geometry/matrix4x4.cpp:118-170):
// Gauss-Jordan elimination with full pivoting, FP32.  Returns false for a
// singular matrix (the reference throws).
static bool matrix_inverse(const float in[16], float out[16]) {
	int indxc[4], indxr[4];
	int ipiv[4] = {0, 0, 0, 0};
	float minv[4][4];
	std::memcpy(minv, in, sizeof(minv));
	for (int i = 0; i < 4; ++i) {
		int irow = -1, icol = -1;
		float big = 0.f;
		for (int j = 0; j < 4; ++j) {
			if (ipiv[j] == 1) continue;
			for (int k = 0; k < 4; ++k) {
				if (ipiv[k] == 0) {
					if (std::fabs(minv[j][k]) >= big) {
						big = std::fabs(minv[j][k]);
						irow = j;
						icol = k;
					}
				} else if (ipiv[k] > 1) {
					return false;
				}
			}
		}
		if (icol < 0) return false;
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
			if (j == icol) continue;
			const float save = minv[j][icol];
			minv[j][icol] = 0.f;
			for (int k = 0; k < 4; ++k) minv[j][k] -= minv[icol][k] * save;
		}
	}
	for (int j = 3; j >= 0; --j) {
		if (indxr[j] != indxc[j])
			for (int k = 0; k < 4; ++k) std::swap(minv[k][indxr[j]], minv[k][indxc[j]]);
	}
	std::memcpy(out, minv, sizeof(minv));
	return true;
}

bool host_matrix_inverse(const float in[16], float out[16]) { return matrix_inverse(in, out); }

// MachineEpsilon::E (include/luxrays/core/epsilon.h:50-55)
static float machine_eps_host(float v) {
	uint32_t u;
	std::memcpy(&u, &v, 4);
	u += 0x80u;
	float n;
	std::memcpy(&n, &u, 4);
	const float e = std::fabs(n - v);
	return e > 1e-5f ? (e < 1e-1f ? e : 1e-1f) : 1e-5f;
}

// Transform * Point with the w divide (transform.h:118-128)
static void xform_point_host(const float m[16], const float p[3], float out[3]) {
	const float x = p[0], y = p[1], z = p[2];
	float r[3] = {m[0] * x + m[1] * y + m[2] * z + m[3], m[4] * x + m[5] * y + m[6] * z + m[7],
			m[8] * x + m[9] * y + m[10] * z + m[11]};
	const float w = m[12] * x + m[13] * y + m[14] * z + m[15];
	if (w != 1.f) {
		const float inv = 1.f / w;
		r[0] *= inv;
		r[1] *= inv;
		r[2] *= inv;
	}
	out[0] = r[0];
	out[1] = r[1];
	out[2] = r[2];
}

// Expands a world box by MachineEpsilon::E as MBVHAccel::Init does
// (mbvhaccel.cpp:189-193), then one more ulp outward.
static void pad_box(float olo[3], float ohi[3]) {
	float e = 0.f;
	for (int k = 0; k < 3; ++k) e = std::max(e, std::max(machine_eps_host(olo[k]), machine_eps_host(ohi[k])));
	for (int k = 0; k < 3; ++k) {
		olo[k] = std::nextafter(olo[k] - e, -INFINITY);
		ohi[k] = std::nextafter(ohi[k] + e, INFINITY);
	}
}

// World box of an instance: the 8 transformed corners of the BLAS box,
// expanded by MachineEpsilon::E as MBVHAccel::Init does (mbvhaccel.cpp:189-193).
static void instance_box(const float m[16], const float lo[3], const float hi[3], float olo[3], float ohi[3]) {
	for (int k = 0; k < 3; ++k) {
		olo[k] = INFINITY;
		ohi[k] = -INFINITY;
	}
	for (int c = 0; c < 8; ++c) {
		const float p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
		float q[3];
		xform_point_host(m, p, q);
		for (int k = 0; k < 3; ++k) {
			olo[k] = std::min(olo[k], q[k]);
			ohi[k] = std::max(ohi[k], q[k]);
		}
	}
	pad_box(olo, ohi);
}

static float bits_as_float(uint32_t u) {
	float f;
	std::memcpy(&f, &u, 4);
	return f;
}

static bool all_finite(const float *v, int n) {
	for (int i = 0; i < n; ++i)
		if (!std::isfinite(v[i])) return false;
	return true;
}

struct Blas {
	uint32_t mesh = kNull;        // instanced mesh, or kNull for the merged plain BLAS
	uint32_t tri_count = 0;
	uint32_t root = kNull;        // absolute node index
	float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

}  // namespace lrx

using namespace lrx;

struct lrx_scene {
	int device = 0;
	bool two_level = false;
	uint32_t root = kNull;
	DevBuf nodes, tris, insts, status, stage_rays, stage_hits;
	std::vector<Blas> blas;
	std::vector<uint32_t> obj_blas;     // per object: BLAS index, kNull if empty
	std::vector<uint32_t> obj_flags;
	uint32_t mesh_count = 0;
	uint32_t plain_blas = kNull;        // index of the merged plain BLAS
	uint32_t tlas_node_offset = 0;
	uint32_t tlas_capacity = 0;
	uint32_t blas_node_total = 0;
	lrx_build_opts opts{};
	// default launch per mode (closest, any-hit): 64-thread blocks, triangles
	// deferred below 8 lanes (best of a block-size x postpone sweep on the
	// heightfield ray sets).  Closest-hit batches run on persistent warps that
	// refill once 8 lanes are idle (+28 % on incoherent bounce rays there, -4 %
	// on coherent primary rays); any-hit batches are reordered by octant +
	// origin first (+20 % on shadow rays; the sort costs more than it saves on
	// closest-hit rays, and persistent warps add nothing after it)
	lrx_trace_config tcfg[2] = {{sizeof(lrx_trace_config), 64, 8, kVarPersistent, 1, 8},
			{sizeof(lrx_trace_config), 64, 8, kVarSortRays, 2, 0}};
	lrx_scene_info info{};
	BuildScratch scratch;
	std::mutex mu;
	float bounds_lo[3] = {0, 0, 0}, bounds_hi[3] = {0, 0, 0};  // world box of the root
	// motion-blurred instances: per object an index into motions (kNull: none)
	struct Motion {
		std::vector<MotionInterval> its;  // keyframes + 1 intervals (the device gets the first keyframes)
		uint32_t offset16 = 0;            // device copy, in 16-byte units from the instance array's base
		bool have_box = false;
		float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // swept world box, padded
	};
	std::vector<uint32_t> obj_motion;
	std::vector<Motion> motions;
};

int lrx::scene_device(const lrx_scene *scene) { return scene->device; }

namespace {

// Children per wide node of a scene's builds (0 in blobs written before the
// option existed: the 8-wide default).
static uint32_t node_width(const lrx_build_opts &o) {
	return o.node_width ? o.node_width : 8u;
}

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

lrx_status validate_meshes(const lrx_mesh_desc *meshes, uint32_t n) {
	for (uint32_t i = 0; i < n; ++i) {
		const lrx_mesh_desc &m = meshes[i];
		if ((m.vertex_count && !m.vertices) || (m.triangle_count && !m.triangles)) {
			set_error("mesh " + std::to_string(i) + ": null vertex or triangle pointer");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		for (uint64_t k = 0; k < 3ull * m.triangle_count; ++k) {
			if (m.triangles[k] >= m.vertex_count) {
				set_error("mesh " + std::to_string(i) + ": vertex index out of range");
				return LRX_ERR_INVALID_ARGUMENT;
			}
		}
	}
	return LRX_OK;
}

// Instance record rows from the object's world->local matrix.
lrx_status object_inverse(const lrx_object_desc &o, float inv[16]) {
	if (!all_finite(o.transform, 16)) {
		set_error("instance transform is not finite");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (o.flags & LRX_OBJECT_HAS_INVERSE) {
		std::memcpy(inv, o.inverse, 64);
		return LRX_OK;
	}
	if (!matrix_inverse(o.transform, inv)) {
		set_error("singular instance transform");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	return LRX_OK;
}

// Builds one BLAS from a host vertex/index array; appends its nodes and
// triangle records to the staging vectors of device buffers.
struct BlasBuild {
	DevBuf nodes, records;
	uint32_t node_count = 0, tri_count = 0, depth = 0;
};

lrx_status build_blas(lrx_scene *s, const float *h_verts, uint32_t nv, const uint32_t *h_idx, uint32_t nt,
		const uint32_t *h_tri_object, uint32_t object_const, cudaStream_t st, BlasBuild &out, Blas &b) {
	lrx_status rc;
	DevBuf d_v, d_i, d_to, d_lo, d_hi;
	if ((rc = d_v.alloc(12ull * nv)) != LRX_OK) return rc;
	if ((rc = d_i.alloc(12ull * nt)) != LRX_OK) return rc;
	if ((rc = d_lo.alloc(16ull * nt)) != LRX_OK) return rc;
	if ((rc = d_hi.alloc(16ull * nt)) != LRX_OK) return rc;
	LRX_CUDA(cudaMemcpyAsync(d_v.ptr, h_verts, 12ull * nv, cudaMemcpyHostToDevice, st));
	LRX_CUDA(cudaMemcpyAsync(d_i.ptr, h_idx, 12ull * nt, cudaMemcpyHostToDevice, st));
	if (h_tri_object) {
		if ((rc = d_to.alloc(8ull * nt)) != LRX_OK) return rc;
		LRX_CUDA(cudaMemcpyAsync(d_to.ptr, h_tri_object, 8ull * nt, cudaMemcpyHostToDevice, st));
	}
	if ((rc = launch_triangle_boxes(nt, d_v.as<float>(), d_i.as<uint32_t>(), d_lo.as<float4>(), d_hi.as<float4>(), st)) != LRX_OK)
		return rc;
	BvhResult r;
	if ((rc = build_wide_bvh(nt, d_lo.as<float4>(), d_hi.as<float4>(), s->opts.leaf_max, node_width(s->opts),
			     s->opts.treelet_passes, st,
			     s->scratch, &r)) != LRX_OK)
		return rc;
	out.node_count = r.node_count;
	out.tri_count = nt;
	out.depth = r.depth;
	if ((rc = out.nodes.alloc(sizeof(WideNode) * (size_t)r.node_count)) != LRX_OK) return rc;
	if ((rc = out.records.alloc(sizeof(TriRecord) * (size_t)nt)) != LRX_OK) return rc;
	LRX_CUDA(cudaMemcpyAsync(out.nodes.ptr, s->scratch.wide_nodes.ptr, sizeof(WideNode) * (size_t)r.node_count,
			cudaMemcpyDeviceToDevice, st));
	if ((rc = launch_triangle_records(nt, s->scratch.prim_order.as<uint32_t>(), d_v.as<float>(), d_i.as<uint32_t>(),
			     h_tri_object ? d_to.as<uint32_t>() : nullptr, object_const, out.records.as<TriRecord>(), st)) != LRX_OK)
		return rc;
	LRX_CUDA(cudaStreamSynchronize(st));  // the temporaries above are freed on return
	std::memcpy(b.lo, r.lo, sizeof(b.lo));
	std::memcpy(b.hi, r.hi, sizeof(b.hi));
	b.tri_count = nt;
	return LRX_OK;
}

// (Re)builds the TLAS over the non-empty objects and writes it after the
// BLAS nodes.  Called at create and by lrx_scene_update_instances.
lrx_status build_tlas(lrx_scene *s, const lrx_object_desc *objects, uint32_t n_objects, cudaStream_t st) {
	std::vector<InstRecord> recs;
	std::vector<float4> blo, bhi;
	recs.reserve(n_objects + 1);
	{
		// swept boxes of motion instances not bounded yet (1025 samples per
		// interval each), spread over the host's cores
		std::vector<uint32_t> todo;
		for (uint32_t i = 0; i < n_objects; ++i)
			if ((s->obj_flags[i] & LRX_OBJECT_INSTANCE) && s->obj_blas[i] != kNull && s->obj_motion[i] != kNull &&
					!s->motions[s->obj_motion[i]].have_box)
				todo.push_back(i);
		std::atomic<uint32_t> next{0};
		std::atomic<int> failed{0};
		auto work = [&]() {
			for (uint32_t k; (k = next.fetch_add(1)) < todo.size();) {
				const uint32_t i = todo[k];
				const Blas &b = s->blas[s->obj_blas[i]];
				lrx_scene::Motion &mo = s->motions[s->obj_motion[i]];
				if (motion_bound(mo.its, b.lo, b.hi, mo.lo, mo.hi) != LRX_OK) {
					failed = 1;
					continue;
				}
				pad_box(mo.lo, mo.hi);
				mo.have_box = true;
			}
		};
		const uint32_t nt = std::min<uint32_t>((uint32_t)todo.size() / 64 + 1,
				std::max(1u, std::min(32u, std::thread::hardware_concurrency())));
		std::vector<std::thread> pool;
		for (uint32_t t = 1; t < nt; ++t) pool.emplace_back(work);
		work();
		for (std::thread &t : pool) t.join();
		if (failed) {
			set_error("motion system: a sampled matrix is singular");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	}
	if (s->plain_blas != kNull) {
		const Blas &b = s->blas[s->plain_blas];
		InstRecord r{};
		r.r0 = make_float4(1, 0, 0, 0);
		r.r1 = make_float4(0, 1, 0, 0);
		r.r2 = make_float4(0, 0, 1, 0);
		r.r3 = make_float4(0, 0, 0, 1);
		r.info = make_uint4(b.root, kNull, kInstIdentity, 0);
		recs.push_back(r);
		blo.push_back(make_float4(b.lo[0], b.lo[1], b.lo[2], 0));
		bhi.push_back(make_float4(b.hi[0], b.hi[1], b.hi[2], 0));
	}
	for (uint32_t i = 0; i < n_objects; ++i) {
		if (!(s->obj_flags[i] & LRX_OBJECT_INSTANCE)) continue;
		const uint32_t bi = s->obj_blas[i];
		if (bi == kNull) continue;
		const Blas &b = s->blas[bi];
		if (s->obj_motion[i] != kNull) {
			// motion instance: the traversal samples its transform at the ray's time
			const lrx_scene::Motion &mo = s->motions[s->obj_motion[i]];
			InstRecord r{};
			const uint32_t n_its = (uint32_t)mo.its.size() - 1;
			r.r0 = make_float4(bits_as_float(n_its), 0, 0, 0);
			r.info = make_uint4(b.root, i, kInstMotion, mo.offset16);
			recs.push_back(r);
			blo.push_back(make_float4(mo.lo[0], mo.lo[1], mo.lo[2], 0));
			bhi.push_back(make_float4(mo.hi[0], mo.hi[1], mo.hi[2], 0));
			continue;
		}
		float inv[16];
		lrx_status rc = object_inverse(objects[i], inv);
		if (rc != LRX_OK) return rc;
		InstRecord r{};
		r.r0 = make_float4(inv[0], inv[1], inv[2], inv[3]);
		r.r1 = make_float4(inv[4], inv[5], inv[6], inv[7]);
		r.r2 = make_float4(inv[8], inv[9], inv[10], inv[11]);
		r.r3 = make_float4(inv[12], inv[13], inv[14], inv[15]);
		r.info = make_uint4(b.root, i, 0, 0);
		recs.push_back(r);
		float lo[3], hi[3];
		instance_box(objects[i].transform, b.lo, b.hi, lo, hi);
		blo.push_back(make_float4(lo[0], lo[1], lo[2], 0));
		bhi.push_back(make_float4(hi[0], hi[1], hi[2], 0));
	}
	const uint32_t n = (uint32_t)recs.size();
	if (n == 0) {
		s->root = kNull;
		return LRX_OK;
	}
	if (n > s->tlas_capacity) {
		set_error("instance count changed");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	lrx_status rc;
	DevBuf d_lo, d_hi;
	if ((rc = d_lo.alloc(16ull * n)) != LRX_OK) return rc;
	if ((rc = d_hi.alloc(16ull * n)) != LRX_OK) return rc;
	LRX_CUDA(cudaMemcpyAsync(d_lo.ptr, blo.data(), 16ull * n, cudaMemcpyHostToDevice, st));
	LRX_CUDA(cudaMemcpyAsync(d_hi.ptr, bhi.data(), 16ull * n, cudaMemcpyHostToDevice, st));
	BvhResult r;
	if ((rc = build_wide_bvh(n, d_lo.as<float4>(), d_hi.as<float4>(), 1, node_width(s->opts), s->opts.treelet_passes, st,
			     s->scratch, &r)) != LRX_OK)
		return rc;
	std::vector<uint32_t> order(n);
	LRX_CUDA(cudaMemcpyAsync(order.data(), s->scratch.prim_order.ptr, 4ull * n, cudaMemcpyDeviceToHost, st));
	LRX_CUDA(cudaStreamSynchronize(st));
	std::vector<InstRecord> sorted(n);
	for (uint32_t k = 0; k < n; ++k) sorted[k] = recs[order[k]];
	LRX_CUDA(cudaMemcpyAsync(s->insts.ptr, sorted.data(), sizeof(InstRecord) * n, cudaMemcpyHostToDevice, st));
	if ((rc = launch_relocate_nodes(s->scratch.wide_nodes.as<WideNode>(), s->nodes.as<WideNode>() + s->tlas_node_offset,
			     r.node_count, s->tlas_node_offset, 0, st)) != LRX_OK)
		return rc;
	LRX_CUDA(cudaStreamSynchronize(st));
	s->root = s->tlas_node_offset;
	std::memcpy(s->bounds_lo, r.lo, sizeof(r.lo));
	std::memcpy(s->bounds_hi, r.hi, sizeof(r.hi));
	s->info.node_count = s->blas_node_total + r.node_count;
	s->info.max_depth = std::max(s->info.max_depth, r.depth);
	return LRX_OK;
}

}  // namespace

extern "C" {

uint32_t lrx_abi_version(void) { return LRX_ABI_VERSION; }

const char *lrx_last_error(void) { return g_last_error.c_str(); }

lrx_status lrx_scene_create(const lrx_mesh_desc *meshes, uint32_t mesh_count, const lrx_object_desc *objects,
		uint32_t object_count, const lrx_build_opts *opts, void *stream, lrx_scene **out_scene) {
	return lrx_scene_create_motion(meshes, mesh_count, objects, object_count, nullptr, 0, opts, stream, out_scene);
}

lrx_status lrx_scene_create_motion(const lrx_mesh_desc *meshes, uint32_t mesh_count, const lrx_object_desc *objects,
		uint32_t object_count, const lrx_motion_desc *motions, uint32_t motion_count, const lrx_build_opts *opts,
		void *stream, lrx_scene **out_scene) {
	try {
		if (!out_scene || (mesh_count && !meshes) || (motion_count && !motions)) {
			set_error("lrx_scene_create: null argument");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		*out_scene = nullptr;
		int dev = 0;
		LRX_CUDA(cudaGetDevice(&dev));
		cudaDeviceProp prop;
		LRX_CUDA(cudaGetDeviceProperties(&prop, dev));
		if (prop.major < 10) {
			set_error("lrx needs a Blackwell (sm_103) device");
			return LRX_ERR_NOT_SUPPORTED;
		}
		lrx_status rc = validate_meshes(meshes, mesh_count);
		if (rc != LRX_OK) return rc;
		std::vector<lrx_object_desc> objs;
		if (objects) {
			objs.assign(objects, objects + object_count);
		} else {
			objs.resize(mesh_count);
			for (uint32_t i = 0; i < mesh_count; ++i) {
				std::memset(&objs[i], 0, sizeof(lrx_object_desc));
				objs[i].mesh = i;
			}
		}
		const uint32_t n_obj = (uint32_t)objs.size();
		std::vector<uint32_t> obj_motion(n_obj, kNull);
		std::vector<lrx_scene::Motion> motion_list(motion_count);
		for (uint32_t k = 0; k < motion_count; ++k) {
			const lrx_motion_desc &md = motions[k];
			if (md.object >= n_obj || !(objs[md.object].flags & LRX_OBJECT_INSTANCE) || obj_motion[md.object] != kNull) {
				set_error("motion " + std::to_string(k) + ": object out of range, not an instance, or given twice");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			if ((rc = motion_intervals(md.times, md.transforms, md.count, motion_list[k].its)) != LRX_OK) return rc;
			obj_motion[md.object] = k;
		}
		for (uint32_t i = 0; i < n_obj; ++i) {
			if (objs[i].mesh >= mesh_count) {
				set_error("object " + std::to_string(i) + ": mesh index out of range");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			if ((objs[i].flags & LRX_OBJECT_INSTANCE) && obj_motion[i] == kNull) {
				float inv[16];
				if ((rc = object_inverse(objs[i], inv)) != LRX_OK) return rc;
			}
		}

		lrx_scene *s = new lrx_scene();
		std::unique_ptr<lrx_scene> guard(s);
		s->obj_motion = std::move(obj_motion);
		s->motions = std::move(motion_list);
		s->device = dev;
		s->mesh_count = mesh_count;
		s->opts.struct_size = sizeof(lrx_build_opts);
		s->opts.leaf_max = 3;
		s->opts.treelet_passes = 2;
		s->opts.node_width = 8;
		if (opts && opts->struct_size >= sizeof(lrx_build_opts)) {
			if (opts->leaf_max) s->opts.leaf_max = std::min(3u, opts->leaf_max);
			s->opts.treelet_passes = opts->treelet_passes;
			if (opts->node_width) s->opts.node_width = opts->node_width;
		}
		if (s->opts.node_width < 4 || s->opts.node_width > 8) {
			set_error("lrx_scene_create: node_width must be 0 or in [4, 8]");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		cudaStream_t st = (cudaStream_t)stream;
		const auto t0 = std::chrono::steady_clock::now();

		s->obj_flags.resize(n_obj);
		s->obj_blas.assign(n_obj, kNull);
		bool any_inst = false;
		for (uint32_t i = 0; i < n_obj; ++i) {
			s->obj_flags[i] = objs[i].flags;
			any_inst |= (objs[i].flags & LRX_OBJECT_INSTANCE) != 0;
		}
		s->two_level = any_inst;

		std::vector<BlasBuild> builds;
		builds.reserve(mesh_count + 1);
		uint64_t eff_tris = 0, unique_tris = 0;
		uint32_t n_inst = 0;

		// Merged BLAS over all plain objects, in world space.
		{
			uint64_t nv = 0, nt = 0;
			uint32_t n_plain = 0, single = kNull;
			for (uint32_t i = 0; i < n_obj; ++i) {
				if (objs[i].flags & LRX_OBJECT_INSTANCE) continue;
				const lrx_mesh_desc &m = meshes[objs[i].mesh];
				if (!m.triangle_count) continue;
				nv += m.vertex_count;
				nt += m.triangle_count;
				++n_plain;
				single = i;
			}
			if (nt > 0xffffffffull / 3 || nv > 0xffffffffull) {
				set_error("too many triangles in one BVH");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			if (nt) {
				std::vector<float> cv;
				std::vector<uint32_t> ci, to;
				const float *pv;
				const uint32_t *pi;
				const uint32_t *pto = nullptr;
				uint32_t oc = kNull;
				if (n_plain == 1) {
					const lrx_mesh_desc &m = meshes[objs[single].mesh];
					pv = m.vertices;
					pi = m.triangles;
					oc = single;
				} else {
					cv.reserve(3 * nv);
					ci.reserve(3 * nt);
					to.reserve(2 * nt);
					for (uint32_t i = 0; i < n_obj; ++i) {
						if (objs[i].flags & LRX_OBJECT_INSTANCE) continue;
						const lrx_mesh_desc &m = meshes[objs[i].mesh];
						if (!m.triangle_count) continue;
						const uint32_t base = (uint32_t)(cv.size() / 3);
						cv.insert(cv.end(), m.vertices, m.vertices + 3ull * m.vertex_count);
						for (uint64_t k = 0; k < 3ull * m.triangle_count; ++k) ci.push_back(m.triangles[k] + base);
						for (uint32_t k = 0; k < m.triangle_count; ++k) {
							to.push_back(i);
							to.push_back(k);
						}
					}
					pv = cv.data();
					pi = ci.data();
					pto = to.data();
				}
				Blas b;
				builds.emplace_back();
				if ((rc = build_blas(s, pv, (uint32_t)nv, pi, (uint32_t)nt, pto, oc, st, builds.back(), b)) != LRX_OK)
					return rc;
				s->plain_blas = (uint32_t)s->blas.size();
				s->blas.push_back(b);
				for (uint32_t i = 0; i < n_obj; ++i)
					if (!(objs[i].flags & LRX_OBJECT_INSTANCE) && meshes[objs[i].mesh].triangle_count)
						s->obj_blas[i] = s->plain_blas;
				eff_tris += nt;
				unique_tris += nt;
			}
		}
		// One BLAS per instanced mesh
		std::vector<uint32_t> mesh_blas(mesh_count, kNull);
		for (uint32_t i = 0; i < n_obj; ++i) {
			if (!(objs[i].flags & LRX_OBJECT_INSTANCE)) continue;
			++n_inst;
			const uint32_t mi = objs[i].mesh;
			const lrx_mesh_desc &m = meshes[mi];
			if (!m.triangle_count) continue;
			eff_tris += m.triangle_count;
			if (mesh_blas[mi] == kNull) {
				Blas b;
				b.mesh = mi;
				builds.emplace_back();
				if ((rc = build_blas(s, m.vertices, m.vertex_count, m.triangles, m.triangle_count, nullptr, kNull, st,
						     builds.back(), b)) != LRX_OK)
					return rc;
				mesh_blas[mi] = (uint32_t)s->blas.size();
				s->blas.push_back(b);
				unique_tris += m.triangle_count;
			}
			s->obj_blas[i] = mesh_blas[mi];
		}

		// Concatenate all BLAS into the scene arrays
		uint64_t total_nodes = 0, total_tris = 0;
		uint32_t max_depth = 0;
		for (const BlasBuild &bb : builds) {
			total_nodes += bb.node_count;
			total_tris += bb.tri_count;
			max_depth = std::max(max_depth, bb.depth);
		}
		const uint32_t tlas_prims = s->two_level ? (uint32_t)s->blas.size() + n_inst : 0;
		s->tlas_capacity = tlas_prims;
		if (total_nodes + tlas_prims > 0x7fffffffull) {
			set_error("scene too large");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		if ((rc = s->nodes.alloc(sizeof(WideNode) * (total_nodes + tlas_prims + 1))) != LRX_OK) return rc;
		if ((rc = s->tris.alloc(sizeof(TriRecord) * (total_tris + 1))) != LRX_OK) return rc;
		if ((rc = s->status.alloc(64)) != LRX_OK) return rc;
		LRX_CUDA(cudaMemsetAsync(s->status.ptr, 0, 64, st));
		uint32_t node_off = 0, tri_off = 0;
		for (size_t k = 0; k < builds.size(); ++k) {
			BlasBuild &bb = builds[k];
			if ((rc = launch_relocate_nodes(bb.nodes.as<WideNode>(), s->nodes.as<WideNode>() + node_off, bb.node_count,
					     node_off, tri_off, st)) != LRX_OK)
				return rc;
			LRX_CUDA(cudaMemcpyAsync(s->tris.as<TriRecord>() + tri_off, bb.records.ptr, sizeof(TriRecord) * bb.tri_count,
					cudaMemcpyDeviceToDevice, st));
			s->blas[k].root = node_off;
			node_off += bb.node_count;
			tri_off += bb.tri_count;
		}
		LRX_CUDA(cudaStreamSynchronize(st));
		builds.clear();
		s->blas_node_total = node_off;
		s->tlas_node_offset = node_off;
		s->info.max_depth = max_depth;
		s->info.node_count = node_off;
		if (s->two_level) {
			// instance records, then the motion intervals the traversal samples
			size_t bytes = sizeof(InstRecord) * (tlas_prims + 1);
			for (lrx_scene::Motion &mo : s->motions) {
				mo.offset16 = (uint32_t)(bytes / 16);
				bytes += sizeof(MotionInterval) * (mo.its.size() - 1);
			}
			if (bytes / 16 > 0xffffffffull) {
				set_error("too many motion keyframes");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			if ((rc = s->insts.alloc(bytes)) != LRX_OK) return rc;
			for (const lrx_scene::Motion &mo : s->motions)
				LRX_CUDA(cudaMemcpyAsync(static_cast<char *>(s->insts.ptr) + 16ull * mo.offset16, mo.its.data(),
						sizeof(MotionInterval) * (mo.its.size() - 1), cudaMemcpyHostToDevice, st));
			if ((rc = build_tlas(s, objs.data(), n_obj, st)) != LRX_OK) return rc;
		} else {
			s->root = s->blas.empty() ? kNull : 0u;
			if (!s->blas.empty()) {
				std::memcpy(s->bounds_lo, s->blas[0].lo, sizeof(s->bounds_lo));
				std::memcpy(s->bounds_hi, s->blas[0].hi, sizeof(s->bounds_hi));
			}
		}
		// scratch is kept only where instance updates need it
		if (!s->two_level) s->scratch = BuildScratch();
		const auto t1 = std::chrono::steady_clock::now();

		s->info.triangle_count = eff_tris;
		s->info.unique_triangle_count = unique_tris;
		s->info.object_count = n_obj;
		s->info.instance_count = n_inst;
		s->info.blas_count = (uint32_t)s->blas.size();
		s->info.two_level = s->two_level ? 1u : 0u;
		s->info.device_bytes = s->nodes.bytes + s->tris.bytes + s->insts.bytes + s->status.bytes;
		s->info.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
		*out_scene = guard.release();
		return LRX_OK;
	} catch (const std::bad_alloc &) {
		set_error("host allocation failed");
		return LRX_ERR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		set_error(e.what());
		return LRX_ERR_INVALID_ARGUMENT;
	}
}

lrx_status lrx_scene_destroy(lrx_scene *scene) {
	if (!scene) return LRX_OK;
	DeviceGuard g(scene->device);
	delete scene;
	return LRX_OK;
}

lrx_status lrx_scene_update_instances(lrx_scene *s, const lrx_object_desc *objects, uint32_t object_count, void *stream) {
	if (!s || !objects) {
		set_error("lrx_scene_update_instances: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	std::lock_guard<std::mutex> lk(s->mu);
	DeviceGuard g(s->device);
	if (object_count != s->obj_flags.size()) {
		set_error("object count differs from the scene's");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	for (uint32_t i = 0; i < object_count; ++i) {
		if ((objects[i].flags & LRX_OBJECT_INSTANCE) != (s->obj_flags[i] & LRX_OBJECT_INSTANCE)) {
			set_error("object " + std::to_string(i) + " changed kind");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	}
	if (!s->two_level) return LRX_OK;  // nothing moves in a flat scene
	return build_tlas(s, objects, object_count, (cudaStream_t)stream);
}

lrx_status lrx_scene_get_info(const lrx_scene *s, lrx_scene_info *info) {
	if (!s || !info) {
		set_error("lrx_scene_get_info: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	*info = s->info;
	return LRX_OK;
}

// ---------------------------------------------------------------------------
// Scene keys and blobs (a cache of built scenes)
// ---------------------------------------------------------------------------

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
constexpr uint32_t kBlobVersion = 2;

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
	uint32_t leaf_max = 3, passes = 2, width = 8;  // the lrx_scene_create defaults
	if (opts && opts->struct_size >= sizeof(lrx_build_opts)) {
		if (opts->leaf_max) leaf_max = std::min(3u, opts->leaf_max);
		passes = opts->treelet_passes;
		if (opts->node_width) width = opts->node_width;
	}
	h.value(leaf_max);
	h.value(passes);
	if (width != 8) h.value(width);  // keys of default-width scenes as before
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
		if (!r.ok || r.n != r.size || len[0] % sizeof(WideNode) || len[1] % sizeof(TriRecord) ||
				len[2] % 16 || s->obj_blas.size() != s->obj_flags.size() || s->obj_motion.size() != s->obj_flags.size() ||
				(s->root != kNull && (uint64_t)s->root * sizeof(WideNode) >= len[0])) {
			set_error("lrx_scene_load: malformed blob");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		lrx_status rc;
		if ((rc = s->nodes.alloc(std::max<size_t>(len[0], sizeof(WideNode)))) != LRX_OK) return rc;
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

// A correct walk visits each node at most once per BLAS entry, so a ray never
// needs more than (instances + 1) x nodes visits.
static uint32_t scene_visit_limit(const lrx_scene *s) {
	const uint64_t lim = (uint64_t)(s->info.instance_count + 1) * (s->info.node_count + 1) + 64;
	return (uint32_t)std::min<uint64_t>(lim, kMaxVisits);
}

static lrx_status trace_common(lrx_scene *s, const void *d_rays, void *d_hits, uint32_t count, uint32_t mode,
		uint64_t *d_counters, cudaStream_t st) {
	if (!s) {
		set_error("lrx_trace: null scene");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (mode > LRX_TRACE_ANY) {
		set_error("lrx_trace: unknown mode");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (count == 0) return LRX_OK;
	if (!d_rays || !d_hits) {
		set_error("lrx_trace: null ray or hit buffer");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	if (((uintptr_t)d_rays & 15u) || ((uintptr_t)d_hits & 3u)) {
		set_error("lrx_trace: rays must be 16-byte aligned, hits 4-byte aligned");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	DeviceGuard g(s->device);
	TraceArgs a{};
	a.nodes = s->nodes.as<WideNode>();
	a.tris = s->tris.as<TriRecord>();
	a.insts = s->insts.as<InstRecord>();
	a.root = s->root;
	a.two_level = s->two_level ? 1u : 0u;
	a.motion = s->motions.empty() ? 0u : 1u;
	a.rays = d_rays;
	a.hits = d_hits;
	a.count = count;
	a.any_hit = mode == LRX_TRACE_ANY;
	a.status = s->status.as<uint32_t>();
	a.counters = reinterpret_cast<unsigned long long *>(d_counters);
	a.visit_limit = scene_visit_limit(s);
	const lrx_trace_config &cfg = s->tcfg[mode == LRX_TRACE_ANY ? 1 : 0];
	a.block_size = cfg.block_size;
	a.postpone = cfg.postpone;
	a.variant = cfg.variant;
	a.refill = cfg.refill;
	if ((a.variant & kVarSortRays) && count >= kSortMinRays && s->root != kNull)
		return launch_trace_sorted(a, s->bounds_lo, s->bounds_hi, st);
	if ((a.variant & kVarCompact) && (a.variant & kVarPersistent) && !d_counters && count < 0x80000000u)
		return launch_trace_compacted(a, st);
	return launch_trace(a, st);
}

lrx_status lrx_scene_set_trace_config(lrx_scene *s, const lrx_trace_config *c) {
	if (!s || !c || c->struct_size < offsetof(lrx_trace_config, refill)) {
		set_error("lrx_scene_set_trace_config: null argument or unknown struct size");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	lrx_trace_config in{};  // fields the caller's struct lacks stay 0
	std::memcpy(&in, c, std::min<size_t>(c->struct_size, sizeof(in)));
	const uint32_t bs = in.block_size ? in.block_size : kTraceBlock;
	if (bs < 32 || bs > 512 || (bs & 31) || in.postpone > 32 || (in.variant & ~kVarAll) || in.modes > 3u ||
			in.refill > 32) {
		set_error("lrx_scene_set_trace_config: value out of range");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	const uint32_t modes = in.modes ? in.modes : 3u;
	for (int m = 0; m < 2; ++m) {
		if (!(modes & (1u << m))) continue;
		s->tcfg[m] = in;
		s->tcfg[m].struct_size = sizeof(lrx_trace_config);
		s->tcfg[m].block_size = bs;
		s->tcfg[m].modes = 1u << m;
	}
	return LRX_OK;
}

lrx_status lrx_scene_get_trace_config(const lrx_scene *s, lrx_trace_config *c) {
	if (!s || !c || c->struct_size < offsetof(lrx_trace_config, refill)) {
		set_error("lrx_scene_get_trace_config: null argument or unknown struct size");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	const size_t n = std::min<size_t>(c->struct_size, sizeof(lrx_trace_config));
	std::memcpy(c, &s->tcfg[(c->modes & 2u) ? 1 : 0], n);
	c->struct_size = (uint32_t)n;
	return LRX_OK;
}

lrx_status lrx_scene_autotune(lrx_scene *s, const void *d_rays, uint32_t count, uint32_t mode, void *stream,
		lrx_trace_config *chosen) {
	if (!s || !d_rays || count == 0 || mode > LRX_TRACE_ANY) {
		set_error("lrx_scene_autotune: null scene/rays, empty sample or unknown mode");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	DeviceGuard g(s->device);
	cudaStream_t st = (cudaStream_t)stream;
	cudaMemPool_t pool;
	lrx_status rc = stream_pool(s->device, &pool);
	if (rc != LRX_OK) return rc;
	void *hits = nullptr;
	LRX_CUDA(cudaMallocFromPoolAsync(&hits, sizeof(lrx_hit) * (size_t)count, pool, st));
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	const int m = mode == LRX_TRACE_ANY ? 1 : 0;
	lrx_trace_config best = s->tcfg[m];
	float best_ms = INFINITY;
	// launch shape, ray order, stack placement (local memory or a shared-memory
	// top) and cache policy for the scene's node and triangle arrays
	static const uint32_t kBlocks[] = {32, 64, 128};
	static const uint32_t kPostpone[] = {0, 8};
	static const uint32_t kVariants[] = {0, LRX_VARIANT_STREAM_RAYS, LRX_VARIANT_SORT_RAYS, LRX_VARIANT_PERSISTENT,
			LRX_VARIANT_PERSISTENT | LRX_VARIANT_STREAM_RAYS, LRX_VARIANT_PERSISTENT | LRX_VARIANT_SMEM_STACK,
			LRX_VARIANT_PERSISTENT | LRX_VARIANT_SCENE_L2_KEEP};
	for (uint32_t bs : kBlocks) {
		for (uint32_t pp : kPostpone) {
			for (uint32_t var : kVariants) {
				if ((var & LRX_VARIANT_SORT_RAYS) && count < kSortMinRays) continue;
				s->tcfg[m] = lrx_trace_config{sizeof(lrx_trace_config), bs, pp, var, 1u << m,
							(var & LRX_VARIANT_PERSISTENT) ? 8u : 0u};
				if ((rc = trace_common(s, d_rays, hits, count, mode, nullptr, st)) != LRX_OK) break;
				cudaEventRecord(e0, st);
				for (int r = 0; r < 3 && rc == LRX_OK; ++r) rc = trace_common(s, d_rays, hits, count, mode, nullptr, st);
				cudaEventRecord(e1, st);
				if (rc != LRX_OK || cudaEventSynchronize(e1) != cudaSuccess) break;
				float ms = 0.f;
				cudaEventElapsedTime(&ms, e0, e1);
				if (ms < best_ms) {
					best_ms = ms;
					best = s->tcfg[m];
				}
			}
		}
	}
	s->tcfg[m] = best;
	cudaFreeAsync(hits, st);
	cudaStreamSynchronize(st);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (rc != LRX_OK) return rc;
	if (chosen) {  // as many bytes as the caller's struct holds (ABI 1 struct: no refill field)
		const size_t n = chosen->struct_size >= sizeof(lrx_trace_config) ? sizeof(lrx_trace_config)
				: offsetof(lrx_trace_config, refill);
		std::memcpy(chosen, &best, n);
		chosen->struct_size = (uint32_t)n;
	}
	return LRX_OK;
}

lrx_status lrx_scene_create_autotuned(const lrx_mesh_desc *meshes, uint32_t mesh_count,
		const lrx_object_desc *objects, uint32_t object_count, const lrx_build_opts *opts, const void *d_sample_rays,
		uint32_t sample_count, uint32_t mode, void *stream, lrx_scene **out_scene, lrx_build_opts *chosen_opts,
		lrx_trace_config *chosen_config) {
	if (!out_scene || !d_sample_rays || sample_count == 0 || mode > LRX_TRACE_ANY) {
		set_error("lrx_scene_create_autotuned: null scene or sample, empty sample or unknown mode");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	*out_scene = nullptr;
	lrx_build_opts base{};
	base.struct_size = sizeof(lrx_build_opts);
	base.treelet_passes = 2;
	if (opts && opts->struct_size >= sizeof(lrx_build_opts)) base.treelet_passes = opts->treelet_passes;
	// candidate builds: node width x triangles per leaf
	static const uint32_t kWidths[] = {8, 4};
	static const uint32_t kLeaves[] = {3, 2};
	cudaStream_t st = (cudaStream_t)stream;
	lrx_scene *best = nullptr;
	float best_ms = INFINITY;
	lrx_build_opts best_opts = base;
	lrx_trace_config best_cfg{};
	lrx_status rc = LRX_OK;
	void *hits = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	for (uint32_t w : kWidths) {
		for (uint32_t leaf : kLeaves) {
			lrx_build_opts o = base;
			o.node_width = w;
			o.leaf_max = leaf;
			lrx_scene *cand = nullptr;
			if ((rc = lrx_scene_create(meshes, mesh_count, objects, object_count, &o, stream, &cand)) != LRX_OK) break;
			DeviceGuard g(cand->device);
			if (!hits) {
				cudaMemPool_t pool;
				if ((rc = stream_pool(cand->device, &pool)) == LRX_OK &&
						cudaMallocFromPoolAsync(&hits, sizeof(lrx_hit) * (size_t)sample_count, pool, st) != cudaSuccess)
					rc = cuda_fail(cudaGetLastError(), "cudaMallocFromPoolAsync");
				if (rc == LRX_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
					rc = cuda_fail(cudaGetLastError(), "cudaEventCreate");
			}
			lrx_trace_config cfg{};
			cfg.struct_size = sizeof(cfg);
			if (rc == LRX_OK) rc = lrx_scene_autotune(cand, d_sample_rays, sample_count, mode, stream, &cfg);
			float ms = INFINITY;
			if (rc == LRX_OK) {  // the candidate at its tuned configuration
				for (int r = 0; r < 2 && rc == LRX_OK; ++r)
					rc = trace_common(cand, d_sample_rays, hits, sample_count, mode, nullptr, st);
				cudaEventRecord(e0, st);
				for (int r = 0; r < 5 && rc == LRX_OK; ++r)
					rc = trace_common(cand, d_sample_rays, hits, sample_count, mode, nullptr, st);
				cudaEventRecord(e1, st);
				if (rc == LRX_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
			}
			if (rc != LRX_OK) {
				lrx_scene_destroy(cand);
				break;
			}
			if (ms < best_ms) {
				if (best) lrx_scene_destroy(best);
				best = cand;
				best_ms = ms;
				best_opts = o;
				best_cfg = cfg;
			} else {
				lrx_scene_destroy(cand);
			}
		}
		if (rc != LRX_OK) break;
	}
	if (hits) cudaFreeAsync(hits, st);
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (rc != LRX_OK || !best) {
		if (best) lrx_scene_destroy(best);
		return rc != LRX_OK ? rc : LRX_ERR_BUILD;
	}
	cudaStreamSynchronize(st);
	*out_scene = best;
	if (chosen_opts) *chosen_opts = best_opts;
	if (chosen_config) {  // as many bytes as the caller's struct holds
		const size_t n = chosen_config->struct_size >= sizeof(lrx_trace_config) ? sizeof(lrx_trace_config)
				: offsetof(lrx_trace_config, refill);
		std::memcpy(chosen_config, &best_cfg, n);
		chosen_config->struct_size = (uint32_t)n;
	}
	return LRX_OK;
}

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
// one on a scene with motion instances, or -- when the call holds at most
// kMaxDirectBatches batches of kDirectBatchRays rays or more -- one of those.
static bool direct_batch(const lrx_batch &b, bool big_direct) {
	return b.count != 0 && ((big_direct && b.count >= kDirectBatchRays) || !b.scene->motions.empty());
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
			q.flags = (b.mode == LRX_TRACE_ANY ? 1u : 0u) | (s->two_level ? 2u : 0u) |
					((cfg.postpone & 0xffu) << 8) | (var << 16);
			q.visit_limit = scene_visit_limit(s);
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
		p.slot = next_queue_slot();
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
		uint32_t n_direct = 0;
		for (uint32_t k = 0; k < n_batches; ++k) {
			const lrx_batch &b = batches[k];
			if (!direct_batch(b, big_direct)) continue;
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
		for (uint32_t k = 0; k < n_batches; ++k) {
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
					LRX_CUDA(cudaMallocFromPoolAsync(&d_hits, hb, pool, s_in));
					LRX_CUDA(cudaMemcpyAsync(d_rays, hr, rb, cudaMemcpyHostToDevice, s_in));
					if (!mapped) LRX_CUDA(cudaMemcpyAsync(d_hits, hh, hb, cudaMemcpyHostToDevice, s_in));
					LRX_CUDA(cudaEventRecord(in_done, s_in));
					LRX_CUDA(cudaStreamWaitEvent(s_tr, in_done, 0));
					lrx_status r = trace_common(b.scene, d_rays, d_hits, n, b.mode, nullptr, s_tr);
					if (r == LRX_OK && mapped)
						r = launch_restore_masked_hits(d_rays, n, static_cast<const lrx_hit *>(mapped_hits) + c0, d_hits,
								s_tr);
					LRX_CUDA(cudaEventRecord(tr_done, s_tr));
					LRX_CUDA(cudaStreamWaitEvent(s_out, tr_done, 0));
					if (r == LRX_OK) LRX_CUDA(cudaMemcpyAsync(hh, d_hits, hb, cudaMemcpyDeviceToHost, s_out));
					cudaFreeAsync(d_rays, s_out);
					cudaFreeAsync(d_hits, s_out);
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

lrx_status lrx_scene_device_status(lrx_scene *s, uint32_t *status, void *stream) {
	if (!s || !status) {
		set_error("lrx_scene_device_status: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	DeviceGuard g(s->device);
	cudaStream_t st = (cudaStream_t)stream;
	uint32_t v = 0;
	LRX_CUDA(cudaMemcpyAsync(&v, s->status.ptr, 4, cudaMemcpyDeviceToHost, st));
	LRX_CUDA(cudaStreamSynchronize(st));
	LRX_CUDA(cudaMemsetAsync(s->status.ptr, 0, 4, st));
	*status = v;
	return v ? LRX_ERR_DEVICE : LRX_OK;
}

}  // extern "C"
