// C-ABI layer of liblrx.so: scene assembly on the device, instance
// transforms, launch configuration, the autotuner and error reporting.  The
// tracing entry points are in lrx_launch.cpp, built-scene blobs in
// lrx_blob.cpp.  Declarations and the reference interfaces each entry point
// replaces are in include/lrx.h.
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
#include "lrx_scene.h"

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

}  // namespace lrx

using namespace lrx;

int lrx::scene_device(const lrx_scene *scene) { return scene->device; }

namespace {

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
		const lrx_build_opts bopts = read_build_opts(opts);
		if (bopts.node_width < 4 || bopts.node_width > 8) {
			set_error("lrx_scene_create: node_width must be 0 or in [4, 8]");
			return LRX_ERR_INVALID_ARGUMENT;
		}
		if (bopts.node_layout > LRX_NODES_COMPACT4 ||
				(bopts.node_layout == LRX_NODES_COMPACT4 && bopts.node_width != 4)) {
			set_error("lrx_scene_create: node_layout must be LRX_NODES_WIDE8, or LRX_NODES_COMPACT4 with node_width 4");
			return LRX_ERR_INVALID_ARGUMENT;
		}
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
		s->opts = bopts;
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
		if (any_inst && s->opts.node_layout == LRX_NODES_COMPACT4) {
			set_error("lrx_scene_create: 64-byte node records (LRX_NODES_COMPACT4) need a flat scene");
			return LRX_ERR_NOT_SUPPORTED;
		}

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
		s->info.node_bytes = node_record_bytes(s->opts);
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
			if (s->opts.node_layout == LRX_NODES_COMPACT4) {  // the tree in 64-byte records
				DevBuf packed;
				if ((rc = packed.alloc(sizeof(Node4) * ((size_t)node_off + 1))) != LRX_OK) return rc;
				if ((rc = pack_nodes4(s->nodes.as<WideNode>(), packed.as<Node4>(), node_off, st)) != LRX_OK) return rc;
				s->nodes = std::move(packed);
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


// A correct walk expands each node of a tree at most once per entry into
// that tree.  A ray's visit count rises by one per expansion and each
// instance entry takes B (the largest BLAS's node count + 64) off it,
// stopping at zero.  Right after the last point where it stood at zero (or
// the start), the count has since grown by at most one BLAS walk (< B) plus
// TLAS expansions, while every later entry takes off more than its walk
// adds; so a valid walk never passes T + B, T the node count of the
// top-level tree (the whole BVH of a flat scene, where B = 0) + 64.
extern "C++" uint32_t lrx::scene_visit_limit(const lrx_scene *s) {
	const uint64_t top = s->two_level ? s->info.node_count - s->blas_node_total : s->info.node_count;
	return (uint32_t)std::min<uint64_t>(top + 64 + scene_blas_visits(s), 0x7fffffffull);
}

extern "C++" uint32_t lrx::scene_blas_visits(const lrx_scene *s) {
	if (!s->two_level) return 0;
	std::vector<uint32_t> roots;  // BLAS node ranges are contiguous, in root order
	for (const Blas &b : s->blas)
		if (b.root != kNull) roots.push_back(b.root);
	std::sort(roots.begin(), roots.end());
	roots.push_back(s->blas_node_total);
	uint64_t widest = 0;
	for (size_t k = 0; k + 1 < roots.size(); ++k) widest = std::max<uint64_t>(widest, roots[k + 1] - roots[k]);
	return (uint32_t)std::min<uint64_t>(widest + 64, 1ull << 30);
}

extern "C++" lrx_status lrx::trace_common(lrx_scene *s, const void *d_rays, void *d_hits, uint32_t count, uint32_t mode,
		uint64_t *d_counters, cudaStream_t st, const FixedScratch *fixed, bool pipeline_chunk) {
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
	a.nodes4 = s->opts.node_layout == LRX_NODES_COMPACT4 ? 1u : 0u;
	a.rays = d_rays;
	a.hits = d_hits;
	a.count = count;
	a.any_hit = mode == LRX_TRACE_ANY;
	a.status = s->status.as<uint32_t>();
	a.counters = reinterpret_cast<unsigned long long *>(d_counters);
	const lrx_trace_config &cfg = s->tcfg[mode == LRX_TRACE_ANY ? 1 : 0];
	a.visit_limit = cfg.max_visits ? cfg.max_visits : scene_visit_limit(s);
	a.blas_visits = cfg.max_visits ? 0u : scene_blas_visits(s);
	a.deadline_ticks = deadline_ticks(cfg.deadline_us, count);
	a.block_size = cfg.block_size;
	a.postpone = cfg.postpone;
	a.variant = cfg.variant;
	a.refill = cfg.refill;
	if (pipeline_chunk && (a.variant & kVarSortRays)) {
		// a chunk of the host pipeline: persistent warps instead of a sort of
		// its own (e2e on the heightfield step: +12 % with 384 k-ray chunks in
		// call order, 2,662 against 2,376 Mrays/s; +3.4 % with 1 M-ray chunks)
		a.variant = (a.variant & ~(kVarSortRays | kVarSortOctantOnly)) | kVarPersistent;
		if (a.refill == 0) a.refill = 8;
	}
	if ((a.variant & kVarSortRays) && count >= kSortMinRays && s->root != kNull)
		return launch_trace_sorted(a, s->bounds_lo, s->bounds_hi, st, fixed);
	if ((a.variant & kVarCompact) && (a.variant & kVarPersistent) && !d_counters && count <= kMaxFetchRays)
		return launch_trace_compacted(a, st, fixed);
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
	// shared-memory stacks deeper than 8 entries: at most 32 KB of shared memory per block
	const uint32_t smem_depth = (uint32_t)smem_stack_depth(in.variant);
	if (bs < 32 || bs > 512 || (bs & 31) || in.postpone > 32 || (in.variant & ~kVarAll) || in.modes > 3u ||
			in.refill > 32 || (smem_depth > 8 && 8u * smem_depth * bs > 32768u)) {
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
			LRX_VARIANT_PERSISTENT | LRX_VARIANT_SMEM_STACK16, LRX_VARIANT_PERSISTENT | LRX_VARIANT_SMEM_STACK32,
			LRX_VARIANT_SORT_RAYS | LRX_VARIANT_SMEM_STACK16, LRX_VARIANT_PERSISTENT | LRX_VARIANT_SCENE_L2_KEEP};
	// closest hit: the persistent shapes also with the drain split (its builds
	// keep the stack in local memory)
	const bool try_split = m == 0;
	for (uint32_t bs : kBlocks) {
		for (uint32_t pp : kPostpone) {
			for (uint32_t v = 0; v < 2 * (sizeof(kVariants) / sizeof(kVariants[0])); ++v) {
				const uint32_t split = v & 1u;
				uint32_t var = kVariants[v >> 1];
				if (split && (!try_split || !(var & LRX_VARIANT_PERSISTENT) || smem_stack_bits(var))) continue;
				if (split) var |= LRX_VARIANT_DRAIN_SPLIT;
				if ((var & LRX_VARIANT_SORT_RAYS) && count < kSortMinRays) continue;
				s->tcfg[m] = lrx_trace_config{sizeof(lrx_trace_config), bs, pp, var, 1u << m,
							(var & LRX_VARIANT_PERSISTENT) ? 8u : 0u, best.max_visits, best.deadline_us};
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
		const size_t n = std::max<size_t>(offsetof(lrx_trace_config, refill),
				std::min<size_t>(chosen->struct_size, sizeof(lrx_trace_config)));
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
	lrx_build_opts base = read_build_opts(opts);  // its treelet passes; the rest is the candidates'
	// candidate builds: (node width, node record) x triangles per leaf -- the
	// 64-byte record only for flat scenes
	bool flat = true;
	for (uint32_t i = 0; objects && i < object_count; ++i) flat &= !(objects[i].flags & LRX_OBJECT_INSTANCE);
	struct Shape {
		uint32_t width, layout;
	};
	std::vector<Shape> shapes = {{8, LRX_NODES_WIDE8}, {4, LRX_NODES_WIDE8}};
	if (flat) shapes.push_back({4, LRX_NODES_COMPACT4});
	static const uint32_t kLeaves[] = {3, 2};
	cudaStream_t st = (cudaStream_t)stream;
	lrx_scene *best = nullptr;
	float best_ms = INFINITY;
	lrx_build_opts best_opts = base;
	lrx_trace_config best_cfg{};
	lrx_status rc = LRX_OK;
	void *hits = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	for (const Shape &sh : shapes) {
		for (uint32_t leaf : kLeaves) {
			lrx_build_opts o = base;
			o.node_width = sh.width;
			o.node_layout = sh.layout;
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
	if (chosen_opts) {  // as many bytes as the caller's struct holds (ABI 1-3: no node_layout)
		const size_t n = std::min<size_t>(std::max<size_t>(chosen_opts->struct_size, kBuildOptsAbi3Size),
				sizeof(lrx_build_opts));
		std::memcpy(chosen_opts, &best_opts, n);
		chosen_opts->struct_size = (uint32_t)n;
	}
	if (chosen_config) {  // as many bytes as the caller's struct holds
		const size_t n = chosen_config->struct_size >= sizeof(lrx_trace_config) ? sizeof(lrx_trace_config)
				: offsetof(lrx_trace_config, refill);
		std::memcpy(chosen_config, &best_cfg, n);
		chosen_config->struct_size = (uint32_t)n;
	}
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
