// GB300Accel / GB300Kernel (gb300accel.h): the LuxRays accelerator over
// liblrx.so.  Errors of the C ABI become std::runtime_error, as the
// reference reports its own.
#include "gb300accel.h"

#include <cstring>
#include <map>
#include <stdexcept>
#include <string>

#include "luxrays/core/context.h"
#include "luxrays/utils/properties.h"

namespace luxrays {

namespace {

void check(lrx_status st, const char *what) {
	if (st != LRX_OK) throw std::runtime_error(std::string(what) + ": " + lrx_last_error());
}

// The tree's build options from the context's configuration, where the
// reference's accelerators read theirs (BVHAccel::ToBVHParams,
// src/luxrays/accelerators/bvhaccel.cpp:39-62):
//   accelerator.gb300.nodewidth      children per wide node, 4-8 (8)
//   accelerator.gb300.nodelayout     "wide8" (80-byte records) or "compact4"
//                                    (64-byte records, node width 4, flat scenes)
//   accelerator.gb300.leafsize       triangles per leaf, 1-3 (3)
//   accelerator.gb300.treeletpasses  treelet SAH passes (2)
// accelerator.bvh.treetype describes the reference's CPU tree and is not
// read: its default (4) is not the shape this engine traverses fastest.
lrx_build_opts BuildOptions(const Context *ctx) {
	lrx_build_opts o;
	std::memset(&o, 0, sizeof(o));
	o.struct_size = sizeof(o);
	o.node_width = 8;
	o.leaf_max = 3;
	o.treelet_passes = 2;
	o.node_layout = LRX_NODES_WIDE8;
	if (!ctx) return o;
	const Properties &cfg = ctx->GetConfig();
	o.node_width = (uint32_t)cfg.Get(Property("accelerator.gb300.nodewidth")(8)).Get<int>();
	o.leaf_max = (uint32_t)cfg.Get(Property("accelerator.gb300.leafsize")(3)).Get<int>();
	o.treelet_passes = (uint32_t)cfg.Get(Property("accelerator.gb300.treeletpasses")(2)).Get<int>();
	const std::string layout = cfg.Get(Property("accelerator.gb300.nodelayout")("wide8")).Get<std::string>();
	if (layout == "compact4") o.node_layout = LRX_NODES_COMPACT4;
	else if (layout != "wide8") throw std::runtime_error("GB300Accel: unknown accelerator.gb300.nodelayout: " + layout);
	return o;  // the ranges are checked by lrx_scene_create
}

}  // namespace

GB300Accel::~GB300Accel() {
	if (scene) lrx_scene_destroy(scene);
}

void GB300Accel::Describe(std::vector<lrx_mesh_desc> &md, std::vector<lrx_object_desc> &od,
		std::deque<MotionKeys> &keys, std::vector<lrx_motion_desc> &motions) const {
	std::map<const TriangleMesh *, uint32_t> meshIndex;
	od.assign(meshes.size(), lrx_object_desc());
	for (size_t i = 0; i < meshes.size(); ++i) {
		const Mesh *m = meshes[i];
		lrx_object_desc &o = od[i];
		std::memset(&o, 0, sizeof(o));
		const TriangleMesh *base = nullptr;
		switch (m->GetType()) {
			case TYPE_TRIANGLE:
			case TYPE_EXT_TRIANGLE:
				base = dynamic_cast<const TriangleMesh *>(m);
				break;
			case TYPE_TRIANGLE_INSTANCE:
			case TYPE_EXT_TRIANGLE_INSTANCE: {
				const InstanceTriangleMesh *itm = dynamic_cast<const InstanceTriangleMesh *>(m);
				base = itm->GetTriangleMesh();
				const Transform &t = itm->GetTransformation();
				o.flags = LRX_OBJECT_INSTANCE | LRX_OBJECT_HAS_INVERSE;
				std::memcpy(o.transform, &t.m.m[0][0], sizeof(o.transform));
				std::memcpy(o.inverse, &t.mInv.m[0][0], sizeof(o.inverse));  // Transform keeps its own inverse
				break;
			}
			case TYPE_TRIANGLE_MOTION:
			case TYPE_EXT_TRIANGLE_MOTION: {
				// keyframe k of a MotionSystem is interpolatedTransforms[k + 1].start
				// (MotionSystem::Init, src/luxrays/core/geometry/motionsystem.cpp:296-330):
				// world -> local, as MBVHAccel applies it to the ray
				const MotionTriangleMesh *mtm = dynamic_cast<const MotionTriangleMesh *>(m);
				base = mtm->GetTriangleMesh();
				const MotionSystem &ms = mtm->GetMotionSystem();
				keys.emplace_back();
				MotionKeys &k = keys.back();
				k.times = ms.times;
				for (size_t j = 0; j < ms.times.size(); ++j) {
					const float *src = &ms.interpolatedTransforms[j + 1].start.m.m[0][0];
					k.mats.insert(k.mats.end(), src, src + 16);
				}
				o.flags = LRX_OBJECT_INSTANCE;  // the motion system replaces the transform
				lrx_motion_desc d;
				d.object = (uint32_t)i;
				d.count = (uint32_t)k.times.size();
				d.times = k.times.data();
				d.transforms = k.mats.data();
				motions.push_back(d);
				break;
			}
			default:
				throw std::runtime_error("GB300Accel: unsupported mesh type");
		}
		if (!base) throw std::runtime_error("GB300Accel: mesh without triangle data");
		auto it = meshIndex.find(base);
		if (it == meshIndex.end()) {
			it = meshIndex.emplace(base, (uint32_t)md.size()).first;
			lrx_mesh_desc d;
			d.vertices = reinterpret_cast<const float *>(base->GetVertices());   // Point: 3 floats
			d.triangles = reinterpret_cast<const uint32_t *>(base->GetTriangles());  // Triangle: 3 u_int
			d.vertex_count = base->GetTotalVertexCount();
			d.triangle_count = base->GetTotalTriangleCount();
			md.push_back(d);
		}
		o.mesh = it->second;
	}
}

void GB300Accel::Init(const std::deque<const Mesh *> &ms, const u_longlong, const u_longlong) {
	meshes = ms;
	std::vector<lrx_mesh_desc> md;
	std::vector<lrx_object_desc> od;
	std::deque<MotionKeys> keys;
	std::vector<lrx_motion_desc> motions;
	Describe(md, od, keys, motions);
	if (scene) {
		lrx_scene_destroy(scene);
		scene = nullptr;
	}
	const lrx_build_opts opts = BuildOptions(ctx);
	if (motions.empty())
		check(lrx_scene_create(md.data(), (uint32_t)md.size(), od.data(), (uint32_t)od.size(), &opts, nullptr, &scene),
				"GB300Accel::Init");
	else
		check(lrx_scene_create_motion(md.data(), (uint32_t)md.size(), od.data(), (uint32_t)od.size(), motions.data(),
				(uint32_t)motions.size(), &opts, nullptr, &scene), "GB300Accel::Init");
}

void GB300Accel::Update() {
	std::vector<lrx_mesh_desc> md;
	std::vector<lrx_object_desc> od;
	std::deque<MotionKeys> keys;
	std::vector<lrx_motion_desc> motions;
	Describe(md, od, keys, motions);
	check(lrx_scene_update_instances(scene, od.data(), (uint32_t)od.size(), nullptr), "GB300Accel::Update");
}

bool GB300Accel::Intersect(const Ray *, RayHit *) const {
	throw std::runtime_error("Internal error: called GB300Accel::Intersect()");
}

HardwareIntersectionKernel *GB300Accel::NewHardwareIntersectionKernel(HardwareIntersectionDevice &device) const {
	return new GB300Kernel(device, *this);
}

void GB300Kernel::EnqueueTraceRayBuffer(HardwareDeviceBuffer *rayBuff, HardwareDeviceBuffer *rayHitBuff,
		const unsigned int rayCount) {
	// CUDADeviceBuffer::GetCUDADevicePointer (include/luxrays/devices/cudadevice.h:152)
	CUDADeviceBuffer *rays = dynamic_cast<CUDADeviceBuffer *>(rayBuff);
	CUDADeviceBuffer *hits = dynamic_cast<CUDADeviceBuffer *>(rayHitBuff);
	if (!rays || !hits) throw std::runtime_error("GB300Kernel: not a CUDA device buffer");
	const CUdeviceptr r = rays->GetCUDADevicePointer(), h = hits->GetCUDADevicePointer();
	check(lrx_trace(accel.GetScene(), reinterpret_cast<const void *>(r), reinterpret_cast<void *>(h), rayCount,
			LRX_TRACE_CLOSEST, nullptr), "GB300Kernel::EnqueueTraceRayBuffer");
}

}  // namespace luxrays
