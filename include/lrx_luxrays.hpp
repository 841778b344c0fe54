// lrx_luxrays.hpp -- C++ host layer over liblrx.so that mirrors the LuxRays
// accelerator interface for the data-parallel intersection path, so code
// written against luxrays::DataSet / Accelerator / HardwareIntersectionKernel
// reads the same.  Header-only; every call goes through the C ABI of lrx.h
// and turns a status code into std::runtime_error, as the reference reports
// errors (include/luxrays/utils/cuda.h:36-69).
//
// Mirrors (by name and meaning):
//   luxrays::Ray / RayHit              include/luxrays/core/geometry/ray.h:35-103
//   luxrays::TriangleMesh              include/luxrays/core/trianglemesh.h:79-201
//   luxrays::InstanceTriangleMesh      trianglemesh.h:203-305 (mesh + Transform)
//   luxrays::MotionTriangleMesh        trianglemesh.h:307-410 (mesh + MotionSystem)
//   luxrays::DataSet::Add/Preprocess   src/luxrays/core/dataset.cpp:66-94
//   luxrays::Accelerator (ACCEL_GB300) include/luxrays/core/accelerator.h:39-59
//   luxrays::HardwareIntersectionKernel::EnqueueTraceRayBuffer / Update
//                                      include/luxrays/core/hardwareintersectiondevice.h:59-72
#pragma once

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lrx.h"

namespace lrx_luxrays {

// Byte-identical to luxrays::Ray / luxrays::RayHit.
typedef lrx_ray Ray;
typedef lrx_hit RayHit;
static_assert(sizeof(Ray) == 48, "luxrays::Ray is 48 bytes");
static_assert(sizeof(RayHit) == 20, "luxrays::RayHit is 20 bytes");

inline void Check(lrx_status st, const char *what) {
	if (st != LRX_OK) throw std::runtime_error(std::string(what) + ": " + lrx_last_error());
}

// A triangle mesh in world space; vertex/index memory stays owned by the
// caller until the DataSet's accelerator is built (the library copies it).
struct TriangleMesh {
	const float *vertices;      // xyz per vertex (luxrays::Point)
	const uint32_t *triangles;  // v0 v1 v2 per triangle (luxrays::Triangle)
	uint32_t vertexCount, triangleCount;
};

// A mesh placed by a row-major 4x4 local-to-world matrix (Transform::m).
struct InstanceTriangleMesh {
	const TriangleMesh *mesh;
	float transform[16];
};

// A mesh moved by a motion system (MotionSystem's keyframes): strictly
// increasing times and row-major world-to-local matrices, 16 floats each --
// the matrices MBVHAccel applies to a ray at its time.
struct MotionTriangleMesh {
	const TriangleMesh *mesh;
	std::vector<float> times;
	std::vector<float> transforms;
};

enum AcceleratorType { ACCEL_AUTO, ACCEL_BVH, ACCEL_MBVH, ACCEL_EMBREE, ACCEL_OPTIX, ACCEL_GB300 };

class HardwareIntersectionKernel;

// GPU accelerator: no CPU path (HasNativeSupport() is false, Intersect()
// throws), like the reference's OptixAccel.
class GB300Accel {
public:
	GB300Accel() : scene(nullptr) {}
	~GB300Accel() { lrx_scene_destroy(scene); }
	GB300Accel(const GB300Accel &) = delete;
	GB300Accel &operator=(const GB300Accel &) = delete;

	AcceleratorType GetType() const { return ACCEL_GB300; }
	bool HasNativeSupport() const { return false; }
	bool HasHWSupport() const { return true; }
	bool DoesSupportUpdate() const { return true; }

	void Init(const std::vector<lrx_mesh_desc> &meshes, const std::vector<lrx_object_desc> &objects,
			const std::vector<lrx_motion_desc> &motions = {}) {
		Check(lrx_scene_create_motion(meshes.data(), (uint32_t)meshes.size(), objects.data(),
				      (uint32_t)objects.size(), motions.data(), (uint32_t)motions.size(), nullptr, nullptr, &scene),
				"GB300Accel::Init");
	}
	bool Intersect(const Ray *, RayHit *) const {
		throw std::runtime_error("Internal error: called GB300Accel::Intersect() (no CPU path)");
	}
	inline std::unique_ptr<HardwareIntersectionKernel> NewHardwareIntersectionKernel() const;

	lrx_scene *Scene() const { return scene; }

private:
	lrx_scene *scene;
};

// The GPU kernel object a device drives; buffers are device addresses
// (what CUDADeviceBuffer::GetCUDADevicePointer returns in the reference).
class HardwareIntersectionKernel {
public:
	explicit HardwareIntersectionKernel(const GB300Accel &a) : accel(a) {}
	void EnqueueTraceRayBuffer(const void *rayBuff, void *rayHitBuff, unsigned int rayCount, void *stream = nullptr,
			uint32_t mode = LRX_TRACE_CLOSEST) {
		Check(lrx_trace(accel.Scene(), rayBuff, rayHitBuff, rayCount, mode, stream), "EnqueueTraceRayBuffer");
	}
	// New instance transforms (same objects, same meshes).
	void Update(const std::vector<lrx_object_desc> &objects, void *stream = nullptr) {
		Check(lrx_scene_update_instances(accel.Scene(), objects.data(), (uint32_t)objects.size(), stream),
				"HardwareIntersectionKernel::Update");
	}

private:
	const GB300Accel &accel;
};

inline std::unique_ptr<HardwareIntersectionKernel> GB300Accel::NewHardwareIntersectionKernel() const {
	return std::unique_ptr<HardwareIntersectionKernel>(new HardwareIntersectionKernel(*this));
}

// Ordered list of meshes; a mesh's position is the meshIndex its hits report.
class DataSet {
public:
	// Returns the TriangleMeshID (= meshIndex in hits).
	uint32_t Add(const TriangleMesh *mesh) {
		objects.push_back(object(meshIndexOf(mesh), nullptr));
		return (uint32_t)objects.size() - 1;
	}
	uint32_t Add(const InstanceTriangleMesh *inst) {
		objects.push_back(object(meshIndexOf(inst->mesh), inst->transform));
		return (uint32_t)objects.size() - 1;
	}
	// The motion system's vectors must stay alive until GetAccelerator.
	uint32_t Add(const MotionTriangleMesh *mm) {
		if (mm->transforms.size() != 16 * mm->times.size())
			throw std::runtime_error("DataSet::Add: one 4x4 matrix per motion keyframe");
		static const float identity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
		objects.push_back(object(meshIndexOf(mm->mesh), identity));
		motions.push_back(lrx_motion_desc{(uint32_t)objects.size() - 1, (uint32_t)mm->times.size(),
				mm->times.data(), mm->transforms.data()});
		return (uint32_t)objects.size() - 1;
	}
	void Preprocess() { preprocessed = true; }
	bool RequiresInstanceSupport() const {
		for (const lrx_object_desc &o : objects)
			if (o.flags & LRX_OBJECT_INSTANCE) return true;
		return false;
	}
	// Builds the GPU accelerator (DataSet::GetAccelerator(ACCEL_GB300)).
	const GB300Accel &GetAccelerator() {
		if (!preprocessed) throw std::runtime_error("DataSet::GetAccelerator before Preprocess");
		if (!accel) {
			accel.reset(new GB300Accel());
			accel->Init(meshes, objects, motions);
		}
		return *accel;
	}
	const std::vector<lrx_object_desc> &Objects() const { return objects; }
	void SetTransform(uint32_t meshIndex, const float m[16]) {
		std::memcpy(objects.at(meshIndex).transform, m, 64);
	}

private:
	uint32_t meshIndexOf(const TriangleMesh *m) {
		for (size_t i = 0; i < sources.size(); ++i)
			if (sources[i] == m) return (uint32_t)i;
		sources.push_back(m);
		meshes.push_back(lrx_mesh_desc{m->vertices, m->triangles, m->vertexCount, m->triangleCount});
		return (uint32_t)meshes.size() - 1;
	}
	static lrx_object_desc object(uint32_t mesh, const float *m) {
		lrx_object_desc o;
		std::memset(&o, 0, sizeof(o));
		o.mesh = mesh;
		if (m) {
			o.flags = LRX_OBJECT_INSTANCE;
			std::memcpy(o.transform, m, 64);
		}
		return o;
	}

	std::vector<const TriangleMesh *> sources;
	std::vector<lrx_mesh_desc> meshes;
	std::vector<lrx_object_desc> objects;
	std::vector<lrx_motion_desc> motions;
	std::unique_ptr<GB300Accel> accel;
	bool preprocessed = false;
};

}  // namespace lrx_luxrays
