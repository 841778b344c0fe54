// The LuxRays side of the drop-in: the accelerator class a maintainer adds
// to the reference (as include/luxrays/accelerators/gb300accel.h) so that
// `accelerator.type = GB300` selects liblrx.so.  Written against the
// reference's own interfaces and compiled against its headers by
// tests/test_luxrays_binding.py:
//   Accelerator                 include/luxrays/core/accelerator.h:39-59
//   HardwareIntersectionKernel  include/luxrays/core/hardwareintersectiondevice.h:59-72
//   CUDADeviceBuffer            include/luxrays/devices/cudadevice.h:129-160
// Like OptixAccel (src/luxrays/accelerators/optixaccel.cpp:57-59) it has no
// CPU path: HasNativeSupport() is false and Intersect() throws.  The CUDA
// intersection device drives it through EnqueueTraceRayBuffer on the
// caller's CUDADeviceBuffers, with no copies.
#ifndef LRX_LUXRAYS_GB300ACCEL_H
#define LRX_LUXRAYS_GB300ACCEL_H

#include <deque>
#include <vector>

#include "luxrays/core/accelerator.h"
#include "luxrays/core/hardwareintersectiondevice.h"
#include "luxrays/devices/cudadevice.h"

#include "lrx.h"

namespace luxrays {

// The enum value the maintainer adds after ACCEL_OPTIX
// (include/luxrays/core/accelerator.h:31-33); spelled here as its value for
// headers that do not have it yet.
#ifndef LUXRAYS_HAS_ACCEL_GB300
static const AcceleratorType ACCEL_GB300 = static_cast<AcceleratorType>(ACCEL_OPTIX + 1);
#endif

class GB300Accel : public Accelerator {
public:
	explicit GB300Accel(const Context *ctx) : ctx(ctx), scene(nullptr) { }
	virtual ~GB300Accel();

	virtual AcceleratorType GetType() const { return ACCEL_GB300; }
	virtual bool HasNativeSupport(const IntersectionDevice &) const { return false; }
	virtual bool HasHWSupport(const IntersectionDevice &device) const { return device.HasHWSupport(); }
	virtual HardwareIntersectionKernel *NewHardwareIntersectionKernel(HardwareIntersectionDevice &device) const;

	// Builds the device scene from the DataSet's meshes, in DataSet order
	// (meshIndex = position): plain TriangleMeshes, InstanceTriangleMeshes
	// (their Transform::m and the mInv Transform keeps) and
	// MotionTriangleMeshes (their MotionSystem's keyframes).
	virtual void Init(const std::deque<const Mesh *> &meshes, const u_longlong totalVertexCount,
			const u_longlong totalTriangleCount);
	// Re-reads the instances' transforms and rebuilds only the top-level BVH,
	// as MBVHAccel::Update does (src/luxrays/accelerators/mbvhaccel.cpp:237-250).
	virtual bool DoesSupportUpdate() const { return true; }
	virtual void Update();

	virtual bool Intersect(const Ray *ray, RayHit *hit) const;

	lrx_scene *GetScene() const { return scene; }

private:
	// lrx object descriptions of the meshes (transforms as they are now);
	// motion keyframes into *motions (times and matrices kept alive in keys)
	struct MotionKeys {
		std::vector<float> times, mats;
	};
	void Describe(std::vector<lrx_mesh_desc> &md, std::vector<lrx_object_desc> &od,
			std::deque<MotionKeys> &keys, std::vector<lrx_motion_desc> &motions) const;

	const Context *ctx;
	std::deque<const Mesh *> meshes;
	lrx_scene *scene;
};

// The kernel object the CUDA intersection device creates in Start() and
// deletes in Stop() (src/luxrays/devices/cudaintersectiondevice.cpp:66-78).
class GB300Kernel : public HardwareIntersectionKernel {
public:
	GB300Kernel(HardwareIntersectionDevice &dev, const GB300Accel &accel) : HardwareIntersectionKernel(dev), accel(accel) { }
	virtual ~GB300Kernel() { }

	// The accelerator's Update already rebuilt the device scene's top level.
	virtual void Update(const DataSet *newDataSet) { }
	// Closest hit of rayCount rays of rayBuff into rayHitBuff, on stream 0 as
	// the CUDA device launches its kernels (src/luxrays/devices/cudadevice.cpp:384-405).
	virtual void EnqueueTraceRayBuffer(HardwareDeviceBuffer *rayBuff, HardwareDeviceBuffer *rayHitBuff,
			const unsigned int rayCount);

private:
	const GB300Accel &accel;
};

}

#endif
