// Drives liblrx.so through the LuxRays-style C++ layer (include/lrx_luxrays.hpp)
// the way a LuxRays device would: DataSet::Add -> Preprocess -> GetAccelerator
// -> NewHardwareIntersectionKernel -> EnqueueTraceRayBuffer on device buffers.
// Input: a binary scene + rays file; output: the hits file (and, after an
// instance Update, a second hits file).  Used by tests/test_luxrays_api.py.
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "lrx_luxrays.hpp"

using namespace lrx_luxrays;

template <class T> static void rd(FILE *f, T *p, size_t n) {
	if (fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input file");
}

int main(int argc, char **argv) {
	if (argc != 4) {
		std::fprintf(stderr, "usage: %s scene.bin hits.bin hits_after_update.bin\n", argv[0]);
		return 2;
	}
	try {
		FILE *f = std::fopen(argv[1], "rb");
		if (!f) throw std::runtime_error("cannot open input");
		uint32_t nm;
		rd(f, &nm, 1);
		std::vector<std::vector<float>> verts(nm);
		std::vector<std::vector<uint32_t>> tris(nm);
		std::vector<TriangleMesh> meshes(nm);
		for (uint32_t i = 0; i < nm; ++i) {
			uint32_t nv, nt;
			rd(f, &nv, 1);
			rd(f, &nt, 1);
			verts[i].resize(3ull * nv);
			tris[i].resize(3ull * nt);
			rd(f, verts[i].data(), verts[i].size());
			rd(f, tris[i].data(), tris[i].size());
			meshes[i] = TriangleMesh{verts[i].data(), tris[i].data(), nv, nt};
		}
		uint32_t no;
		rd(f, &no, 1);
		std::vector<InstanceTriangleMesh> insts;
		insts.reserve(no);
		DataSet ds;
		for (uint32_t i = 0; i < no; ++i) {
			uint32_t mesh, has;
			float m[16];
			rd(f, &mesh, 1);
			rd(f, &has, 1);
			rd(f, m, 16);
			if (has) {
				insts.push_back(InstanceTriangleMesh{&meshes[mesh], {}});
				std::memcpy(insts.back().transform, m, 64);
				ds.Add(&insts.back());
			} else {
				ds.Add(&meshes[mesh]);
			}
		}
		uint32_t nr;
		rd(f, &nr, 1);
		std::vector<Ray> rays(nr);
		rd(f, rays.data(), nr);
		std::vector<float> moved(16ull * no);  // transforms used after Update
		rd(f, moved.data(), moved.size());
		std::fclose(f);

		ds.Preprocess();
		const GB300Accel &accel = ds.GetAccelerator();
		bool threw = false;
		try {
			RayHit h;
			accel.Intersect(&rays[0], &h);
		} catch (const std::runtime_error &) {
			threw = true;  // no CPU path, as the reference's GPU-only accelerators
		}
		if (!threw || accel.HasNativeSupport()) throw std::runtime_error("Intersect() must throw");
		std::unique_ptr<HardwareIntersectionKernel> kernel = accel.NewHardwareIntersectionKernel();

		void *d_rays = nullptr, *d_hits = nullptr;
		if (cudaMalloc(&d_rays, sizeof(Ray) * nr) != cudaSuccess || cudaMalloc(&d_hits, sizeof(RayHit) * nr) != cudaSuccess)
			throw std::runtime_error("cudaMalloc");
		cudaMemcpy(d_rays, rays.data(), sizeof(Ray) * nr, cudaMemcpyHostToDevice);
		std::vector<RayHit> hits(nr);
		for (int pass = 0; pass < 2; ++pass) {
			if (pass == 1) {
				for (uint32_t i = 0; i < no; ++i)
					if (ds.Objects()[i].flags & LRX_OBJECT_INSTANCE) ds.SetTransform(i, &moved[16ull * i]);
				kernel->Update(ds.Objects());
			}
			kernel->EnqueueTraceRayBuffer(d_rays, d_hits, nr);
			if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("cudaDeviceSynchronize");
			cudaMemcpy(hits.data(), d_hits, sizeof(RayHit) * nr, cudaMemcpyDeviceToHost);
			FILE *o = std::fopen(argv[2 + pass], "wb");
			if (!o || std::fwrite(hits.data(), sizeof(RayHit), nr, o) != nr) throw std::runtime_error("cannot write hits");
			std::fclose(o);
		}
		cudaFree(d_rays);
		cudaFree(d_hits);
		std::printf("ok %u rays\n", nr);
		return 0;
	} catch (const std::exception &e) {
		std::fprintf(stderr, "error: %s\n", e.what());
		return 1;
	}
}
