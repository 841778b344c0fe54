// Runs the reference's own CUDA intersection kernel on the GPU -- TEST
// INFRASTRUCTURE, a comparison arm only (bench.py, tests/).
//
// The kernel text is the reference's, stitched by oracle/build_ref.sh into
// oracle/_ref/refcu_bvh_kernel.cu exactly as the reference assembles it for
// its CUDA device:
//   CUDADevice::GetKernelSource (src/luxrays/devices/cudadevice.cpp:235-241)
//     prefixes the OpenCL emulation (cudadevice_oclemul_types.cl,
//     cudadevice_math.cl, cudadevice_oclemul_funcs.cl) to
//   BVHKernel's source (src/luxrays/accelerators/bvhaccelhw.cpp:173-202):
//     the page defines, then luxrays_types.cl ... bvhbuild_types.cl, bvh.cl.
// This file compiles that text with NVRTC under the options the reference
// uses (and once more with --fmad=false instead of --use_fast_math, which
// matches the CPU run of the same text exactly) -- src/luxrays/utils/cuda.cpp:63-129
// (--device-as-default-execution-space, compute_75 as GetCuda10Architecture
// caps it, the -Xcudafe suppressions), bvhaccelhw.cpp:167-170 (LUXRAYS_OPENCL_KERNEL and the
// MachineEpsilon bounds), cudadevice.cpp:220-226 (LUXRAYS_CUDA_DEVICE, the OS
// define) and the --use_fast_math its PATHOCL engine adds
// (src/slg/engines/pathoclbase/pathoclbase.cpp:79-85) -- loads the result
// with the driver (which compiles it for the GPU at hand) and launches
// Accelerator_Intersect_RayBuffer over the oracle's BVHArrayNode[] with
// 32-thread blocks, one page of vertices and one of nodes.  The compiled
// code is only run, never read.
#include <cuda.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

namespace {

// Two builds of the kernel: [0] exact (--fmad=false), [1] --use_fast_math.
std::mutex g_mu;
CUmodule g_module[2] = {nullptr, nullptr};
CUfunction g_kernel[2] = {nullptr, nullptr};
std::string g_info[2];

void put(char *out, size_t size, const std::string &s) {
	if (!out || size == 0) return;
	const size_t n = std::min(size - 1, s.size());
	std::memcpy(out, s.data(), n);
	out[n] = 0;
}

// Compiles `src` for `arch` with the reference's options plus
// --use_fast_math (`fast`, as PATHOCL deploys it) or --fmad=false (no
// contraction of multiply-adds: the FP32 operations of the CPU run of the
// same text, compiled with -ffp-contract=off); empty on failure (the log in
// *log).
std::string compile_ptx(const std::string &src, const std::string &arch, bool fast, std::string *log) {
	nvrtcProgram prog;
	if (nvrtcCreateProgram(&prog, src.c_str(), "BVHKernel", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
		*log = "nvrtcCreateProgram failed";
		return {};
	}
	const std::string arch_opt = "--gpu-architecture=" + arch;
	const char *opts[] = {"--device-as-default-execution-space", arch_opt.c_str(),
			"-Xcudafe", "--display_error_number", "-Xcudafe", "--diag_suppress=550",
			"-Xcudafe", "--diag_suppress=1055", "-Xcudafe", "--diag_suppress=68",
			"-D", "LUXRAYS_OPENCL_KERNEL", "-D", "PARAM_RAY_EPSILON_MIN=1e-05f", "-D", "PARAM_RAY_EPSILON_MAX=0.1f",
			"-D", "LUXRAYS_CUDA_DEVICE", "-D", "LUXRAYS_OS_LINUX",
			fast ? "--use_fast_math" : "--fmad=false"};
	const nvrtcResult rc = nvrtcCompileProgram(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
	size_t log_size = 0;
	nvrtcGetProgramLogSize(prog, &log_size);
	std::string l(log_size, '\0');
	if (log_size) nvrtcGetProgramLog(prog, &l[0]);
	*log = l;
	std::string ptx;
	if (rc == NVRTC_SUCCESS) {
		size_t n = 0;
		nvrtcGetPTXSize(prog, &n);
		ptx.resize(n);
		nvrtcGetPTX(prog, &ptx[0]);
	}
	nvrtcDestroyProgram(&prog);
	return ptx;
}

}  // namespace

// Compiles and loads the stitched kernel on the current CUDA device (its
// primary context, the one the CUDA runtime uses): `fast_math` 1 with the
// --use_fast_math the reference's PATHOCL engine compiles it with, 0 exact
// (--fmad=false).  Returns 0 on success; `info` gets what was compiled, or
// the error.
extern "C" int refcu_load(const char *src_path, int fast_math, char *info, size_t info_size) {
	std::lock_guard<std::mutex> lk(g_mu);
	const int f = fast_math ? 1 : 0;
	if (g_kernel[f]) {
		put(info, info_size, g_info[f]);
		return 0;
	}
	std::ifstream file(src_path, std::ios::binary);
	if (!file) {
		put(info, info_size, std::string("kernel text not found: ") + src_path);
		return 1;
	}
	std::stringstream ss;
	ss << file.rdbuf();
	const std::string src = ss.str();
	if (cuInit(0) != CUDA_SUCCESS) {
		put(info, info_size, "cuInit failed");
		return 2;
	}
	CUcontext ctx = nullptr;
	cuCtxGetCurrent(&ctx);
	CUdevice dev = 0;
	if (!ctx) {
		if (cuDeviceGet(&dev, 0) != CUDA_SUCCESS || cuDevicePrimaryCtxRetain(&ctx, dev) != CUDA_SUCCESS ||
				cuCtxSetCurrent(ctx) != CUDA_SUCCESS) {
			put(info, info_size, "no CUDA context");
			return 2;
		}
	} else {
		cuCtxGetDevice(&dev);
	}
	// compute_75 as the reference caps it; the device's own architecture if
	// this NVRTC no longer accepts compute_75
	std::string log, arch = "compute_75";
	std::string ptx = compile_ptx(src, arch, f != 0, &log);
	if (ptx.empty()) {
		int major = 0, minor = 0;
		cuDeviceGetAttribute(&major, CU_DEVICE_ATTRIBUTE_COMPUTE_CAPABILITY_MAJOR, dev);
		cuDeviceGetAttribute(&minor, CU_DEVICE_ATTRIBUTE_COMPUTE_CAPABILITY_MINOR, dev);
		arch = "compute_" + std::to_string(major) + std::to_string(minor);
		ptx = compile_ptx(src, arch, f != 0, &log);
		if (ptx.empty()) {
			put(info, info_size, "NVRTC: " + log.substr(0, 2000));
			return 3;
		}
		arch += " (compute_75 rejected)";
	}
	if (cuModuleLoadData(&g_module[f], ptx.c_str()) != CUDA_SUCCESS ||
			cuModuleGetFunction(&g_kernel[f], g_module[f], "Accelerator_Intersect_RayBuffer") != CUDA_SUCCESS) {
		g_module[f] = nullptr;
		g_kernel[f] = nullptr;
		put(info, info_size, "cuModuleLoadData / cuModuleGetFunction failed");
		return 4;
	}
	g_info[f] = "NVRTC " + arch + (f ? ", --use_fast_math" : ", --fmad=false") + ", driver JIT to the device";
	put(info, info_size, g_info[f]);
	return 0;
}

// One launch over `count` rays (device addresses: 48-byte rays, 20-byte hits,
// 12-byte vertices, 32-byte BVHArrayNode records) on `stream`, `block`
// threads per block (the reference's default is 32).  Returns the CUresult.
extern "C" int refcu_trace(int fast_math, unsigned long long rays, unsigned long long hits, unsigned int count,
		unsigned long long verts, unsigned long long nodes, unsigned int block, void *stream) {
	CUfunction fn = g_kernel[fast_math ? 1 : 0];
	if (!fn) return -1;
	if (count == 0) return 0;
	if (block == 0) block = 32;
	CUdeviceptr r = rays, h = hits, v = verts, n = nodes, null_ptr = 0;
	unsigned int c = count;
	void *params[19];
	params[0] = &r;
	params[1] = &h;
	params[2] = &c;
	params[3] = &v;
	for (int k = 4; k < 11; ++k) params[k] = &null_ptr;
	params[11] = &n;
	for (int k = 12; k < 19; ++k) params[k] = &null_ptr;
	const unsigned int grid = (count + block - 1) / block;
	return (int)cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, (CUstream)stream, params, nullptr);
}
