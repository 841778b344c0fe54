// OpenCL-C emulation for compiling the reference's kernel text on the CPU --
// TEST INFRASTRUCTURE (parity pin of the oracle; see build_ref.sh).
//
// Just enough of OpenCL C for the reference's luxrays_types.cl, epsilon_*.cl,
// point/vector/ray/bbox/triangle *.cl and bvh.cl: vector types with
// component-wise arithmetic, dot/cross (textual left-to-right order, no FMA),
// fmin/fmax/clamp, as_uint/as_float, vloadN/vstoreN and get_global_id.
// Written for this project; it shares no code with the reference's own CUDA
// emulation headers.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#define __kernel
#define __global
#define __constant const
#define __local
#define restrict __restrict__
#define OPENCL_FORCE_INLINE static inline
#define OPENCL_FORCE_NOT_INLINE static

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned long ulong;

struct float2 { float x, y; };
struct float3 { float x, y, z, _pad; };
struct alignas(16) float4 { float x, y, z, w; };

static inline float2 make_f2(float x, float y) { return {x, y}; }
static inline float3 make_f3(float x, float y, float z) { return {x, y, z, 0.f}; }
static inline float4 make_f4(float x, float y, float z, float w) { return {x, y, z, w}; }
#define MAKE_FLOAT2(x, y) make_f2((x), (y))
#define MAKE_FLOAT3(x, y, z) make_f3((x), (y), (z))
#define MAKE_FLOAT4(x, y, z, w) make_f4((x), (y), (z), (w))

#define F3OP(op)                                                                              \
	static inline float3 operator op(const float3 &a, const float3 &b) {                      \
		return make_f3(a.x op b.x, a.y op b.y, a.z op b.z);                                   \
	}                                                                                         \
	static inline float3 operator op(const float3 &a, float b) {                              \
		return make_f3(a.x op b, a.y op b, a.z op b);                                         \
	}                                                                                         \
	static inline float3 operator op(float a, const float3 &b) {                              \
		return make_f3(a op b.x, a op b.y, a op b.z);                                         \
	}
F3OP(+)
F3OP(-)
F3OP(*)
F3OP(/)
#undef F3OP
static inline float3 operator-(const float3 &a) { return make_f3(-a.x, -a.y, -a.z); }
static inline float3 &operator+=(float3 &a, const float3 &b) { a = a + b; return a; }
static inline float3 &operator-=(float3 &a, const float3 &b) { a = a - b; return a; }
static inline float3 &operator*=(float3 &a, float b) { a = a * b; return a; }

#define F2OP(op)                                                                              \
	static inline float2 operator op(const float2 &a, const float2 &b) {                      \
		return make_f2(a.x op b.x, a.y op b.y);                                               \
	}                                                                                         \
	static inline float2 operator op(const float2 &a, float b) { return make_f2(a.x op b, a.y op b); } \
	static inline float2 operator op(float a, const float2 &b) { return make_f2(a op b.x, a op b.y); }
F2OP(+)
F2OP(-)
F2OP(*)
F2OP(/)
#undef F2OP

#define F4OP(op)                                                                              \
	static inline float4 operator op(const float4 &a, const float4 &b) {                      \
		return make_f4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w);                       \
	}                                                                                         \
	static inline float4 operator op(const float4 &a, float b) {                              \
		return make_f4(a.x op b, a.y op b, a.z op b, a.w op b);                               \
	}                                                                                         \
	static inline float4 operator op(float a, const float4 &b) {                              \
		return make_f4(a op b.x, a op b.y, a op b.z, a op b.w);                               \
	}
F4OP(+)
F4OP(-)
F4OP(*)
F4OP(/)
#undef F4OP

static inline float dot(const float3 &a, const float3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float dot(const float2 &a, const float2 &b) { return a.x * b.x + a.y * b.y; }
static inline float dot(const float4 &a, const float4 &b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline float3 cross(const float3 &a, const float3 &b) {
	return make_f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float length(const float3 &a) { return std::sqrt(dot(a, a)); }
static inline float3 normalize(const float3 &a) { return a * (1.f / length(a)); }

static inline float fmin(float a, float b) { return std::fmin(a, b); }
static inline float fmax(float a, float b) { return std::fmax(a, b); }
static inline float3 fmin(const float3 &a, const float3 &b) { return make_f3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
static inline float3 fmax(const float3 &a, const float3 &b) { return make_f3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
static inline float clamp(float v, float lo, float hi) { return std::fmin(std::fmax(v, lo), hi); }
static inline float fabs(float v) { return std::fabs(v); }
using std::sqrt;

static inline uint as_uint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
static inline float as_float(uint u) { float f; std::memcpy(&f, &u, 4); return f; }

static inline float2 vload2(size_t o, const float *p) { return make_f2(p[2 * o], p[2 * o + 1]); }
static inline float3 vload3(size_t o, const float *p) { return make_f3(p[3 * o], p[3 * o + 1], p[3 * o + 2]); }
static inline float4 vload4(size_t o, const float *p) { return make_f4(p[4 * o], p[4 * o + 1], p[4 * o + 2], p[4 * o + 3]); }
static inline void vstore2(const float2 &v, size_t o, float *p) { p[2 * o] = v.x; p[2 * o + 1] = v.y; }
static inline void vstore3(const float3 &v, size_t o, float *p) { p[3 * o] = v.x; p[3 * o + 1] = v.y; p[3 * o + 2] = v.z; }
static inline void vstore4(const float4 &v, size_t o, float *p) { p[4 * o] = v.x; p[4 * o + 1] = v.y; p[4 * o + 2] = v.z; p[4 * o + 3] = v.w; }

// One "work item" at a time: the harness sets the global id before each call.
static thread_local size_t refcl_global_id = 0;
static inline size_t get_global_id(int) { return refcl_global_id; }
