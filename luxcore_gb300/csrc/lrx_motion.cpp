// Motion systems of motion-blurred instances, on the host: keyframes are
// decomposed once into MotionInterval records (uploaded for the traversal
// to sample at each ray's time) and the instance's swept world box is
// computed for the top-level BVH.  Restates, with the same FP32 operation
// order (compiled with -ffp-contract=off):
//   MotionSystem::Init / Sample / Bound     src/luxrays/core/geometry/motionsystem.cpp:296-345
//   InterpolatedTransform ctor / Sample / Bound                           :33-160
//   DecomposedTransform                                                   :168-270
//   Quaternion(Matrix4x4), orthoNormalize, Slerp, ToMatrix   src/luxrays/core/geometry/quaternion.cpp:27-165
//   Matrix4x4::Determinant                          src/luxrays/core/geometry/matrix4x4.cpp:67-116
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lrx_common.cuh"
#include "lrx_internal.h"

namespace lrx {

namespace {

typedef float M44[4][4];

float det2(float a00, float a01, float a10, float a11) { return a00 * a11 - a01 * a10; }

float det3(const float A[3][3]) {
	return A[0][0] * det2(A[1][1], A[1][2], A[2][1], A[2][2]) - A[0][1] * det2(A[1][0], A[1][2], A[2][0], A[2][2]) +
			A[0][2] * det2(A[1][0], A[1][1], A[2][0], A[2][1]);
}

// Matrix4x4::Determinant: expansion along the last row
float determinant(const M44 &m) {
	float result = 0.f, s = -1.f, A[3][3];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) A[i][j] = m[i][j + 1];
	for (int k = 0;; ++k) {
		if (m[3][k] != 0.f) result += s * m[3][k] * det3(A);
		if (k >= 3) break;
		s *= -1.f;
		for (int i = 0; i < 3; ++i) A[i][k] = m[i][k];
	}
	return result;
}

struct V {
	float x, y, z;
};
float vdot(const V &a, const V &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V vcross(const V &a, const V &b) {
	return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
V vscale(const V &v, float f) { return {f * v.x, f * v.y, f * v.z}; }
V vsub(const V &a, const V &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

struct Decomposed {
	bool valid = false;
	float Sx = 0, Sy = 0, Sz = 0, Tx = 0, Ty = 0, Tz = 0;
	M44 R;
};

Decomposed decompose(const M44 &m) {
	Decomposed d;
	std::memcpy(d.R, m, sizeof(M44));
	M44 &R = d.R;
	if (R[3][3] == 0.f) return d;
	const float r33 = R[3][3];  // every element, R[3][3] last, is divided by its original value
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j) R[i][j] /= r33;
	M44 pmat;
	std::memcpy(pmat, R, sizeof(M44));
	for (int i = 0; i < 3; ++i) pmat[i][3] = 0.f;
	pmat[3][3] = 1.f;
	if (determinant(pmat) == 0.f) return d;
	if (R[3][0] != 0.f || R[3][1] != 0.f || R[3][2] != 0.f) {
		// perspective partition: solved only to be cleared (its terms are unused)
		R[3][0] = R[3][1] = R[3][2] = 0.f;
		R[3][3] = 1.f;
	}
	d.Tx = R[0][3];
	d.Ty = R[1][3];
	d.Tz = R[2][3];
	for (int i = 0; i < 3; ++i) R[i][3] = 0.f;
	V row[3];
	for (int i = 0; i < 3; ++i) row[i] = {R[i][0], R[i][1], R[i][2]};
	d.Sx = std::sqrt(vdot(row[0], row[0]));
	row[0] = vscale(row[0], 1.f / d.Sx);
	float Sxy = vdot(row[0], row[1]);
	row[1] = vsub(row[1], vscale(row[0], Sxy));
	d.Sy = std::sqrt(vdot(row[1], row[1]));
	row[1] = vscale(row[1], 1.f / d.Sy);
	const float Sxz = vdot(row[0], row[2]);
	row[2] = vsub(row[2], vscale(row[0], Sxz));
	const float Syz = vdot(row[1], row[2]);
	row[2] = vsub(row[2], vscale(row[1], Syz));
	d.Sz = std::sqrt(vdot(row[2], row[2]));
	row[2] = vscale(row[2], 1.f / d.Sz);
	if (vdot(row[0], vcross(row[1], row[2])) < 0.f) {
		d.Sx *= -1.f;
		d.Sy *= -1.f;
		d.Sz *= -1.f;
		for (int i = 0; i < 3; ++i) row[i] = vscale(row[i], -1.f);
	}
	for (int i = 0; i < 3; ++i) {
		R[i][0] = row[i].x;
		R[i][1] = row[i].y;
		R[i][2] = row[i].z;
	}
	d.valid = true;
	return d;
}

struct Quat {
	float w, x, y, z;
};
float qdot(const Quat &a, const Quat &b) { return a.w * b.w + (a.x * b.x + a.y * b.y + a.z * b.z); }

void ortho_normalize(M44 &m) {
	float len, t[3][3];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) t[i][j] = m[i][j];
	len = std::sqrt(t[0][0] * t[0][0] + t[0][1] * t[0][1] + t[0][2] * t[0][2]);
	len = (len == 0.f) ? 1.f : 1.f / len;
	t[0][0] *= len; t[0][1] *= len; t[0][2] *= len;
	t[2][0] = (t[0][1] * t[1][2] - t[0][2] * t[1][1]);
	t[2][1] = (t[0][2] * t[1][0] - t[0][0] * t[1][2]);
	t[2][2] = (t[0][0] * t[1][1] - t[0][1] * t[1][0]);
	len = std::sqrt(t[2][0] * t[2][0] + t[2][1] * t[2][1] + t[2][2] * t[2][2]);
	len = (len == 0.f) ? 1.f : 1.f / len;
	t[2][0] *= len; t[2][1] *= len; t[2][2] *= len;
	t[1][0] = (t[2][1] * t[0][2] - t[2][2] * t[0][1]);
	t[1][1] = (t[2][2] * t[0][0] - t[2][0] * t[0][2]);
	t[1][2] = (t[2][0] * t[0][1] - t[2][1] * t[0][0]);
	len = std::sqrt(t[1][0] * t[1][0] + t[1][1] * t[1][1] + t[1][2] * t[1][2]);
	len = (len == 0.f) ? 1.f : 1.f / len;
	t[1][0] *= len; t[1][1] *= len; t[1][2] *= len;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) m[i][j] = t[i][j];
}

Quat quat_from_matrix(const M44 &m) {
	M44 o;
	std::memcpy(o, m, sizeof(M44));
	ortho_normalize(o);
	Quat q;
	const float trace = o[0][0] + o[1][1] + o[2][2] + 1.f;
	if (trace > 1e-6f) {
		const float s = std::sqrt(trace) * 2.f;
		q.x = (o[1][2] - o[2][1]) / s;
		q.y = (o[2][0] - o[0][2]) / s;
		q.z = (o[0][1] - o[1][0]) / s;
		q.w = 0.25f * s;
	} else if (o[0][0] > o[1][1] && o[0][0] > o[2][2]) {
		const float s = std::sqrt(1.f + o[0][0] - o[1][1] - o[2][2]) * 2.f;
		q.x = 0.25f * s;
		q.y = (o[0][1] + o[1][0]) / s;
		q.z = (o[2][0] + o[0][2]) / s;
		q.w = (o[1][2] - o[2][1]) / s;
	} else if (o[1][1] > o[2][2]) {
		const float s = std::sqrt(1.f + o[1][1] - o[0][0] - o[2][2]) * 2.f;
		q.x = (o[0][1] + o[1][0]) / s;
		q.y = 0.25f * s;
		q.z = (o[1][2] + o[2][1]) / s;
		q.w = (o[2][0] - o[0][2]) / s;
	} else {
		const float s = std::sqrt(1.f + o[2][2] - o[0][0] - o[1][1]) * 2.f;
		q.x = (o[2][0] + o[0][2]) / s;
		q.y = (o[1][2] + o[2][1]) / s;
		q.z = 0.25f * s;
		q.w = (o[0][1] - o[1][0]) / s;
	}
	return q;
}

Quat quat_normalize(const Quat &q) {
	const float f = 1.f / std::sqrt(qdot(q, q));
	return {q.w * f, f * q.x, f * q.y, f * q.z};
}

// The interval's constant part of Slerp: its flags and phi, sinf(phi).
void slerp_setup(const Quat &q1, const Quat &q2, MotionInterval &it) {
	float cos_phi = qdot(q1, q2);
	const float sign = (cos_phi > 0.f) ? 1.f : -1.f;
	cos_phi *= sign;
	if (sign < 0.f) it.flags |= kMiSlerpNegate;
	if (1.f - cos_phi > 1e-6f) {
		it.phi = std::acos(cos_phi);
		it.sin_phi = std::sin(it.phi);
	} else {
		it.flags |= kMiSlerpLinear;
	}
}

// Slerp at t from the interval's quaternions and slerp_setup's constants
Quat slerp(float t, const MotionInterval &it) {
	const Quat q1{it.q0[0], it.q0[1], it.q0[2], it.q0[3]}, q2{it.q1[0], it.q1[1], it.q1[2], it.q1[3]};
	const float sign = (it.flags & kMiSlerpNegate) ? -1.f : 1.f;
	float f1, f2;
	if (!(it.flags & kMiSlerpLinear)) {
		f1 = std::sin((1.f - t) * it.phi) / it.sin_phi;
		f2 = std::sin(t * it.phi) / it.sin_phi;
	} else {
		f1 = 1.f - t;
		f2 = t;
	}
	const float g = sign * f2;
	return {q1.w * f1 + q2.w * g, f1 * q1.x + g * q2.x, f1 * q1.y + g * q2.y, f1 * q1.z + g * q2.z};
}

void quat_to_matrix(const Quat &q, M44 &m) {
	const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
	const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
	const float xw = q.x * q.w, yw = q.y * q.w, zw = q.z * q.w;
	m[0][0] = 1.f - 2.f * (yy + zz);
	m[1][0] = 2.f * (xy - zw);
	m[2][0] = 2.f * (xz + yw);
	m[0][1] = 2.f * (xy + zw);
	m[1][1] = 1.f - 2.f * (xx + zz);
	m[2][1] = 2.f * (yz - xw);
	m[0][2] = 2.f * (xz - yw);
	m[1][2] = 2.f * (yz + xw);
	m[2][2] = 1.f - 2.f * (xx + yy);
	m[0][3] = m[1][3] = m[2][3] = 0.f;
	m[3][0] = m[3][1] = m[3][2] = 0.f;
	m[3][3] = 1.f;
}

float lerp(float t, float a, float b) { return a + t * (b - a); }

// InterpolatedTransform constructor
bool make_interval(float st, float et, const float *s, const float *e, MotionInterval &it) {
	std::memset(&it, 0, sizeof(it));
	it.start_time = st;
	it.end_time = et;
	std::memcpy(it.start_m, s, 64);
	std::memcpy(it.end_m, e, 64);
	if (st == et) return true;
	const Decomposed a = decompose(*reinterpret_cast<const M44 *>(s)), b = decompose(*reinterpret_cast<const M44 *>(e));
	if (!a.valid || !b.valid) return false;
	const Quat q0 = quat_normalize(quat_from_matrix(a.R)), q1 = quat_normalize(quat_from_matrix(b.R));
	std::memcpy(it.start_r, a.R, 64);
	const float s0[3] = {a.Sx, a.Sy, a.Sz}, t0[3] = {a.Tx, a.Ty, a.Tz};
	const float s1[3] = {b.Sx, b.Sy, b.Sz}, t1[3] = {b.Tx, b.Ty, b.Tz};
	std::memcpy(it.s0, s0, 12);
	std::memcpy(it.t0, t0, 12);
	std::memcpy(it.s1, s1, 12);
	std::memcpy(it.t1, t1, 12);
	const float qa[4] = {q0.w, q0.x, q0.y, q0.z}, qb[4] = {q1.w, q1.x, q1.y, q1.z};
	std::memcpy(it.q0, qa, 16);
	std::memcpy(it.q1, qb, 16);
	uint32_t f = 0;
	if (a.Tx != b.Tx) f |= kMiTransX;
	if (a.Ty != b.Ty) f |= kMiTransY;
	if (a.Tz != b.Tz) f |= kMiTransZ;
	if (a.Sx != b.Sx) f |= kMiScaleX;
	if (a.Sy != b.Sy) f |= kMiScaleY;
	if (a.Sz != b.Sz) f |= kMiScaleZ;
	if (std::fabs(qdot(q0, q1) - 1.f) >= 1e-6f) f |= kMiRotation;
	if (f) f |= kMiActive;
	it.flags = f;
	slerp_setup(q0, q1, it);
	return true;
}

// InterpolatedTransform::Sample
void sample_interval(const MotionInterval &it, float time, M44 &out) {
	const M44 &sm = *reinterpret_cast<const M44 *>(it.start_m);
	if (!(it.flags & kMiActive) || time <= it.start_time) {
		std::memcpy(out, sm, sizeof(M44));
		return;
	}
	if (time >= it.end_time) {
		std::memcpy(out, it.end_m, sizeof(M44));
		return;
	}
	const float w = it.end_time - it.start_time, d = time - it.start_time, le = d / w;
	if ((it.flags & kMiTrans) && !(it.flags & (kMiScale | kMiRotation))) {
		std::memcpy(out, sm, sizeof(M44));
		if (it.flags & kMiTransX) out[0][3] = lerp(le, it.t0[0], it.t1[0]);
		if (it.flags & kMiTransY) out[1][3] = lerp(le, it.t0[1], it.t1[1]);
		if (it.flags & kMiTransZ) out[2][3] = lerp(le, it.t0[2], it.t1[2]);
		return;
	}
	if (it.flags & kMiRotation) {
		quat_to_matrix(slerp(le, it), out);
	} else {
		std::memcpy(out, it.start_r, sizeof(M44));
	}
	float S[3];
	for (int k = 0; k < 3; ++k) S[k] = (it.flags & kMiScale) ? lerp(le, it.s0[k], it.s1[k]) : it.s0[k];
	for (int j = 0; j < 3; ++j) {
		out[0][j] = S[0] * out[0][j];
		out[1][j] = S[1] * out[1][j];
		out[2][j] = S[2] * out[2][j];
	}
	out[0][3] = (it.flags & kMiTransX) ? lerp(le, it.t0[0], it.t1[0]) : it.t0[0];
	out[1][3] = (it.flags & kMiTransY) ? lerp(le, it.t0[1], it.t1[1]) : it.t0[1];
	out[2][3] = (it.flags & kMiTransZ) ? lerp(le, it.t0[2], it.t1[2]) : it.t0[2];
}

void xform_point(const M44 &m, const float p[3], float out[3]) {
	const float x = p[0], y = p[1], z = p[2];
	float r[3] = {m[0][0] * x + m[0][1] * y + m[0][2] * z + m[0][3], m[1][0] * x + m[1][1] * y + m[1][2] * z + m[1][3],
			m[2][0] * x + m[2][1] * y + m[2][2] * z + m[2][3]};
	const float w = m[3][0] * x + m[3][1] * y + m[3][2] * z + m[3][3];
	if (w != 1.f) {
		const float inv = 1.f / w;
		for (float &v : r) v *= inv;
	}
	std::memcpy(out, r, 12);
}

}  // namespace

lrx_status motion_intervals(const float *times, const float *mats, uint32_t count,
		std::vector<MotionInterval> &out) {
	out.clear();
	if (count == 0 || !times || !mats) {
		set_error("motion system: no keyframes");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	for (uint32_t k = 1; k < count; ++k)
		if (!(times[k] > times[k - 1])) {  // MotionTransform::Valid: strictly increasing
			set_error("motion system: keyframe times must be strictly increasing");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	for (uint64_t k = 0; k < 16ull * count; ++k)
		if (!std::isfinite(mats[k]) || !std::isfinite(times[k / 16])) {
			set_error("motion system: non-finite keyframe");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	// MotionSystem::Init: (t[k-1], t[k]) for k = 0..count-1 (the first one
	// degenerate), then (t[last], t[last]); Sample uses the first `count`.
	out.resize(count + 1);
	for (uint32_t k = 0; k <= count; ++k) {
		const uint32_t a = k == 0 ? 0 : (k == count ? count - 1 : k - 1), b = k == count ? count - 1 : k;
		if (!make_interval(times[a], times[b], mats + 16ull * a, mats + 16ull * b, out[k])) {
			set_error("motion system: singular keyframe matrix");
			return LRX_ERR_INVALID_ARGUMENT;
		}
	}
	return LRX_OK;
}

// MotionSystem::Bound(box, storingGlobal2Local = true): the union over every
// interval of 1,025 sampled matrices, inverted, applied to the box.
lrx_status motion_bound(const std::vector<MotionInterval> &its, const float lo[3], const float hi[3], float olo[3],
		float ohi[3]) {
	for (int k = 0; k < 3; ++k) {
		olo[k] = INFINITY;
		ohi[k] = -INFINITY;
	}
	const float N = 1024.f;
	for (const MotionInterval &it : its) {
		for (float i = 0; i <= N; ++i) {
			const float t = lerp(i / N, it.start_time, it.end_time);
			M44 m, inv;
			sample_interval(it, t, m);
			if (!host_matrix_inverse(&m[0][0], &inv[0][0])) {
				set_error("motion system: singular sampled matrix");
				return LRX_ERR_INVALID_ARGUMENT;
			}
			for (int c = 0; c < 8; ++c) {
				const float p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
				float q[3];
				xform_point(inv, p, q);
				for (int k = 0; k < 3; ++k) {
					olo[k] = std::fmin(olo[k], q[k]);
					ohi[k] = std::fmax(ohi[k], q[k]);
				}
			}
		}
	}
	return LRX_OK;
}

}  // namespace lrx
