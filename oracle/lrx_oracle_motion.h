// Oracle restatement of LuxRays' motion systems (test infrastructure only;
// included by lrx_oracle.cpp, compiled with -ffp-contract=off):
//   MotionSystem::Init / Sample / Bound       src/luxrays/core/geometry/motionsystem.cpp:296-345
//   InterpolatedTransform ctor / Sample / Bound                             :33-160
//   InterpolatedTransform::DecomposedTransform                              :168-270
//   Quaternion(Matrix4x4), orthoNormalize, Slerp, ToMatrix  src/luxrays/core/geometry/quaternion.cpp:27-165
//   Matrix4x4::Determinant                      src/luxrays/core/geometry/matrix4x4.cpp:67-116
// MBVHAccel applies Sample(ray.time) of a MotionTriangleMesh's motion system
// to the ray (mbvhaccel.cpp:326-327) and bounds its leaf with
// Bound(mesh box, true) (trianglemesh.cpp:268-275).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace orc_motion {

struct Vec {
	float x, y, z;
};
static inline float dot(const Vec &a, const Vec &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline Vec cross(const Vec &a, const Vec &b) {
	return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
static inline Vec mul(const Vec &v, float f) { return {f * v.x, f * v.y, f * v.z}; }  // vector.h:76-78
static inline Vec minus(const Vec &a, const Vec &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

static inline float Det2x2(float a00, float a01, float a10, float a11) { return a00 * a11 - a01 * a10; }
static inline float Det3x3(float A[3][3]) {
	return A[0][0] * Det2x2(A[1][1], A[1][2], A[2][1], A[2][2]) - A[0][1] * Det2x2(A[1][0], A[1][2], A[2][0], A[2][2]) +
			A[0][2] * Det2x2(A[1][0], A[1][1], A[2][0], A[2][1]);
}
static inline float Determinant(const float m[4][4]) {
	float result = 0, s = -1, A[3][3];
	for (int i = 0; i < 3; i++)
		for (int j = 0; j < 3; j++) A[i][j] = m[i][j + 1];
	int k = 0;
	while (true) {
		if (m[3][k] != 0.f) result += s * m[3][k] * Det3x3(A);
		if (k >= 3) break;
		s *= -1;
		for (int i = 0; i < 3; i++) A[i][k] = m[i][k];
		k++;
	}
	return result;
}

struct Quaternion {
	float w;
	Vec v;
};
static inline float qdot(const Quaternion &a, const Quaternion &b) { return a.w * b.w + dot(a.v, b.v); }
static inline Quaternion qscale(float f, const Quaternion &q) { return {q.w * f, mul(q.v, f)}; }
static inline Quaternion qadd(const Quaternion &a, const Quaternion &b) {
	return {a.w + b.w, {a.v.x + b.v.x, a.v.y + b.v.y, a.v.z + b.v.z}};
}

static void orthoNormalize(float m[4][4]) {
	float len, temp[3][3];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) temp[i][j] = m[i][j];
	len = sqrtf(temp[0][0] * temp[0][0] + temp[0][1] * temp[0][1] + temp[0][2] * temp[0][2]);
	len = (len == 0.f) ? 1.f : 1.f / len;
	temp[0][0] *= len; temp[0][1] *= len; temp[0][2] *= len;
	temp[2][0] = (temp[0][1] * temp[1][2] - temp[0][2] * temp[1][1]);
	temp[2][1] = (temp[0][2] * temp[1][0] - temp[0][0] * temp[1][2]);
	temp[2][2] = (temp[0][0] * temp[1][1] - temp[0][1] * temp[1][0]);
	len = sqrtf(temp[2][0] * temp[2][0] + temp[2][1] * temp[2][1] + temp[2][2] * temp[2][2]);
	len = (len == 0.f) ? 1.f : 1.f / len;
	temp[2][0] *= len; temp[2][1] *= len; temp[2][2] *= len;
	temp[1][0] = (temp[2][1] * temp[0][2] - temp[2][2] * temp[0][1]);
	temp[1][1] = (temp[2][2] * temp[0][0] - temp[2][0] * temp[0][2]);
	temp[1][2] = (temp[2][0] * temp[0][1] - temp[2][1] * temp[0][0]);
	len = sqrtf(temp[1][0] * temp[1][0] + temp[1][1] * temp[1][1] + temp[1][2] * temp[1][2]);
	len = (len == 0.f) ? 1.f : 1.f / len;
	temp[1][0] *= len; temp[1][1] *= len; temp[1][2] *= len;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) m[i][j] = temp[i][j];
}

static Quaternion QuaternionFromMatrix(const float m[4][4]) {
	float ortho[4][4];
	std::memcpy(ortho, m, sizeof(ortho));
	orthoNormalize(ortho);
	Quaternion q;
	const float trace = ortho[0][0] + ortho[1][1] + ortho[2][2] + 1.f;
	if (trace > 1e-6f) {
		const float s = sqrtf(trace) * 2.f;
		q.v.x = (ortho[1][2] - ortho[2][1]) / s;
		q.v.y = (ortho[2][0] - ortho[0][2]) / s;
		q.v.z = (ortho[0][1] - ortho[1][0]) / s;
		q.w = 0.25f * s;
	} else if (ortho[0][0] > ortho[1][1] && ortho[0][0] > ortho[2][2]) {
		const float s = sqrtf(1.f + ortho[0][0] - ortho[1][1] - ortho[2][2]) * 2.f;
		q.v.x = 0.25f * s;
		q.v.y = (ortho[0][1] + ortho[1][0]) / s;
		q.v.z = (ortho[2][0] + ortho[0][2]) / s;
		q.w = (ortho[1][2] - ortho[2][1]) / s;
	} else if (ortho[1][1] > ortho[2][2]) {
		const float s = sqrtf(1.f + ortho[1][1] - ortho[0][0] - ortho[2][2]) * 2.f;
		q.v.x = (ortho[0][1] + ortho[1][0]) / s;
		q.v.y = 0.25f * s;
		q.v.z = (ortho[1][2] + ortho[2][1]) / s;
		q.w = (ortho[2][0] - ortho[0][2]) / s;
	} else {
		const float s = sqrtf(1.f + ortho[2][2] - ortho[0][0] - ortho[1][1]) * 2.f;
		q.v.x = (ortho[2][0] + ortho[0][2]) / s;
		q.v.y = (ortho[1][2] + ortho[2][1]) / s;
		q.v.z = 0.25f * s;
		q.w = (ortho[0][1] - ortho[1][0]) / s;
	}
	return q;
}

static inline Quaternion Normalize(const Quaternion &q) { return qscale(1.f / sqrtf(qdot(q, q)), q); }

static Quaternion Slerp(float t, const Quaternion &q1, const Quaternion &q2) {
	float cos_phi = qdot(q1, q2);
	const float sign = (cos_phi > 0.f) ? 1.f : -1.f;
	cos_phi *= sign;
	float f1, f2;
	if (1.f - cos_phi > 1e-6f) {
		const float phi = acosf(cos_phi);
		const float sin_phi = sinf(phi);
		f1 = sinf((1.f - t) * phi) / sin_phi;
		f2 = sinf(t * phi) / sin_phi;
	} else {
		f1 = 1.f - t;
		f2 = t;
	}
	return qadd(qscale(f1, q1), qscale(sign * f2, q2));
}

static void ToMatrix(const Quaternion &q, float m[4][4]) {
	const float xx = q.v.x * q.v.x, yy = q.v.y * q.v.y, zz = q.v.z * q.v.z;
	const float xy = q.v.x * q.v.y, xz = q.v.x * q.v.z, yz = q.v.y * q.v.z;
	const float xw = q.v.x * q.w, yw = q.v.y * q.w, zw = q.v.z * q.w;
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

static inline float Lerp(float t, float v1, float v2) { return v1 + t * (v2 - v1); }  // utils.h:122-125

struct Decomposed {
	float R[4][4];
	float Sx = 0, Sy = 0, Sz = 0, Tx = 0, Ty = 0, Tz = 0;
	bool Valid = false;
};

static Decomposed Decompose(const float m[4][4]) {
	Decomposed d;
	std::memcpy(d.R, m, sizeof(d.R));
	float (&R)[4][4] = d.R;
	if (R[3][3] == 0) return d;
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j) R[i][j] /= R[3][3];
	float pmat[4][4];
	std::memcpy(pmat, R, sizeof(pmat));
	for (int i = 0; i < 3; ++i) pmat[i][3] = 0.f;
	pmat[3][3] = 1.f;
	if (Determinant(pmat) == 0.f) return d;
	if (R[3][0] != 0.f || R[3][1] != 0.f || R[3][2] != 0.f) {
		R[3][0] = R[3][1] = R[3][2] = 0.f;  // perspective terms: solved, then cleared
		R[3][3] = 1.f;
	}
	d.Tx = R[0][3];
	d.Ty = R[1][3];
	d.Tz = R[2][3];
	for (int i = 0; i < 3; ++i) R[i][3] = 0.f;
	Vec row[3];
	for (int i = 0; i < 3; ++i) row[i] = {R[i][0], R[i][1], R[i][2]};
	d.Sx = sqrtf(dot(row[0], row[0]));
	row[0] = mul(row[0], 1.f / d.Sx);
	float Sxy = dot(row[0], row[1]);
	row[1] = minus(row[1], mul(row[0], Sxy));
	d.Sy = sqrtf(dot(row[1], row[1]));
	row[1] = mul(row[1], 1.f / d.Sy);
	float Sxz = dot(row[0], row[2]);
	row[2] = minus(row[2], mul(row[0], Sxz));
	float Syz = dot(row[1], row[2]);
	row[2] = minus(row[2], mul(row[1], Syz));
	d.Sz = sqrtf(dot(row[2], row[2]));
	row[2] = mul(row[2], 1.f / d.Sz);
	if (dot(row[0], cross(row[1], row[2])) < 0.f) {
		d.Sx *= -1.f;
		d.Sy *= -1.f;
		d.Sz *= -1.f;
		for (int i = 0; i < 3; ++i) row[i] = mul(row[i], -1.f);
	}
	for (int i = 0; i < 3; ++i) {
		R[i][0] = row[i].x;
		R[i][1] = row[i].y;
		R[i][2] = row[i].z;
	}
	d.Valid = true;
	return d;
}

struct InterpolatedTransform {
	float startTime = 0, endTime = 0;
	float start[4][4], end[4][4];
	Decomposed startT, endT;
	Quaternion startQ{1, {0, 0, 0}}, endQ{1, {0, 0, 0}};
	bool hasRotation = false, hasTranslation = false, hasTranslationX = false, hasTranslationY = false,
	     hasTranslationZ = false, hasScale = false, hasScaleX = false, hasScaleY = false, hasScaleZ = false,
	     isActive = false;

	InterpolatedTransform(float st, float et, const float s[4][4], const float e[4][4]) {
		startTime = st;
		endTime = et;
		std::memcpy(start, s, sizeof(start));
		std::memcpy(end, e, sizeof(end));
		if (startTime == endTime) return;
		startT = Decompose(start);
		endT = Decompose(end);
		if (!startT.Valid || !endT.Valid) throw std::runtime_error("Singular matrix in InterpolatedTransform");
		startQ = Normalize(QuaternionFromMatrix(startT.R));
		endQ = Normalize(QuaternionFromMatrix(endT.R));
		hasTranslationX = startT.Tx != endT.Tx;
		hasTranslationY = startT.Ty != endT.Ty;
		hasTranslationZ = startT.Tz != endT.Tz;
		hasTranslation = hasTranslationX || hasTranslationY || hasTranslationZ;
		hasScaleX = startT.Sx != endT.Sx;
		hasScaleY = startT.Sy != endT.Sy;
		hasScaleZ = startT.Sz != endT.Sz;
		hasScale = hasScaleX || hasScaleY || hasScaleZ;
		hasRotation = fabsf(qdot(startQ, endQ) - 1.f) >= 1e-6f;
		isActive = hasTranslation || hasScale || hasRotation;
	}

	void Sample(float time, float out[4][4]) const {
		if (!isActive || time <= startTime) {
			std::memcpy(out, start, sizeof(start));
			return;
		}
		if (time >= endTime) {
			std::memcpy(out, end, sizeof(end));
			return;
		}
		const float w = endTime - startTime;
		const float d = time - startTime;
		const float le = d / w;
		if (hasTranslation && !(hasScale || hasRotation)) {
			std::memcpy(out, start, sizeof(start));
			if (hasTranslationX) out[0][3] = Lerp(le, startT.Tx, endT.Tx);
			if (hasTranslationY) out[1][3] = Lerp(le, startT.Ty, endT.Ty);
			if (hasTranslationZ) out[2][3] = Lerp(le, startT.Tz, endT.Tz);
			return;
		}
		if (hasRotation) ToMatrix(Slerp(le, startQ, endQ), out);
		else std::memcpy(out, startT.R, sizeof(startT.R));
		if (hasScale) {
			const float Sx = Lerp(le, startT.Sx, endT.Sx);
			const float Sy = Lerp(le, startT.Sy, endT.Sy);
			const float Sz = Lerp(le, startT.Sz, endT.Sz);
			for (int j = 0; j < 3; ++j) {
				out[0][j] = Sx * out[0][j];
				out[1][j] = Sy * out[1][j];
				out[2][j] = Sz * out[2][j];
			}
		} else {
			for (int j = 0; j < 3; ++j) {
				out[0][j] = startT.Sx * out[0][j];
				out[1][j] = startT.Sy * out[1][j];
				out[2][j] = startT.Sz * out[2][j];
			}
		}
		out[0][3] = hasTranslationX ? Lerp(le, startT.Tx, endT.Tx) : startT.Tx;
		out[1][3] = hasTranslationY ? Lerp(le, startT.Ty, endT.Ty) : startT.Ty;
		out[2][3] = hasTranslationZ ? Lerp(le, startT.Tz, endT.Tz) : startT.Tz;
	}
};

struct MotionSystem {
	std::vector<float> times;
	std::vector<InterpolatedTransform> interpolatedTransforms;

	// MotionSystem::Init: one interval per keyframe (the first degenerate)
	// plus a degenerate one at the end.
	MotionSystem(const std::vector<float> &t, const std::vector<const float (*)[4]> &transforms) : times(t) {
		size_t prev = 0;
		for (size_t k = 0; k < t.size(); ++k) {
			interpolatedTransforms.emplace_back(times[prev], times[k], transforms[prev], transforms[k]);
			prev = k;
		}
		interpolatedTransforms.emplace_back(times[prev], times[prev], transforms[prev], transforms[prev]);
	}

	void Sample(float time, float out[4][4]) const {
		size_t index = std::upper_bound(times.begin(), times.end(), time) - times.begin();
		index = std::min(index, times.size() - 1);
		interpolatedTransforms[index].Sample(time, out);
	}
};

}  // namespace orc_motion
