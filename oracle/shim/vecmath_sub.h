// Test infrastructure: layout-only stand-in for the reference's vecmath.h.
//
// The reference's NBodySimulation/vecmath.h:11-219 declares its vector types as
// unions of anonymous structs whose members have constructors, an MSVC-only
// extension that GCC rejects.  This header defines the same type names with
// plain members so that the reference's demo4.cpp / sph.h compile headless
// under GCC, and restates the free functions sph.h and demo4.cpp call
// (vecmath.h:227-330) with the same floating-point operation sequence: one
// IEEE operation per C expression, no fused multiply-add (the recipe builds
// with -ffp-contract=off), sqrtf / cosf / sinf from libm.
//
// It pre-empts the reference header by defining its include guard, so it
// must be included before any reference file.
#ifndef SPH_ORACLE_VECMATH_SUB_H
#define SPH_ORACLE_VECMATH_SUB_H
#define VECMATH_H 1

#define _USE_MATH_DEFINES
#include <math.h>
#include <stdlib.h>
#include <stdint.h>
#include <algorithm>

const float kDeg2Rad = (float)M_PI / 180.0f;

struct Vec2i {
	int x, y;
	Vec2i() : x(0), y(0) {}
	Vec2i(int ix, int iy) : x(ix), y(iy) {}
};

struct Vec2f {
	float x, y;
	Vec2f() : x(0), y(0) {}
	Vec2f(float s) : x(s), y(s) {}  // implicit, as the reference relies on it
	Vec2f(float ix, float iy) : x(ix), y(iy) {}
};

struct Mat2f {
	Vec2f col1, col2;
	Mat2f() : col1(1, 0), col2(0, 1) {}
};

struct Vec3f {
	float x, y, z;
	Vec3f() : x(0), y(0), z(0) {}
	Vec3f(float s) : x(s), y(s), z(s) {}
	Vec3f(float ix, float iy, float iz) : x(ix), y(iy), z(iz) {}
};

union Vec4f {
	struct { float x, y, z, w; };
	struct { float r, g, b, a; };
	float m[4];
	Vec4f() { x = y = z = 0; w = 1; }
	Vec4f(float ix, float iy, float iz, float iw) { x = ix; y = iy; z = iz; w = iw; }
};

const static Vec4f ColorWhite = Vec4f(1.0f, 1.0f, 1.0f, 1.0f);
const static Vec4f ColorRed = Vec4f(1.0f, 0.0f, 0.0f, 1.0f);
const static Vec4f ColorGreen = Vec4f(0.0f, 1.0f, 0.0f, 1.0f);
const static Vec4f ColorBlue = Vec4f(0.0f, 0.0f, 1.0f, 1.0f);
const static Vec4f ColorLightGray = Vec4f(0.3f, 0.3f, 0.3f, 1.0f);
const static Vec4f ColorDarkGray = Vec4f(0.2f, 0.2f, 0.2f, 1.0f);

// Component-wise operators, each a single rounding per component.
inline Vec2f operator*(const Vec2f &v, float s) { return Vec2f(v.x * s, v.y * s); }
inline Vec2f &operator*=(Vec2f &v, float s) { v = v * s; return v; }
inline Vec2f operator-(const Vec2f &v) { return Vec2f(-v.x, -v.y); }
inline Vec2f operator+(const Vec2f &p, const Vec2f &q) { return Vec2f(p.x + q.x, p.y + q.y); }
inline Vec2f &operator+=(Vec2f &p, const Vec2f &q) { p = q + p; return p; }
inline Vec2f operator-(const Vec2f &p, const Vec2f &q) { return Vec2f(p.x - q.x, p.y - q.y); }
inline Vec2f &operator-=(Vec2f &p, const Vec2f &q) { p = p - q; return p; }

inline float ScalarLerp(float a, float t, float b) { return (1.0f - t) * a + t * b; }
inline float Vec2Dot(const Vec2f &p, const Vec2f &q) { return p.x * q.x + p.y * q.y; }
inline float Vec2Length(const Vec2f &v) { return sqrtf(v.x * v.x + v.y * v.y); }
inline Vec2f Vec2Normalize(const Vec2f &v) {
	// Zero length maps to a divisor of one, so a zero vector stays zero.
	float len = Vec2Length(v);
	if (len == 0) len = 1;
	float inv = 1.0f / len;
	return Vec2f(v) * inv;
}
inline Vec2f Vec2Hadamard(const Vec2f &p, const Vec2f &q) { return Vec2f(p.x * q.x, p.y * q.y); }
inline Vec2f Vec2MultMat2(const Mat2f &m, const Vec2f &v) {
	return Vec2f(m.col1.x * v.x + m.col2.x * v.y, m.col1.y * v.x + m.col2.y * v.y);
}
// Kept exactly as the reference defines it: the squared product of the
// coordinate differences, not a squared distance (vecmath.h:292-296).
inline float Vec2DistanceSquared(const Vec2f &p, const Vec2f &q) {
	float f = (q.x - p.x) * (q.y - p.y);
	return f * f;
}
inline Vec2f Vec2Cross(const Vec2f &v, float s) { return Vec2f(s * v.y, -s * v.x); }
inline Vec2f Vec2Cross(float s, const Vec2f &v) { return Vec2f(-s * v.y, s * v.x); }
inline float Vec2Cross(const Vec2f &p, const Vec2f &q) { return p.x * q.y - p.y * q.x; }
inline float Vec2AxisToAngle(const Vec2f &axis) { return atan2f(axis.y, axis.x); }
inline Vec2f Vec2RandomDirection() {
	float d = rand() / (float)RAND_MAX;
	float angle = d * ((float)M_PI * 2.0f);
	return Vec2f(cosf(angle), sinf(angle));
}
inline Vec2f Vec2Lerp(const Vec2f &p, float t, const Vec2f &q) {
	return Vec2f(ScalarLerp(p.x, t, q.x), ScalarLerp(p.y, t, q.y));
}

inline Mat2f Mat2Identity() { return Mat2f(); }
inline Mat2f Mat2FromAngle(float angle) {
	float s = sinf(angle);
	float c = cosf(angle);
	Mat2f m;
	m.col1 = Vec2f(c, s);
	m.col2 = Vec2f(-s, c);
	return m;
}
inline Mat2f Mat2FromAxis(const Vec2f &axis) {
	Mat2f m;
	m.col1 = axis;
	m.col2 = Vec2Cross(1.0f, axis);
	return m;
}

#endif
