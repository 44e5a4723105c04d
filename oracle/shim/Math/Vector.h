// Small vector types with the operations the EDXRaster core uses
// (Clipper.h:16-33,141-149,211-224; Rasterizer.h:39-95; Renderer.cpp:229-285;
// InputBuffer.h:16-41).  Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	struct Vector2i
	{
		int x, y;
		// A single int broadcasts: FrameBuffer-sample lookups bind an int to a
		// const Vector2i& (Rasterizer.h:247,382), which needs this conversion.
		Vector2i(int v = 0) : x(v), y(v) {}
		Vector2i(int a, int b) : x(a), y(b) {}
		Vector2i operator+(const Vector2i& o) const { return Vector2i(x + o.x, y + o.y); }
		Vector2i operator-(const Vector2i& o) const { return Vector2i(x - o.x, y - o.y); }
		Vector2i operator*(int s) const { return Vector2i(x * s, y * s); }
	};

	struct Vector3i
	{
		int x, y, z;
		Vector3i(int v = 0) : x(v), y(v), z(v) {}
		Vector3i(int a, int b, int c) : x(a), y(b), z(c) {}
	};

	struct Vector2
	{
		float x, y;
		Vector2() : x(0.0f), y(0.0f) {}
		Vector2(float a, float b) : x(a), y(b) {}
		Vector2 operator+(const Vector2& o) const { return Vector2(x + o.x, y + o.y); }
		Vector2 operator-(const Vector2& o) const { return Vector2(x - o.x, y - o.y); }
		Vector2 operator*(float s) const { return Vector2(x * s, y * s); }
		static const Vector2 ZERO;
	};
	inline Vector2 operator*(float s, const Vector2& v) { return Vector2(s * v.x, s * v.y); }

	struct Vector3
	{
		float x, y, z;
		Vector3() : x(0.0f), y(0.0f), z(0.0f) {}
		Vector3(float a, float b, float c) : x(a), y(b), z(c) {}
		Vector3 operator+(const Vector3& o) const { return Vector3(x + o.x, y + o.y, z + o.z); }
		Vector3 operator-(const Vector3& o) const { return Vector3(x - o.x, y - o.y, z - o.z); }
		Vector3 operator*(float s) const { return Vector3(x * s, y * s, z * s); }
		Vector3 operator-() const { return Vector3(-x, -y, -z); }
		static const Vector3 ZERO, UNIT_X, UNIT_Y, UNIT_Z, UNIT_SCALE;
	};
	inline Vector3 operator*(float s, const Vector3& v) { return Vector3(s * v.x, s * v.y, s * v.z); }

	// Result of Vector4::HomogeneousProject.  Clipper.h:161-163,178-180 pass
	// the projected point straight into RasterTriangle::Setup(Vector3&, ...),
	// a non-const lvalue reference (RasterTriangle.h:27).  The value converts
	// to an lvalue Vector3 that lives until the end of the full expression.
	struct HomogeneousPoint
	{
		mutable Vector3 v;
		operator Vector3&() const { return v; }
	};

	struct Vector4
	{
		float x, y, z, w;
		Vector4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
		Vector4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
		Vector4 operator+(const Vector4& o) const { return Vector4(x + o.x, y + o.y, z + o.z, w + o.w); }
		Vector4 operator-(const Vector4& o) const { return Vector4(x - o.x, y - o.y, z - o.z, w - o.w); }
		Vector4 operator*(float s) const { return Vector4(x * s, y * s, z * s, w * s); }

		// Project contract of this build: one reciprocal of w, then three
		// products (x*(1/w), y*(1/w), z*(1/w)), each rounded to float.
		HomogeneousPoint HomogeneousProject() const
		{
			const float invW = 1.0f / w;
			HomogeneousPoint p;
			p.v = Vector3(x * invW, y * invW, z * invW);
			return p;
		}
		static const Vector4 ZERO;
	};
	inline Vector4 operator*(float s, const Vector4& v) { return Vector4(s * v.x, s * v.y, s * v.z, s * v.w); }

	inline const Vector2 Vector2::ZERO = Vector2(0.0f, 0.0f);
	inline const Vector3 Vector3::ZERO = Vector3(0.0f, 0.0f, 0.0f);
	inline const Vector3 Vector3::UNIT_X = Vector3(1.0f, 0.0f, 0.0f);
	inline const Vector3 Vector3::UNIT_Y = Vector3(0.0f, 1.0f, 0.0f);
	inline const Vector3 Vector3::UNIT_Z = Vector3(0.0f, 0.0f, 1.0f);
	inline const Vector3 Vector3::UNIT_SCALE = Vector3(1.0f, 1.0f, 1.0f);
	inline const Vector4 Vector4::ZERO = Vector4(0.0f, 0.0f, 0.0f, 0.0f);

	namespace Math
	{
		inline float Dot(const Vector3& a, const Vector3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
		inline Vector3 Normalize(const Vector3& v)
		{
			const float invLen = 1.0f / std::sqrt(Dot(v, v));
			return Vector3(v.x * invLen, v.y * invLen, v.z * invLen);
		}
	}
}
