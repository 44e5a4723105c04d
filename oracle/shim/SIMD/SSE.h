// Portable 4-lane stand-ins for the EDXUtil SSE wrappers used by the EDXRaster
// core (RasterTriangle.h:192-338, Rasterizer.h:17-415, Shader.h:52-282,
// FrameBuffer.cpp:54-68, Renderer.cpp:319-362).  Lanes are plain arrays so the
// same code builds on x86-64 and AArch64 with identical results.
//
// Semantics fixed by this build (EDXUtil's are unpinned):
//  * integer lanes are int32 with two's-complement wraparound (SSE paddd /
//    psubd / pmulld);
//  * comparisons give all-ones (-1) for true and 0 for false, and a BoolSSE
//    converts to IntSSE by reinterpretation, so true becomes -1
//    (RasterTriangle.h:296-299 relies on this);
//  * IntSSE -> FloatSSE converts each lane with round-to-nearest-even
//    (cvtdq2ps), float lanes are IEEE single precision with no fused
//    multiply-add;
//  * Rsqrt is 1/sqrt rounded to float (the hardware approximation of rsqrtps
//    is CPU-specific; colour is not part of the bit-exact contract).
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

#include <cstdint>
#include <cstring>
#include <cmath>
#include <climits>

// MSVC layout of __m128i, including the byte view that Renderer.cpp:319-342
// reads through (m128i_u8).  Deliberately no <immintrin.h>: this shim must
// build unchanged on AArch64.
union __m128i
{
	int8_t m128i_i8[16];
	uint8_t m128i_u8[16];
	int16_t m128i_i16[8];
	uint16_t m128i_u16[8];
	int32_t m128i_i32[4];
	uint32_t m128i_u32[4];
	int64_t m128i_i64[2];
	uint64_t m128i_u64[2];
};

inline __m128i _mm_loadu_si128(const __m128i* p)
{
	__m128i r;
	std::memcpy(&r, p, sizeof(r));
	return r;
}

namespace EDX
{
	static inline int WrapAdd(int a, int b) { return (int)((uint32_t)a + (uint32_t)b); }
	static inline int WrapSub(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }
	static inline int WrapMul(int a, int b) { return (int)((uint32_t)a * (uint32_t)b); }

	struct BoolSSE
	{
		int32_t v[4];

		BoolSSE() = default;
		BoolSSE(const Constants::TrueTy&) { v[0] = v[1] = v[2] = v[3] = -1; }
		BoolSSE(const Constants::FalseTy&) { v[0] = v[1] = v[2] = v[3] = 0; }
		static BoolSSE FromBools(bool a, bool b, bool c, bool d)
		{
			BoolSSE r;
			r.v[0] = a ? -1 : 0; r.v[1] = b ? -1 : 0; r.v[2] = c ? -1 : 0; r.v[3] = d ? -1 : 0;
			return r;
		}
		int operator[](int i) const { return v[i]; }
	};
	inline BoolSSE operator|(const BoolSSE& a, const BoolSSE& b)
	{
		BoolSSE r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i] | b.v[i]; return r;
	}
	inline BoolSSE operator&(const BoolSSE& a, const BoolSSE& b)
	{
		BoolSSE r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i] & b.v[i]; return r;
	}
	inline BoolSSE operator!(const BoolSSE& a)
	{
		BoolSSE r; for (int i = 0; i < 4; i++) r.v[i] = ~a.v[i]; return r;
	}

	struct IntSSE
	{
		__m128i m128;

		IntSSE() = default;
		IntSSE(int a) { for (int i = 0; i < 4; i++) m128.m128i_i32[i] = a; }
		IntSSE(int a, int b, int c, int d)
		{
			m128.m128i_i32[0] = a; m128.m128i_i32[1] = b; m128.m128i_i32[2] = c; m128.m128i_i32[3] = d;
		}
		IntSSE(const __m128i& a) : m128(a) {}
		IntSSE(const BoolSSE& b) { for (int i = 0; i < 4; i++) m128.m128i_i32[i] = b.v[i]; }
		IntSSE(const Math::ZeroTy&) : IntSSE(0) {}
		IntSSE(const Math::OneTy&) : IntSSE(1) {}
		IntSSE(const Math::InfinityTy&) : IntSSE(INT_MAX) {}

		int operator[](int i) const { return m128.m128i_i32[i]; }
		int& operator[](int i) { return m128.m128i_i32[i]; }

		IntSSE& operator+=(const IntSSE& o) { for (int i = 0; i < 4; i++) m128.m128i_i32[i] = WrapAdd(m128.m128i_i32[i], o.m128.m128i_i32[i]); return *this; }
		IntSSE& operator-=(const IntSSE& o) { for (int i = 0; i < 4; i++) m128.m128i_i32[i] = WrapSub(m128.m128i_i32[i], o.m128.m128i_i32[i]); return *this; }
		IntSSE& operator*=(const IntSSE& o) { for (int i = 0; i < 4; i++) m128.m128i_i32[i] = WrapMul(m128.m128i_i32[i], o.m128.m128i_i32[i]); return *this; }
	};

#define EDX_SHIM_INT_BINOP(op, expr) \
	inline IntSSE operator op(const IntSSE& a, const IntSSE& b) \
	{ IntSSE r; for (int i = 0; i < 4; i++) { const int x = a.m128.m128i_i32[i], y = b.m128.m128i_i32[i]; r.m128.m128i_i32[i] = (expr); } return r; }
	EDX_SHIM_INT_BINOP(+, WrapAdd(x, y))
	EDX_SHIM_INT_BINOP(-, WrapSub(x, y))
	EDX_SHIM_INT_BINOP(*, WrapMul(x, y))
	EDX_SHIM_INT_BINOP(|, x | y)
	EDX_SHIM_INT_BINOP(&, x & y)
	EDX_SHIM_INT_BINOP(^, x ^ y)
#undef EDX_SHIM_INT_BINOP

#define EDX_SHIM_INT_CMP(op) \
	inline BoolSSE operator op(const IntSSE& a, const IntSSE& b) \
	{ BoolSSE r; for (int i = 0; i < 4; i++) r.v[i] = (a.m128.m128i_i32[i] op b.m128.m128i_i32[i]) ? -1 : 0; return r; }
	EDX_SHIM_INT_CMP(<)
	EDX_SHIM_INT_CMP(>)
	EDX_SHIM_INT_CMP(<=)
	EDX_SHIM_INT_CMP(>=)
	EDX_SHIM_INT_CMP(==)
	EDX_SHIM_INT_CMP(!=)
#undef EDX_SHIM_INT_CMP

	struct FloatSSE
	{
		float v[4];

		FloatSSE() = default;
		FloatSSE(float a) { v[0] = v[1] = v[2] = v[3] = a; }
		FloatSSE(float a, float b, float c, float d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
		explicit FloatSSE(const IntSSE& a) { for (int i = 0; i < 4; i++) v[i] = (float)a.m128.m128i_i32[i]; }
		FloatSSE(const Math::ZeroTy&) : FloatSSE(0.0f) {}
		FloatSSE(const Math::OneTy&) : FloatSSE(1.0f) {}
		FloatSSE(const Math::InfinityTy&) : FloatSSE((float)Math::EDX_INFINITY) {}

		float operator[](int i) const { return v[i]; }
		float& operator[](int i) { return v[i]; }

		FloatSSE& operator+=(const FloatSSE& o) { for (int i = 0; i < 4; i++) v[i] = v[i] + o.v[i]; return *this; }
		FloatSSE& operator-=(const FloatSSE& o) { for (int i = 0; i < 4; i++) v[i] = v[i] - o.v[i]; return *this; }
		FloatSSE& operator*=(const FloatSSE& o) { for (int i = 0; i < 4; i++) v[i] = v[i] * o.v[i]; return *this; }
		FloatSSE& operator/=(const FloatSSE& o) { for (int i = 0; i < 4; i++) v[i] = v[i] / o.v[i]; return *this; }
	};

#define EDX_SHIM_FLT_BINOP(op) \
	inline FloatSSE operator op(const FloatSSE& a, const FloatSSE& b) \
	{ FloatSSE r; for (int i = 0; i < 4; i++) r.v[i] = a.v[i] op b.v[i]; return r; }
	EDX_SHIM_FLT_BINOP(+)
	EDX_SHIM_FLT_BINOP(-)
	EDX_SHIM_FLT_BINOP(*)
	EDX_SHIM_FLT_BINOP(/)
#undef EDX_SHIM_FLT_BINOP
	inline FloatSSE operator-(const FloatSSE& a) { FloatSSE r; for (int i = 0; i < 4; i++) r.v[i] = -a.v[i]; return r; }

#define EDX_SHIM_FLT_CMP(op) \
	inline BoolSSE operator op(const FloatSSE& a, const FloatSSE& b) \
	{ BoolSSE r; for (int i = 0; i < 4; i++) r.v[i] = (a.v[i] op b.v[i]) ? -1 : 0; return r; }
	EDX_SHIM_FLT_CMP(<)
	EDX_SHIM_FLT_CMP(>)
	EDX_SHIM_FLT_CMP(<=)
	EDX_SHIM_FLT_CMP(>=)
	EDX_SHIM_FLT_CMP(==)
#undef EDX_SHIM_FLT_CMP

	namespace SSE
	{
		inline bool Any(const BoolSSE& b) { return (b.v[0] | b.v[1] | b.v[2] | b.v[3]) != 0; }
		inline bool All(const BoolSSE& b) { return (b.v[0] & b.v[1] & b.v[2] & b.v[3]) != 0; }
		inline FloatSSE Select(const BoolSSE& m, const FloatSSE& t, const FloatSSE& f)
		{
			FloatSSE r; for (int i = 0; i < 4; i++) r.v[i] = m.v[i] ? t.v[i] : f.v[i]; return r;
		}
		inline IntSSE Select(const BoolSSE& m, const IntSSE& t, const IntSSE& f)
		{
			IntSSE r; for (int i = 0; i < 4; i++) r.m128.m128i_i32[i] = m.v[i] ? t.m128.m128i_i32[i] : f.m128.m128i_i32[i]; return r;
		}
		inline FloatSSE Rsqrt(const FloatSSE& a)
		{
			FloatSSE r; for (int i = 0; i < 4; i++) r.v[i] = 1.0f / std::sqrt(a.v[i]); return r;
		}
	}

	struct Vec2f_SSE
	{
		union { FloatSSE x; FloatSSE u; };
		union { FloatSSE y; FloatSSE v; };

		Vec2f_SSE() : x(), y() {}
		Vec2f_SSE(float a, float b) : x(a), y(b) {}
		Vec2f_SSE(const FloatSSE& a, const FloatSSE& b) : x(a), y(b) {}
		Vec2f_SSE(const Vec2f_SSE& o) : x(o.x), y(o.y) {}
		Vec2f_SSE& operator=(const Vec2f_SSE& o) { x = o.x; y = o.y; return *this; }
	};
	inline Vec2f_SSE operator+(const Vec2f_SSE& a, const Vec2f_SSE& b) { return Vec2f_SSE(a.x + b.x, a.y + b.y); }
	inline Vec2f_SSE operator*(const FloatSSE& s, const Vec2f_SSE& a) { return Vec2f_SSE(s * a.x, s * a.y); }

	struct Vec2i_SSE
	{
		IntSSE x, y;

		Vec2i_SSE() = default;
		Vec2i_SSE(int a, int b) : x(a), y(b) {}
		Vec2i_SSE(const IntSSE& a, const IntSSE& b) : x(a), y(b) {}
		Vec2i_SSE(const Vector2i& p) : x(p.x), y(p.y) {}
		// Float -> int lanes by round-to-nearest (cvtps2dq); only exact
		// integers pass through here (Rasterizer.h:323,371).
		Vec2i_SSE(const Vec2f_SSE& f)
		{
			for (int i = 0; i < 4; i++)
			{
				x.m128.m128i_i32[i] = (int)std::nearbyint(f.x.v[i]);
				y.m128.m128i_i32[i] = (int)std::nearbyint(f.y.v[i]);
			}
		}
	};
	inline Vec2i_SSE operator+(const Vec2i_SSE& a, const Vec2i_SSE& b) { return Vec2i_SSE(a.x + b.x, a.y + b.y); }

	struct Vec3i_SSE
	{
		IntSSE x, y, z;
	};

	struct Vec3f_SSE
	{
		FloatSSE x, y, z;

		Vec3f_SSE() = default;
		Vec3f_SSE(const FloatSSE& a) : x(a), y(a), z(a) {}
		Vec3f_SSE(const FloatSSE& a, const FloatSSE& b, const FloatSSE& c) : x(a), y(b), z(c) {}
		Vec3f_SSE(float a, float b, float c) : x(a), y(b), z(c) {}
		Vec3f_SSE(const Vector3& p) : x(p.x), y(p.y), z(p.z) {}

		Vec3f_SSE& operator*=(const FloatSSE& s) { x *= s; y *= s; z *= s; return *this; }
		Vec3f_SSE& operator+=(const Vec3f_SSE& o) { x += o.x; y += o.y; z += o.z; return *this; }
	};
	inline Vec3f_SSE operator+(const Vec3f_SSE& a, const Vec3f_SSE& b) { return Vec3f_SSE(a.x + b.x, a.y + b.y, a.z + b.z); }
	inline Vec3f_SSE operator-(const Vec3f_SSE& a, const Vec3f_SSE& b) { return Vec3f_SSE(a.x - b.x, a.y - b.y, a.z - b.z); }
	inline Vec3f_SSE operator*(const FloatSSE& s, const Vec3f_SSE& a) { return Vec3f_SSE(s * a.x, s * a.y, s * a.z); }
	inline Vec3f_SSE operator*(const Vec3f_SSE& a, const FloatSSE& s) { return Vec3f_SSE(a.x * s, a.y * s, a.z * s); }
	inline Vec3f_SSE operator*(const Vec3f_SSE& a, const Vec3f_SSE& b) { return Vec3f_SSE(a.x * b.x, a.y * b.y, a.z * b.z); }

	namespace Math
	{
		inline FloatSSE Dot(const Vec3f_SSE& a, const Vec3f_SSE& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
	}
}
