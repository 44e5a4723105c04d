// Scalar math names used by the EDXRaster core (Renderer.cpp:48,168-171,
// Rasterizer.h:132-135, RasterTriangle.h:60, Shader.h:203,275).
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

#include <cmath>
#include <climits>
#include <limits>
#include <type_traits>

namespace EDX
{
	namespace Math
	{
		// Tag constants.  The SSE wrappers convert them lane-wise:
		// EDX_ZERO -> 0, EDX_ONE -> 1, EDX_INFINITY -> INT_MAX for integer
		// lanes (Rasterizer.h:56 uses it as "this edge always accepts") and
		// +inf for float lanes.
		struct ZeroTy { operator float() const { return 0.0f; } operator int() const { return 0; } };
		struct OneTy { operator float() const { return 1.0f; } operator int() const { return 1; } };
		struct InfinityTy
		{
			operator float() const { return std::numeric_limits<float>::infinity(); }
			operator int() const { return INT_MAX; }
		};
		static const ZeroTy EDX_ZERO = ZeroTy();
		static const OneTy EDX_ONE = OneTy();
		static const InfinityTy EDX_INFINITY = InfinityTy();

		static const float EDX_PI = 3.14159265358979323846f;
		static const float EDX_INV_PI = 0.31830988618379067154f;

		template<typename A, typename B>
		inline typename std::common_type<A, B>::type Min(A a, B b)
		{
			typedef typename std::common_type<A, B>::type T;
			return T(a) < T(b) ? T(a) : T(b);
		}
		template<typename A, typename B>
		inline typename std::common_type<A, B>::type Max(A a, B b)
		{
			typedef typename std::common_type<A, B>::type T;
			return T(a) > T(b) ? T(a) : T(b);
		}
		inline int Abs(int a) { return a < 0 ? -a : a; }
		inline float Abs(float a) { return std::fabs(a); }
		inline float Pow(float a, float b) { return std::pow(a, b); }
		inline float Sqrt(float a) { return std::sqrt(a); }
	}

	namespace Constants
	{
		struct TrueTy {};
		struct FalseTy {};
		static const TrueTy EDX_TRUE = TrueTy();
		static const FalseTy EDX_FALSE = FalseTy();
	}
}
