// Project-written stand-in for the EDXUtil prerequisites header that the
// EDXRaster core sources include first (EDXRaster/Core/Renderer.h:3,
// Clipper.h:3, RasterTriangle.h:3).  EDXUtil itself is not vendored with the
// reference and has no pinned version; every name below is defined from what
// the reference's call sites need, nothing more.  Test infrastructure only:
// this shim exists so the reference's own pipeline code can be compiled and
// run as the parity oracle.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cstring>
#include <cstdio>
#include <cassert>
#include <cmath>
#include <utility>
#include <type_traits>

typedef unsigned int uint;
typedef unsigned char _byte;

#ifndef __forceinline
#define __forceinline inline __attribute__((always_inline))
#endif

#ifndef MAX_PATH
#define MAX_PATH 260
#endif

#define sprintf_s(buf, size, ...) snprintf((buf), (size), __VA_ARGS__)

namespace EDX
{
	template<typename T>
	inline void Swap(T& a, T& b) { T t = a; a = b; b = t; }
}

#define Assert(x) assert(x)

#include "Math/EDXMath.h"
#include "Math/Vector.h"
#include "Math/Matrix.h"
#include "Containers/Array.h"
#include "Containers/DimensionalArray.h"
#include "Core/Memory.h"
#include "Core/SmartPointer.h"
#include "SIMD/SSE.h"
#include "Graphics/Color.h"
