// Colour types used by the EDXRaster core: Color (float RGBA) and Color4b
// (8-bit RGBA) with FromFloats (Renderer.cpp:295-299), byte construction
// (Renderer.cpp:319-342) and the MSAA resolve arithmetic (FrameBuffer.cpp:78-85).
// Float -> byte contract of this build: clamp to [0,1], scale by 255, round
// half up.  Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	struct Color4b;

	struct Color
	{
		float r, g, b, a;
		Color(float v = 0.0f) : r(v), g(v), b(v), a(v) {}
		Color(float R, float G, float B, float A = 1.0f) : r(R), g(G), b(B), a(A) {}
		inline Color(const Color4b& c);
		Color& operator+=(const Color& o) { r += o.r; g += o.g; b += o.b; a += o.a; return *this; }
		Color& operator*=(float s) { r *= s; g *= s; b *= s; a *= s; return *this; }
		Color operator*(float s) const { return Color(r * s, g * s, b * s, a * s); }
		static const Color WHITE;
		static const Color BLACK;
	};
	inline Color operator*(float s, const Color& c) { return c * s; }
	inline const Color Color::WHITE = Color(1.0f, 1.0f, 1.0f, 1.0f);
	inline const Color Color::BLACK = Color(0.0f, 0.0f, 0.0f, 1.0f);

	struct Color4b
	{
		_byte r, g, b, a;
		Color4b() : r(0), g(0), b(0), a(0) {}
		Color4b(_byte R, _byte G, _byte B, _byte A = 255) : r(R), g(G), b(B), a(A) {}
		explicit Color4b(const Color& c) { FromFloats(c.r, c.g, c.b); a = ToByte(c.a); }
		static _byte ToByte(float f)
		{
			f = f < 0.0f ? 0.0f : (f > 1.0f ? 1.0f : f);
			return (_byte)(f * 255.0f + 0.5f);
		}
		void FromFloats(float R, float G, float B)
		{
			r = ToByte(R); g = ToByte(G); b = ToByte(B); a = 255;
		}
	};
	inline Color::Color(const Color4b& c) : r(c.r / 255.0f), g(c.g / 255.0f), b(c.b / 255.0f), a(c.a / 255.0f) {}
}
