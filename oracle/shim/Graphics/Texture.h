// Texture interface used by LambertianAlbedoPixelShader (Shader.h:231-239)
// and RenderStates (RenderStates.h:17,28).  Only a constant-colour texture is
// provided: texture loading and filtering are not part of the hot path this
// build re-implements.  Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"
#include "Graphics/Color.h"

namespace EDX
{
	enum class TextureFilter
	{
		Nearest,
		Linear,
		TriLinear,
		Anisotropic4x,
		Anisotropic8x,
		Anisotropic16x
	};

	template<typename T>
	class Texture2D
	{
	public:
		virtual ~Texture2D() {}
		virtual T Sample(const Vector2& texCoord, const Vector2* differentials) const = 0;
		virtual void SetFilter(const TextureFilter filter) {}
	};

	template<typename T>
	class ConstantTexture2D : public Texture2D<T>
	{
		T mVal;
	public:
		ConstantTexture2D(const T& v) : mVal(v) {}
		T Sample(const Vector2&, const Vector2*) const override { return mVal; }
	};
}
