// Memory helpers used by Renderer.cpp:367-368 and InputBuffer.h:131.
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	namespace Memory
	{
		template<typename T>
		inline void SafeDeleteArray(T*& p) { delete[] p; p = nullptr; }
		template<typename T>
		inline void SafeDelete(T*& p) { delete p; p = nullptr; }
	}
}
