// Frame dump used only when SetWriteFrames(true) (Renderer.cpp:114-115,
// 352-358); a no-op here.  Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	struct Bitmap
	{
		static void SaveBitmapFile(const char*, const _byte*, int, int) {}
	};
}
