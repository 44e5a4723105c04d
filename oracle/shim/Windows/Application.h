// Application::GetBaseDirectory (Renderer.cpp:355).
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	struct Application
	{
		static const char* GetBaseDirectory() { return "."; }
	};
}
