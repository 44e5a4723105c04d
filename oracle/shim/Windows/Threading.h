// GetNumberOfCores (Renderer.cpp:55).  Tile.h:34 holds per-core bins in a
// fixed array of 12, so the count is capped at 12.  The harness may pin it
// with EDXR_REF_CORES.  Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

#include <thread>
#include <cstdlib>

namespace EDX
{
	inline int GetNumberOfCores()
	{
		int n = (int)std::thread::hardware_concurrency();
		if (const char* e = std::getenv("EDXR_REF_CORES"))
			n = std::atoi(e);
		if (n < 1) n = 1;
		if (n > 12) n = 12;
		return n;
	}
}
