// Axis-aligned box held by Mesh (Mesh.h:26,63-66).
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	struct BoundingBox
	{
		Vector3 mMin, mMax;
	};
}
