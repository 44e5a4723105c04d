// Mesh.h:3 includes the OBJ loader header; OBJ loading is outside the hot path
// and Mesh.cpp is not compiled, so only the name is declared.
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	class ObjMesh;
}
