/* Embree-4 header name used by the reference (RenderMesh.h:14); the shim declares everything in rtcore.h. */
#include "rtcore.h"
