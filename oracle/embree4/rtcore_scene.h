/* Embree-4 header name used by the reference (RenderMesh.cpp:19); the shim declares everything in rtcore.h. */
#include "rtcore.h"
