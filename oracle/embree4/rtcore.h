/*
 * Embree-4-API stand-in used ONLY to compile the reference renderer here (test
 * infrastructure, never shipped).  Intel Embree 4.1.0 is pinned by the
 * reference build (pathtracer/CMakeLists.txt:80-84) and downloaded at configure
 * time (CMakeLists.txt:100-111); it is not vendored and cannot be fetched
 * without network, so this header declares exactly the subset of the public
 * Embree 4 API that the reference calls (RenderScene.cpp:14-48,225-272,281-317,
 * RenderMesh.cpp:518-520, BDPTRenderer.cpp:42-50,57,75-86,130-131,220-229,
 * 309-320), written from Embree's documented semantics:
 *
 *   - two-level scenes: a triangle geometry per mesh scene, instance
 *     geometries (3x4 row-major object-to-world transform) in the top scene;
 *   - rtcIntersect1 = closest hit; on a hit it writes ray.tfar = t and
 *     hit.{u,v,primID,geomID,instID[0]}; on a miss the hit record is left
 *     untouched;
 *   - hit point = (1-u-v)*v0 + u*v1 + v*v2, no back-face culling.
 *
 * The implementation (embree_shim.c) is built on the oracle's own SAH BVH and
 * watertight triangle test, which define the hit contract shared with the
 * GPU traversal (ties on equal t broken by lowest instance id, then lowest
 * primitive id).
 */
#ifndef OMV_EMBREE4_SHIM_RTCORE_H
#define OMV_EMBREE4_SHIM_RTCORE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct RTCDeviceTy* RTCDevice;
typedef struct RTCSceneTy* RTCScene;
typedef struct RTCGeometryTy* RTCGeometry;

enum RTCError {
    RTC_ERROR_NONE = 0,
    RTC_ERROR_UNKNOWN = 1,
    RTC_ERROR_INVALID_ARGUMENT = 2,
    RTC_ERROR_INVALID_OPERATION = 3,
    RTC_ERROR_OUT_OF_MEMORY = 4
};

typedef void (*RTCErrorFunction)(void* userPtr, enum RTCError code, const char* str);

#define RTC_INVALID_GEOMETRY_ID ((unsigned int)-1)
#define RTC_MAX_INSTANCE_LEVEL_COUNT 1

enum RTCFormat {
    RTC_FORMAT_UNDEFINED = 0,
    RTC_FORMAT_UINT3 = 0x5003,
    RTC_FORMAT_FLOAT3 = 0x9003,
    RTC_FORMAT_FLOAT3X4_ROW_MAJOR = 0x9134
};

enum RTCBufferType {
    RTC_BUFFER_TYPE_INDEX = 0,
    RTC_BUFFER_TYPE_VERTEX = 1
};

enum RTCGeometryType {
    RTC_GEOMETRY_TYPE_TRIANGLE = 0,
    RTC_GEOMETRY_TYPE_INSTANCE = 121
};

enum RTCSceneFlags {
    RTC_SCENE_FLAG_NONE = 0,
    RTC_SCENE_FLAG_DYNAMIC = 1,
    RTC_SCENE_FLAG_COMPACT = 2,
    RTC_SCENE_FLAG_ROBUST = 4
};

enum RTCBuildQuality {
    RTC_BUILD_QUALITY_LOW = 0,
    RTC_BUILD_QUALITY_MEDIUM = 1,
    RTC_BUILD_QUALITY_HIGH = 2
};

struct RTCRay {
    float org_x, org_y, org_z;
    float tnear;
    float dir_x, dir_y, dir_z;
    float time;
    float tfar;
    unsigned int mask;
    unsigned int id;
    unsigned int flags;
};

struct RTCHit {
    float Ng_x, Ng_y, Ng_z;
    float u, v;
    unsigned int primID;
    unsigned int geomID;
    unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT];
};

struct RTCRayHit {
    struct RTCRay ray;
    struct RTCHit hit;
};

struct RTCIntersectArguments {
    unsigned int flags;
    unsigned int feature_mask;
};

RTCDevice rtcNewDevice(const char* config);
void rtcReleaseDevice(RTCDevice device);
void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction error, void* userPtr);

RTCScene rtcNewScene(RTCDevice device);
void rtcReleaseScene(RTCScene scene);
void rtcSetSceneFlags(RTCScene scene, enum RTCSceneFlags flags);
void rtcSetSceneBuildQuality(RTCScene scene, enum RTCBuildQuality quality);
void rtcCommitScene(RTCScene scene);
unsigned int rtcAttachGeometryByID(RTCScene scene, RTCGeometry geometry, unsigned int geomID);

RTCGeometry rtcNewGeometry(RTCDevice device, enum RTCGeometryType type);
void rtcReleaseGeometry(RTCGeometry geometry);
void rtcCommitGeometry(RTCGeometry geometry);
void rtcSetSharedGeometryBuffer(RTCGeometry geometry, enum RTCBufferType type, unsigned int slot,
                                enum RTCFormat format, const void* ptr, size_t byteOffset,
                                size_t byteStride, size_t itemCount);
void rtcSetGeometryInstancedScene(RTCGeometry geometry, RTCScene scene);
void rtcSetGeometryTransform(RTCGeometry geometry, unsigned int timeStep, enum RTCFormat format,
                             const void* xfm);

void rtcInitIntersectArguments(struct RTCIntersectArguments* args);
void rtcIntersect1(RTCScene scene, struct RTCRayHit* rayhit, struct RTCIntersectArguments* args);

/* shim-only instrumentation (not part of Embree): number of rtcIntersect1 calls */
unsigned long long omvShimRayCount(void);

#ifdef __cplusplus
}
#endif

#endif
