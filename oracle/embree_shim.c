/*
 * ORACLE -- test infrastructure only.  Implementation of the Embree-4-API
 * subset declared in embree4/rtcore.h on top of the oracle BVH (oc_bvh.c), so
 * that the unmodified reference sources link and run here.
 *
 * Instrumentation (not part of Embree):
 *   - omvShimRayCount(): number of rtcIntersect1 calls (the "ray" unit);
 *   - environment OMV_SHIM_LOG=<file>: appends one 64-byte record per
 *     rtcIntersect1 call: org(3f) tnear dir(3f) tfar_in | hit(u32: 1/0)
 *     geomID instID primID u v tfar_out pad (used to pin primary-hit ids).
 */
#include "embree4/rtcore.h"
#include "oc_bvh.h"

#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

struct RTCDeviceTy {
    RTCErrorFunction err;
    void* user;
};

struct RTCGeometryTy {
    enum RTCGeometryType type;
    int refs;
    /* triangle */
    const void* idx;
    size_t idx_off, idx_stride, idx_count;
    const void* vtx;
    size_t vtx_off, vtx_stride, vtx_count;
    /* instance */
    RTCScene inst_scene;
    float xf[3][4];
};

#define SHIM_MAX_GEOMS (1 << 20)

struct RTCSceneTy {
    RTCDevice dev;
    int refs;
    unsigned n_geoms;             /* max attached id + 1 */
    RTCGeometry* geoms;           /* by id */
    unsigned cap;
    int committed;
    /* mesh scene */
    oc_tri_mesh mesh;
    int is_mesh;
    /* top scene */
    oc_accel accel;
};

static atomic_ullong g_ray_count;
static FILE* g_log;
static pthread_mutex_t g_log_mu = PTHREAD_MUTEX_INITIALIZER;
static int g_log_init;

unsigned long long omvShimRayCount(void) { return atomic_load(&g_ray_count); }

static void shim_error(RTCDevice d, enum RTCError code, const char* msg)
{
    if (d && d->err) d->err(d->user, code, msg);
}

RTCDevice rtcNewDevice(const char* config)
{
    (void)config;
    RTCDevice d = (RTCDevice)calloc(1, sizeof(*d));
    return d;
}

void rtcReleaseDevice(RTCDevice device) { free(device); }

void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction error, void* userPtr)
{
    if (!device) return;
    device->err = error;
    device->user = userPtr;
}

RTCScene rtcNewScene(RTCDevice device)
{
    RTCScene s = (RTCScene)calloc(1, sizeof(*s));
    if (!s) return NULL;
    s->dev = device;
    s->refs = 1;
    return s;
}

static void geom_release(RTCGeometry g);

void rtcReleaseScene(RTCScene scene)
{
    if (!scene) return;
    if (--scene->refs > 0) return;
    for (unsigned i = 0; i < scene->n_geoms; ++i)
        if (scene->geoms[i]) geom_release(scene->geoms[i]);
    free(scene->geoms);
    oc_free_bvh(&scene->mesh.bvh);
    oc_free_bvh(&scene->accel.tlas);
    free(scene->accel.inst);
    free(scene);
}

void rtcSetSceneFlags(RTCScene scene, enum RTCSceneFlags flags) { (void)scene; (void)flags; }
void rtcSetSceneBuildQuality(RTCScene scene, enum RTCBuildQuality quality) { (void)scene; (void)quality; }

RTCGeometry rtcNewGeometry(RTCDevice device, enum RTCGeometryType type)
{
    if (type != RTC_GEOMETRY_TYPE_TRIANGLE && type != RTC_GEOMETRY_TYPE_INSTANCE) {
        shim_error(device, RTC_ERROR_INVALID_ARGUMENT, "unsupported geometry type");
        return NULL;
    }
    RTCGeometry g = (RTCGeometry)calloc(1, sizeof(*g));
    if (!g) return NULL;
    g->type = type;
    g->refs = 1;
    return g;
}

static void geom_release(RTCGeometry g)
{
    if (!g) return;
    if (--g->refs > 0) return;
    if (g->inst_scene) rtcReleaseScene(g->inst_scene);
    free(g);
}

void rtcReleaseGeometry(RTCGeometry geometry) { geom_release(geometry); }
void rtcCommitGeometry(RTCGeometry geometry) { (void)geometry; }

void rtcSetSharedGeometryBuffer(RTCGeometry g, enum RTCBufferType type, unsigned int slot, enum RTCFormat format,
                                const void* ptr, size_t byteOffset, size_t byteStride, size_t itemCount)
{
    (void)slot;
    (void)format;
    if (!g) return;
    if (type == RTC_BUFFER_TYPE_INDEX) {
        g->idx = ptr;
        g->idx_off = byteOffset;
        g->idx_stride = byteStride;
        g->idx_count = itemCount;
    } else if (type == RTC_BUFFER_TYPE_VERTEX) {
        g->vtx = ptr;
        g->vtx_off = byteOffset;
        g->vtx_stride = byteStride;
        g->vtx_count = itemCount;
    }
}

void rtcSetGeometryInstancedScene(RTCGeometry g, RTCScene scene)
{
    if (!g || !scene) return;
    scene->refs++;
    if (g->inst_scene) rtcReleaseScene(g->inst_scene);
    g->inst_scene = scene;
}

void rtcSetGeometryTransform(RTCGeometry g, unsigned int timeStep, enum RTCFormat format, const void* xfm)
{
    (void)timeStep;
    (void)format; /* only FLOAT3X4_ROW_MAJOR is used: the top 3 rows of the 4x4 */
    if (!g || !xfm) return;
    memcpy(g->xf, xfm, sizeof(g->xf));
}

unsigned int rtcAttachGeometryByID(RTCScene scene, RTCGeometry g, unsigned int geomID)
{
    if (!scene || !g || geomID >= SHIM_MAX_GEOMS) return RTC_INVALID_GEOMETRY_ID;
    if (geomID >= scene->cap) {
        unsigned nc = scene->cap ? scene->cap : 16;
        while (nc <= geomID) nc *= 2;
        RTCGeometry* ng = (RTCGeometry*)realloc(scene->geoms, sizeof(RTCGeometry) * nc);
        if (!ng) return RTC_INVALID_GEOMETRY_ID;
        memset(ng + scene->cap, 0, sizeof(RTCGeometry) * (nc - scene->cap));
        scene->geoms = ng;
        scene->cap = nc;
    }
    g->refs++;
    if (scene->geoms[geomID]) geom_release(scene->geoms[geomID]);
    scene->geoms[geomID] = g;
    if (geomID + 1 > scene->n_geoms) scene->n_geoms = geomID + 1;
    return geomID;
}

void rtcCommitScene(RTCScene s)
{
    if (!s) return;
    /* a mesh scene holds exactly one triangle geometry; a top scene holds instances */
    RTCGeometry tri = NULL;
    unsigned tri_id = 0, n_inst = 0;
    for (unsigned i = 0; i < s->n_geoms; ++i) {
        RTCGeometry g = s->geoms[i];
        if (!g) continue;
        if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) {
            tri = g;
            tri_id = i;
        } else {
            ++n_inst;
        }
    }
    if (tri) {
        s->is_mesh = 1;
        oc_free_bvh(&s->mesh.bvh);
        s->mesh.n_tri = (int32_t)tri->idx_count;
        s->mesh.idx = (const uint32_t*)((const unsigned char*)tri->idx + tri->idx_off);
        s->mesh.idx_stride = tri->idx_stride;
        s->mesh.vtx = (const unsigned char*)tri->vtx + tri->vtx_off;
        s->mesh.vtx_stride = tri->vtx_stride;
        s->mesh.geom_id = tri_id;
        if (oc_build_mesh_bvh(&s->mesh) != 0) shim_error(s->dev, RTC_ERROR_OUT_OF_MEMORY, "bvh build failed");
    } else {
        oc_free_bvh(&s->accel.tlas);
        free(s->accel.inst);
        s->accel.inst = (oc_instance*)calloc(n_inst ? n_inst : 1, sizeof(oc_instance));
        s->accel.n_inst = 0;
        for (unsigned i = 0; i < s->n_geoms; ++i) {
            RTCGeometry g = s->geoms[i];
            if (!g || g->type != RTC_GEOMETRY_TYPE_INSTANCE || !g->inst_scene) continue;
            oc_instance* in = &s->accel.inst[s->accel.n_inst++];
            in->mesh = &g->inst_scene->mesh;
            memcpy(in->xf, g->xf, sizeof(in->xf));
            in->inst_id = i;
        }
        if (oc_build_tlas(&s->accel) != 0) shim_error(s->dev, RTC_ERROR_OUT_OF_MEMORY, "tlas build failed");
    }
    s->committed = 1;
}

void rtcInitIntersectArguments(struct RTCIntersectArguments* args)
{
    if (args) memset(args, 0, sizeof(*args));
}

static void log_record(const struct RTCRayHit* in, int hit, const struct RTCRayHit* out)
{
    if (!g_log_init) {
        pthread_mutex_lock(&g_log_mu);
        if (!g_log_init) {
            const char* p = getenv("OMV_SHIM_LOG");
            if (p && *p) g_log = fopen(p, "wb");
            g_log_init = 1;
        }
        pthread_mutex_unlock(&g_log_mu);
    }
    if (!g_log) return;
    float f[8] = {in->ray.org_x, in->ray.org_y, in->ray.org_z, in->ray.tnear,
                  in->ray.dir_x, in->ray.dir_y, in->ray.dir_z, in->ray.tfar};
    uint32_t r[6];
    r[0] = (uint32_t)hit;
    r[1] = hit ? out->hit.geomID : RTC_INVALID_GEOMETRY_ID;
    r[2] = hit ? out->hit.instID[0] : RTC_INVALID_GEOMETRY_ID;
    r[3] = hit ? out->hit.primID : RTC_INVALID_GEOMETRY_ID;
    float uvt[3] = {hit ? out->hit.u : 0.0f, hit ? out->hit.v : 0.0f, out->ray.tfar};
    pthread_mutex_lock(&g_log_mu);
    fwrite(f, sizeof(float), 8, g_log);
    fwrite(r, sizeof(uint32_t), 4, g_log);
    fwrite(uvt, sizeof(float), 2, g_log);
    fwrite(&uvt[2], sizeof(float), 1, g_log);
    fwrite(&r[5], sizeof(uint32_t), 1, g_log);
    fflush(g_log);
    pthread_mutex_unlock(&g_log_mu);
}

void rtcIntersect1(RTCScene scene, struct RTCRayHit* rh, struct RTCIntersectArguments* args)
{
    (void)args;
    atomic_fetch_add(&g_ray_count, 1ULL);
    struct RTCRayHit before = *rh;
    if (!scene || !rh) return;
    oc_ray r;
    r.org[0] = rh->ray.org_x;
    r.org[1] = rh->ray.org_y;
    r.org[2] = rh->ray.org_z;
    r.dir[0] = rh->ray.dir_x;
    r.dir[1] = rh->ray.dir_y;
    r.dir[2] = rh->ray.dir_z;
    r.tnear = rh->ray.tnear;
    r.tfar = rh->ray.tfar;
    oc_hitrec h;
    int hit = oc_intersect(&scene->accel, &r, &h);
    if (hit) {
        rh->ray.tfar = h.t;
        rh->hit.u = h.u;
        rh->hit.v = h.v;
        rh->hit.primID = h.prim;
        rh->hit.geomID = h.geom;
        rh->hit.instID[0] = h.inst;
        rh->hit.Ng_x = rh->hit.Ng_y = rh->hit.Ng_z = 0.0f;
    }
    log_record(&before, hit, rh);
}
