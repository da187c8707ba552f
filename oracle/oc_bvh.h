/*
 * ORACLE -- test infrastructure only (see oc_core.h).
 *
 * CPU closest-hit acceleration standing in for Intel Embree 4.1.0 (the
 * reference's ray/scene intersection, RenderScene.cpp:225-272 build,
 * BDPTRenderer.cpp:84 query).  Embree is a third-party binary dependency of the
 * reference that is not present here; its published semantics are restated:
 * two-level instancing (instance transform applied to the ray, t preserved),
 * closest hit, no back-face culling, barycentrics (u,v) of vertices 1 and 2.
 *
 * The hit contract, shared bit-for-bit with the GPU traversal:
 *   - ray setup: Woop/Benthin/Wald "Watertight Ray/Triangle Intersection"
 *     (JCGT 2013) shear constants; the triangle test in the instance's object
 *     space, float arithmetic in a fixed order, a double-precision retry of the
 *     2D edge functions when one is exactly zero;
 *   - world-to-object transform: inverse of the 3x4 instance matrix, computed in
 *     double and rounded to float;
 *   - a hit is accepted for tnear <= t <= tfar; among equal t the lowest
 *     (instance id, primitive id) wins, so the result does not depend on the
 *     BVH layout as long as every BVH box test is conservative.
 */
#ifndef OMV_ORACLE_BVH_H
#define OMV_ORACLE_BVH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_bnode {
    float lo[3];
    int32_t left;  /* internal: left child index (right = left + 1); leaf: first item */
    float hi[3];
    int32_t count; /* 0: internal node; > 0: leaf item count */
} oc_bnode;

typedef struct oc_bvh {
    int32_t n_nodes;
    oc_bnode* nodes;
    int32_t n_items;
    int32_t* items;
} oc_bvh;

typedef struct oc_tri_mesh {
    int32_t n_tri;
    const uint32_t* idx;      /* base of the index buffer */
    size_t idx_stride;        /* bytes */
    const unsigned char* vtx; /* base of the vertex buffer, byte offset applied */
    size_t vtx_stride;        /* bytes */
    uint32_t geom_id;
    oc_bvh bvh;
} oc_tri_mesh;

typedef struct oc_instance {
    const oc_tri_mesh* mesh;
    float xf[3][4];
    float inv[3][4];
    float lo[3], hi[3];
    uint32_t inst_id;
} oc_instance;

typedef struct oc_accel {
    int32_t n_inst;
    oc_instance* inst;
    oc_bvh tlas;
} oc_accel;

typedef struct oc_ray {
    float org[3];
    float tnear;
    float dir[3];
    float tfar;
} oc_ray;

typedef struct oc_hitrec {
    uint32_t inst, geom, prim;
    float t, u, v;
} oc_hitrec;

/* vertex fetch of a triangle mesh */
const float* oc_mesh_vertex(const oc_tri_mesh* m, uint32_t vi);
void oc_mesh_face(const oc_tri_mesh* m, int32_t f, uint32_t out[3]);

int oc_build_mesh_bvh(oc_tri_mesh* m);
void oc_free_bvh(oc_bvh* b);
/* affine inverse of a 3x4 matrix, computed in double, rounded to float */
void oc_affine_inverse(const float xf[3][4], float inv[3][4]);
int oc_build_tlas(oc_accel* a);

/* closest hit; returns 1 and fills *h on a hit */
int oc_intersect(const oc_accel* a, const oc_ray* r, oc_hitrec* h);

#ifdef __cplusplus
}
#endif

#endif
