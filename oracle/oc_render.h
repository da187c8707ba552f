/*
 * ORACLE -- test infrastructure only (see oc_core.h).  C API of the CPU
 * restatement of the reference hot path, loaded by the tests and by bench.py's
 * CPU-baseline leg through ctypes.  Scene, camera and parameter structs are the
 * public ones of include/omv.h.
 */
#ifndef OMV_ORACLE_RENDER_H
#define OMV_ORACLE_RENDER_H

#include <stdint.h>

#include "../include/omv.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_scene oc_scene;

/* RenderScene::allocate, the set* calls and commitScene (RenderScene.cpp:51-223) + the
 * acceleration build.  Returns NULL when commitScene would fail (no valid
 * instance) or on allocation failure. */
oc_scene* oc_scene_create(const omv_scene_desc* desc);
void oc_scene_destroy(oc_scene* s);

/* Copies of the committed scene for flattening checks: per mesh the
 * interleaved vertex block (pos, normal, tangent: 10 floats per vertex) and
 * material id; per instance the normal matrix. */
int32_t oc_scene_mesh_info(const oc_scene* s, int32_t mesh, int32_t* vn, int32_t* fn, int32_t* mat);
int32_t oc_scene_mesh_vertices(const oc_scene* s, int32_t mesh, float* out);
int32_t oc_scene_normal_matrix(const oc_scene* s, int32_t inst, float* out9);

/* BDPTRenderer::render over rows [row_begin,row_end) into `film` (W*H*4,
 * PinholeCamera's RGBA sum + count layout; NOT normalised: call
 * oc_film_stop afterwards).
 *   mode 0: one std::mt19937(seed) stream consumed in row order by one
 *           thread -- the reference at -C 1, bit for bit;
 *   mode 1: `threads` workers, rows handed out by an atomic counter, each row
 *           with its own mt19937(seed ^ hash(row)) stream (same estimator,
 *           no shared-generator data race).
 * rays_out (may be NULL) receives the number of closest-hit queries. */
int32_t oc_render(const oc_scene* s, const omv_camera* cam, const omv_params* p, int32_t mode, uint32_t seed,
                  int32_t threads, int32_t row_begin, int32_t row_end, float* film, double* sumsq,
                  uint64_t* rays_out);
/* PinholeCamera::stop (PinholeCamera.cpp:70-78) */
void oc_film_stop(float* film, int64_t pixels);
/* The light-box loop (main.cpp:491-521): n views of equal resolution rendered
 * in turn from one mt19937(seed) stream, each film normalised (n*W*H*4). */
int32_t oc_render_views(const oc_scene* s, int32_t n, const omv_camera* cams, const omv_params* p, uint32_t seed,
                        float* films);

/* Replay of the false-colour / ID pass (main.cpp:261-270: spp 1, one bounce, no
 * lights, no background) with one mt19937(seed) stream: per pixel the jittered
 * primary ray (org, dir: 6 floats) and its hit. */
int32_t oc_render_ids(const oc_scene* s, const omv_camera* cam, uint32_t seed, float* rays, omv_hit* hits);

/* The false-colour pass of the FC_VALIDATION build for one subject
 * (OMV_FC_* of omv.h) with one mt19937(seed) stream; per pixel (each output
 * may be NULL) the colour (rgba, alpha 1), the 4 argument bytes, the 4
 * uniforms drawn (dx, dy, hemisphere pair of a missing-material hit, else 0)
 * and the hit.  `palette` colours the enumerated subjects (0xRRGGBB). */
int32_t oc_render_fc(const oc_scene* s, const omv_camera* cam, uint32_t seed, int32_t subject,
                     const uint32_t* palette, int32_t palette_size, float* rgba, uint32_t* args, float* uniforms,
                     omv_hit* hits);
/* scene minimum and maximum triangle density (1 / area) */
void oc_density_range(const oc_scene* s, float* out2);

/* closest-hit queries (sceneIntersect incl. the alpha-mask retry loop) */
int32_t oc_trace_rays(const oc_scene* s, int64_t n, const float* rays, omv_hit* hits);

/* kernel-level restatements; layouts as the omv_* test hooks in omv.h */
void oc_brdf_eval_direct(int64_t n, const float* in, float* out);
void oc_brdf_sample_indirect(int64_t n, const float* in, float* out);
void oc_om_fresnel(int64_t n, const float* in, float* out);
void oc_camera_rays(const omv_camera* cam, const float* jitter, float* rays);
void oc_env_radiance(const oc_scene* s, int64_t n, const float* dirs, float* rgb);
/* AssetMaterialIor::getIor linear branch (AssetMaterialIor.cpp:133-145) */
float oc_ior_lookup(const float* table, int32_t count, float wl);
/* BitmapTexture::texture(u, v, fvec4) (BitmapTexture.cpp:73-125): n pairs in, 4 floats each out */
void oc_texture_sample(int32_t w, int32_t h, const uint8_t* rgba, int64_t n, const float* uv, float* out);
/* first n uniforms of std::mt19937(seed) + uniform_real_distribution<float> */
void oc_mt_uniforms(uint32_t seed, int64_t n, float* out);

#ifdef __cplusplus
}
#endif

#endif
