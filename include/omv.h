/*
 * omv.h -- C ABI of the GB300-native OpenMATERIAL BDPT render path.
 *
 * The reference renderer is a C++ class facade with no plugin or FFI layer:
 *   BDPTRenderer::setParameters / setScene / render   (pathtracer/src/renderer/BDPTRenderer.h:147-155)
 *   RenderScene::allocate / setMesh / setInstance / setMaterial / setLight /
 *               setBackground / commitScene           (pathtracer/src/scene/RenderScene.h:109-204)
 *   PinholeCamera (ViewPoint + half sizes + focus)   (pathtracer/src/sensors/PinholeCamera.h,
 *                                                     pathtracer/src/sensors/RenderSensor.h:36-49)
 * This header replaces that facade one level above the per-ray Embree call
 * (rtcIntersect1, BDPTRenderer.cpp:84), which is the only C ABI the reference hot
 * path itself crosses.  All entry points take plain pointers and sizes; every
 * pointer argument is a HOST pointer unless the entry point name ends in
 * `_device`.  The caller owns all buffers it passes; the library owns the
 * device-side scene behind the opaque `omv_scene` handle.
 *
 * Errors: every entry point returns an `omv_status` (0 = OK).  The message of
 * the last failing call on the calling thread is returned by omv_last_error().
 * No C++ exception crosses this boundary (the reference reports failures with
 * C++ exceptions, Exceptions.h:34-104, and a bool from commitScene,
 * RenderScene.cpp:194).
 *
 * Threading: an omv_scene handle is not re-entrant; distinct handles may be
 * used from different threads.  Each handle owns one CUDA stream.
 */
#ifndef OMV_H
#define OMV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t omv_status;
enum {
    OMV_OK = 0,
    OMV_ERR_INVALID_ARGUMENT = 1,
    OMV_ERR_CUDA = 2,
    OMV_ERR_OUT_OF_MEMORY = 3,
    OMV_ERR_EMPTY_SCENE = 4,     /* no valid instance: RenderScene::commitScene returns false */
    OMV_ERR_TIMEOUT = 5,         /* reserved for bounded device-side waits (no kernel waits on another today) */
    OMV_ERR_INTERNAL = 6,
    OMV_ERR_NO_DEVICE = 7
};

/* ---------------------------------------------------------------- scene --- */

/* One triangle mesh, laid out like RenderScene::setMesh (RenderScene.cpp:82-99).
 * Strides are in floats.  normals / tangents / texcoord0 may be NULL: the
 * library then derives them at commit exactly as RenderMesh::commitMesh does
 * (RenderMesh.cpp:246-264, computeNormals :300, computeTangents :332/:411). */
typedef struct omv_mesh_desc {
    int32_t num_vertices;
    int32_t num_faces;
    const uint32_t* faces;          /* 3 * num_faces vertex indices */
    const float* positions;  int32_t position_stride;
    const float* normals;    int32_t normal_stride;
    const float* tangents;   int32_t tangent_stride;   /* xyz + handedness w */
    const float* texcoord0;  int32_t texcoord_stride;
    int32_t material;               /* <0 or >= num_materials: the missing material */
    const float* texcoord1;         /* TEXCOORD_1 (same stride as texcoord0) or NULL */
} omv_mesh_desc;

/* RenderScene::setInstance (RenderScene.cpp:101-109): row-major 4x4 object-to-world. */
typedef struct omv_instance_desc {
    float transform[4][4];
    int32_t mesh;
} omv_instance_desc;

enum { OMV_MATERIAL_PBR = 0, OMV_MATERIAL_OPENMATERIAL = 1 };
enum { OMV_ALPHA_OPAQUE = 0, OMV_ALPHA_MASK = 1, OMV_ALPHA_BLEND = 2 };

/* Bitmap texture (RenderScene::setTexture, BitmapTexture.cpp:20-36): 8-bit RGBA
 * texels, rows in image order (texture coordinate v = 0 is the first row), as
 * ImageData::load converts a glTF image (ImageData.cpp:33-100). */
typedef struct omv_texture_desc {
    int32_t width;
    int32_t height;
    const uint8_t* rgba;            /* width * height * 4 */
} omv_texture_desc;

/* One texture slot of a PBR material (PbrMaterial::TextureData, PbrMaterial.h:24-34;
 * loaded at PbrMaterial.cpp:122-190).  `texture` is 1 + the index into
 * omv_scene_desc.textures (0: no texture), `texcoord` the TEXCOORD set (0 or 1),
 * and with has_transform the KHR_texture_transform rows: (u', v') = M (u, v, 1)
 * (getTextureTransform, PbrMaterial.cpp:25-57); otherwise the identity. */
typedef struct omv_texture_ref {
    int32_t texture;
    int32_t texcoord;
    int32_t has_transform;
    float transform[2][3];
} omv_texture_ref;

/* PBR: PhysicallyBasedMaterial over PbrMaterial factors (PbrMaterial.cpp:100-204).
 * OpenMaterial: OpenMaterial over AssetMaterialIor (OpenMaterial.cpp, AssetMaterialIor.cpp):
 * the (wavelength [m], value) tables of the temperature closest to `temperature`,
 * sorted by wavelength; the library evaluates AssetMaterialIor::getIor at the three
 * RGB wavelengths (Constants.h:53) once at commit. */
typedef struct omv_material_desc {
    int32_t type;
    float base_color[4];
    float metallic;
    float roughness;
    float ior;                      /* PbrMaterial default 1.5 (PbrMaterial.cpp:119) */
    int32_t alpha_mode;
    float alpha_cutoff;
    int32_t double_sided;
    float temperature;
    int32_t ior_n_count;
    const float* ior_n;             /* ior_n_count (wavelength, n) pairs */
    int32_t ior_k_count;
    const float* ior_k;             /* ior_k_count (wavelength, k) pairs */
    /* PBR textures (PhysicallyBasedMaterial.cpp:27-124, 147-167, 280-316); a
     * zero-filled block means none */
    omv_texture_ref base_color_texture;
    omv_texture_ref metallic_roughness_texture;   /* G roughness, B metallic, R occlusion */
    omv_texture_ref normal_texture;
    omv_texture_ref occlusion_texture;
    omv_texture_ref emissive_texture;
    float normal_scale;             /* normalTexture.scale (glTF default 1; used with a normal texture) */
    float occlusion_strength;       /* occlusionTexture.strength (glTF default 1; used with an occlusion
                                       or metallic-roughness texture) */
    float emissive_factor[3];       /* emission needs the factor and an emissive texture */
} omv_material_desc;

/* RenderLightPoint::set (RenderLightPoint.cpp:20-26).  `intensity` is the
 * already-flattened RGB intensity (main.cpp:362-363, including its G/B order);
 * range <= 0 means unlimited (std::numeric_limits<float>::max()). */
typedef struct omv_light_desc {
    float position[3];
    float intensity[3];
    float range;
} omv_light_desc;

/* HDRBackground (HdrBackground.cpp:38-97): equirectangular RGB float image,
 * rotation applied as dir * R (row vector times matrix) and a radiance scale. */
typedef struct omv_hdri_desc {
    int32_t width;
    int32_t height;
    const float* rgb;               /* width * height * 3 */
    float rotation[3][3];
    float scale;
} omv_hdri_desc;

typedef struct omv_scene_desc {
    int32_t num_meshes;
    const omv_mesh_desc* meshes;
    int32_t num_instances;
    const omv_instance_desc* instances;
    int32_t num_materials;
    const omv_material_desc* materials;
    int32_t num_lights;
    const omv_light_desc* lights;
    const omv_hdri_desc* hdri;      /* NULL: no background */
    int32_t num_textures;
    const omv_texture_desc* textures;
    int32_t bvh_builder;            /* OMV_BVH_*: how the binary trees are built (0: device SAH) */
} omv_scene_desc;

/* Builders of the acceleration structure (Embree's build, RenderScene.cpp:225-272).
 * Each builds a binary tree per mesh and one over the instances, which the
 * device collapses into 8-wide nodes with 16-bit quantized child boxes.
 *   OMV_BVH_SAH       on the device (default): top-down surface area heuristic,
 *                     binned above 32 items, full sweep below, all meshes at once
 *   OMV_BVH_PLOC      on the device: Morton codes, radix sort, parallel
 *                     locally-ordered clustering of all meshes at once
 *   OMV_BVH_LBVH      on the device: Morton codes, radix sort, Karras LBVH
 *   OMV_BVH_HOST_SAH  the SAH build of OMV_BVH_SAH on host threads
 * Hits do not depend on the builder; build time and traversal speed do. */
enum { OMV_BVH_SAH = 0, OMV_BVH_PLOC = 1, OMV_BVH_LBVH = 2, OMV_BVH_HOST_SAH = 3 };

typedef struct omv_scene omv_scene;

/* RenderScene::allocate + set* + commitScene.  Builds the acceleration
 * structure with desc->bvh_builder (omv_scene_info.build_ms times the whole
 * call). */
omv_status omv_scene_create(const omv_scene_desc* desc, int32_t device, omv_scene** out);
omv_status omv_scene_destroy(omv_scene* scene);

/* Several independent scenes in one handle (a group); the reference has no
 * counterpart (one RenderScene per process).  Each scene keeps its meshes,
 * instances, materials, lights and textures and gets its own top-level tree;
 * all geometry lives in one device copy and the bottom-level trees of every
 * mesh are built in one pass.  Batch jobs (omv_job.part) and adjoint jobs
 * choose their scene, so one wave pipeline renders many scenes at once.
 *   - Scene p's materials are numbered after those of scenes 0..p-1 (the
 *     group's material order), followed by the one missing material;
 *     omv_batch_set_materials and omv_scene_set_materials take the group's
 *     order.  Each scene's light pick uses its own lights only.
 *   - Either every scene has point lights or none has; the scenes share one
 *     HDRI background (the same image, rotation and scale) or none has one.
 *     descs[0].bvh_builder builds all of them.
 *   - The single-frame calls (omv_render, omv_render_device, omv_render_ids,
 *     omv_trace_rays, omv_adjoint, ...) render scene 0. */
omv_status omv_scene_create_group(int32_t num_scenes, const omv_scene_desc* descs, int32_t device, omv_scene** out);

typedef struct omv_scene_info {
    int64_t num_triangles;
    int64_t num_blas_nodes;
    int64_t num_tlas_nodes;
    int64_t device_bytes;
    double build_ms;
} omv_scene_info;
omv_status omv_scene_get_info(const omv_scene* scene, omv_scene_info* info);

/* --------------------------------------------------------------- camera --- */

/* PinholeCamera (PinholeCamera.cpp:80-95): ray = rotation * normalize(x+.5-half_w+dx,
 * y+.5-half_h+dy, focus), from `position`.  rotation rows = (left, up, forward)
 * columns as built by ViewPoint (RenderSensor.cpp:19-26). */
typedef struct omv_camera {
    int32_t width;
    int32_t height;
    float position[3];
    float rotation[3][3];
    float half_width;
    float half_height;
    float focus;
} omv_camera;

/* ----------------------------------------------------------- parameters --- */

/* OMV_ESTIMATOR_REFERENCE: BDPTRenderer's estimator (BDPTRenderer.cpp:237-302).
 * OMV_ESTIMATOR_MIS: the same, plus at every camera vertex on a PBR surface a
 * direction drawn from the HDRI's 2D alias table (cells weighted by luminance
 * times solid angle), traced as a sampled ray in that direction would be
 * (shifted origin, no end point: it reaches the environment when nothing is
 * hit) and weighted against the vertex's own sampling by the power heuristic;
 * the background seen by a sampled escape gets the complementary weight.
 * Both strategies estimate the reference sampler's own integrand, so the
 * image converges to the reference estimator's with less variance under
 * bright, small environment features.
 * No effect without an HDRI; not available in omv_render_device_static or the
 * adjoint. */
enum { OMV_ESTIMATOR_REFERENCE = 0, OMV_ESTIMATOR_MIS = 1 };

/* RendererParameters (RendererParameters.h:20-96) plus the build's own keys. */
typedef struct omv_params {
    int32_t camera_bounces;             /* cameraBouncesN, default 10 */
    int32_t light_bounces;              /* lightBouncesN,  default 10 */
    int32_t max_path_length;            /* maxPathLength,  default 8 */
    int32_t samples_per_pixel;          /* samplesPerPixel, default 20 */
    int32_t light_distance_attenuation; /* default 1 */
    float light_scale;                  /* lightScaleValue, default 100 */
    float light_min_distance;           /* lightMinDistance, default 0.01 */
    float ray_cut_value;                /* rayCutPixValue, default 0.002 */
    uint64_t seed;                      /* Philox key */
    int32_t estimator;                  /* OMV_ESTIMATOR_REFERENCE or OMV_ESTIMATOR_MIS */
    int32_t sample_offset;              /* first sample index (progressive rendering) */
    int32_t accumulate_variance;        /* also accumulate per-pixel sum of squares */
    int32_t wave_paths;                 /* paths per wavefront wave; 0 = automatic */
    int32_t time_kernels;               /* record CUDA events around every closest-hit
                                           kernel launch (omv_stats.extend_ms) */
} omv_params;

/* Fills `p` with the reference defaults (RendererParameters.h:56-89). */
void omv_params_default(omv_params* p);

/* --------------------------------------------------------------- render --- */

typedef struct omv_stats {
    int64_t paths;
    int64_t extension_rays;
    int64_t shadow_rays;
    int64_t light_rays;
    double render_ms;
    int64_t kernel_launches;
    int64_t nodes_visited;     /* 8-wide BVH nodes fetched by the extension-ray kernels (camera and light
                                  subpaths) */
    int64_t triangles_tested;  /* triangle records fetched by the extension-ray kernels */
    double extend_ms;          /* summed device time of the extension-ray kernel (time_kernels) */
    int64_t extend_launches;
    double shadow_ms;          /* summed device time of the shadow-ray kernel (time_kernels) */
    int64_t shadow_launches;
    int64_t stack_overflows;   /* warps whose traversal stack (64 entries) overflowed and dropped
                                  entries; 0 unless a tree is degenerate */
    int64_t shadow_nodes_visited;     /* nodes fetched by the shadow-ray kernel */
    int64_t shadow_triangles_tested;  /* triangle records fetched by the shadow-ray kernel */
    int64_t tail_bounce;              /* the camera bounce from which the tail kernel took each
                                         path still alive to its end, once few enough were left
                                         (the latest over the frame's waves; 0: none) */
    int64_t tail_nodes_visited;       /* nodes fetched by the tail kernel (its extension,
                                         connection and environment rays) */
    int64_t tail_triangles_tested;    /* triangle records fetched by the tail kernel */
    double tail_ms;                   /* device time of the tail kernel (time_kernels) */
} omv_stats;

/* BDPTRenderer::render (BDPTRenderer.cpp:372-393) for one camera.
 * Outputs (host, caller-allocated, any may be NULL):
 *   image_rgba  width*height*4 floats, normalised like PinholeCamera::stop
 *               (rgb / count, alpha 1; PinholeCamera.cpp:70-78)
 *   sum_rgb     width*height*3 doubles, per-pixel radiance sums (FP64)
 *   sumsq_rgb   width*height*3 doubles, per-pixel sums of squares
 *               (requires params->accumulate_variance)
 *   count       width*height uint32 sample counts
 *   stats       counters and device time of the render. */
omv_status omv_render(omv_scene* scene, const omv_camera* camera, const omv_params* params,
                      float* image_rgba, double* sum_rgb, double* sumsq_rgb, uint32_t* count,
                      omv_stats* stats);

/* Same as omv_render, but the film lives in caller-owned DEVICE memory and is
 * accumulated into (not cleared): d_sum_rgb (3*W*H doubles), d_sumsq_rgb (may
 * be NULL), d_count (W*H uint32).  `stream` is a cudaStream_t (NULL: the
 * legacy default stream, as in CUDA and torch).  Asynchronous: returns after
 * enqueueing all work. */
omv_status omv_render_device(omv_scene* scene, const omv_camera* camera, const omv_params* params,
                             double* d_sum_rgb, double* d_sumsq_rgb, uint32_t* d_count,
                             void* stream, omv_stats* stats);

/* Capacity of the fixed device scratch used by omv_render_device_static. */
#define OMV_STATIC_SCRATCH_BYTES ((size_t)32 << 20)

/* omv_render_device without any device allocation; the reference has no
 * counterpart (its BDPTRenderer::render renders on the host).
 *
 * For callers that may not allocate device memory while rendering: a host
 * framework whose own pool owns the device memory, or a render loop that cannot
 * take the device-wide synchronisation of cudaFree.  omv_render_device grows a
 * per-scene scratch buffer with cudaMalloc; this call instead carves its wave
 * queues out of one fixed array of OMV_STATIC_SCRATCH_BYTES in the library's
 * device image and makes no cudaMalloc, cudaFree or other allocating call.
 *
 *   - Same film contract as omv_render_device: caller-owned device buffers,
 *     accumulated into (zero them before the first call), asynchronous on
 *     `stream` (NULL: the legacy default stream).
 *   - The scratch bounds the wave size: params->wave_paths = 0 picks the
 *     largest wave that fits; a larger explicit wave_paths fails with
 *     OMV_ERR_INVALID_ARGUMENT and a message giving the limit.  The number of
 *     waves only changes the order of the FP64 film additions.
 *   - Nothing in the scratch has to be zero on entry: the call clears its queue
 *     and ray counters itself (cudaMemsetAsync on `stream`).
 *   - No stats and no timing (it creates no CUDA events); time_kernels must be 0.
 *   - The reference estimator only: OMV_ESTIMATOR_MIS on a scene with an HDRI
 *     fails with OMV_ERR_INVALID_ARGUMENT (its table is allocated on first use);
 *     on a scene without one it has no effect, as in omv_render_device.
 *   - Every call looks up the scratch address in the current context
 *     (cudaGetSymbolAddress) and makes sure every kernel a frame can launch is
 *     loaded (cudaFuncGetAttributes).  Under lazy module loading the first call
 *     in a context loads them, which allocates the module's device memory
 *     (the scratch included) once; later calls allocate nothing, whatever the
 *     scene (lights, alpha masks).  Make one call before any stream capture.
 *   - One scratch per device for all scenes: calls that overlap on the device
 *     (different streams or threads, any scenes) race on it; keep them ordered
 *     on one stream or serialise them. */
omv_status omv_render_device_static(omv_scene* scene, const omv_camera* camera, const omv_params* params,
                                    double* d_sum_rgb, double* d_sumsq_rgb, uint32_t* d_count,
                                    void* stream);

/* -------------------------------------------------------------- batches --- */

/* One render job of a batch.  Jobs share the scene geometry, lights, HDRI and
 * the bounce / cutoff parameters; each has its own camera (and resolution),
 * samples per pixel, sample offset, seed and material set, and accumulates
 * into its own caller-owned DEVICE film like omv_render_device (not cleared).
 * The reference renders one camera per process (main.cpp:426-511); a batch is
 * the same render loop for many cameras and material variants at once. */
typedef struct omv_job {
    omv_camera camera;
    int32_t samples_per_pixel;
    int32_t sample_offset;
    uint64_t seed;
    int32_t material_set;   /* index into omv_batch_set_materials' sets; -1: the scene's materials */
    int32_t part;           /* scene of a group (omv_scene_create_group); 0 for a single scene */
    double* d_sum_rgb;      /* 3 * width * height */
    double* d_sumsq_rgb;    /* may be NULL (required when params->accumulate_variance) */
    uint32_t* d_count;      /* width * height */
} omv_job;

/* Material variants for batch jobs: num_sets consecutive groups of
 * num_materials descriptors, in the scene's material order (the missing
 * material is appended to every set).  Which materials are alpha-masked may
 * not change.  Replaces the previous sets. */
omv_status omv_batch_set_materials(omv_scene* scene, int32_t num_sets, const omv_material_desc* sets);

enum { OMV_BATCH_GRAPH = 1 };  /* capture the batch once as a CUDA graph; replay it for an identical job list */

/* Renders all jobs through one wave pipeline: the jobs' paths are concatenated
 * (job by job, pixel by pixel, sample by sample) into waves that the same
 * persistent kernels process, with a device job table giving each path its
 * camera, material set and film.  params->samples_per_pixel, seed,
 * sample_offset and wave_paths are ignored (per job / autotuned).
 * Asynchronous on `stream` (NULL: the legacy default stream; a captured graph
 * then replays on the scene's stream, ordered after and before it by events)
 * unless stats is given. */
omv_status omv_render_batch(omv_scene* scene, int32_t num_jobs, const omv_job* jobs, const omv_params* params,
                            void* stream, int32_t flags, omv_stats* stats);

/* Times wave sizes (the ray and shadow queue capacities follow them) and the
 * threads per block of the shading kernels (128, 256) on this job list
 * (renders it several times into the jobs' films: clear them afterwards) and
 * keeps the fastest pair for the scene's later batches; *chosen_wave_paths
 * and *chosen_block_threads (either may be NULL) receive it. */
omv_status omv_batch_autotune(omv_scene* scene, int32_t num_jobs, const omv_job* jobs, const omv_params* params,
                              void* stream, int64_t* chosen_wave_paths, int32_t* chosen_block_threads);

/* ------------------------------------------------------- differentiation --- */

/* Parameters per material, in this order: base colour r, g, b, roughness and
 * metallic (glTF PBR materials); complex IOR n at 650/510/440 nm and k at
 * 650/510/440 nm (OpenMATERIAL conductors).  A material uses the slots of its
 * type (PBR 5, OpenMATERIAL 6); the others stay zero. */
#define OMV_MATERIAL_PARAMS 11

/* Replaces the scene's materials (num_materials descriptors, as given to
 * omv_scene_create, whose alpha-mask status may not change).  Geometry and
 * acceleration structure are kept.  Waits for all work queued on the device
 * (cudaDeviceSynchronize) before the table is replaced, so a render still
 * queued on any stream uses the old materials throughout and one enqueued
 * after the call the new ones. */
omv_status omv_scene_set_materials(omv_scene* scene, int32_t num_materials, const omv_material_desc* materials);

/* Gradient of an image loss with respect to the material parameters by path
 * replay: d_adjoint_rgb (DEVICE, width*height*3 floats) is dLoss/dImage for
 * the normalised image (film sum / sample count); the paths of `params`
 * (samples_per_pixel, seed, sample_offset, bounces) are replayed and
 * d_grad (DEVICE, num_materials * OMV_MATERIAL_PARAMS floats, material order
 * of the scene without the missing material) is ACCUMULATED into.  Sampled
 * directions are held fixed (GGX-sampled vertices add the score of their
 * half-vector density), so the result estimates the gradient of the expected
 * image; luminance cutoffs are not differentiated.  At most 15 camera and 15
 * light bounces and 16 materials.  Asynchronous on `stream` (NULL: the
 * legacy default stream).  The reference has no counterpart (it renders only). */
omv_status omv_adjoint(omv_scene* scene, const omv_camera* camera, const omv_params* params,
                       const float* d_adjoint_rgb, float* d_grad, void* stream);

/* One replay of a batch of adjoints: the job's scene (job.part), material set,
 * camera, samples, sample offset and seed, as the forward batch job rendered
 * them (films are not used).  d_grad (DEVICE) receives the gradient with
 * respect to the parameters of that scene's materials only, in their order
 * within the scene (num materials of the scene x OMV_MATERIAL_PARAMS). */
typedef struct omv_adjoint_job {
    omv_job job;
    const float* d_adjoint_rgb;  /* DEVICE, width * height * 3: dLoss / dImage */
    float* d_grad;               /* DEVICE, accumulated into */
} omv_adjoint_job;

/* The adjoints of all jobs, enqueued back to back on `stream` (NULL: the
 * legacy default stream); params->samples_per_pixel, seed and sample_offset
 * are taken from each job.  The reference has no counterpart. */
omv_status omv_adjoint_batch(omv_scene* scene, int32_t num_jobs, const omv_adjoint_job* jobs,
                             const omv_params* params, void* stream);

/* ----------------------------------------------------- rays / ID buffers --- */

/* One closest-hit query (the reference's sceneIntersect, BDPTRenderer.cpp:75-102,
 * including the alpha-mask retry loop).  geom = mesh index (Embree geomID),
 * inst = instance index (instID[0]), prim = local face index (primID),
 * material = mesh material index (the missing material = num_materials).
 * All ids are 0xFFFFFFFF on a miss. */
typedef struct omv_hit {
    uint32_t inst;
    uint32_t geom;
    uint32_t prim;
    uint32_t material;
    float t;
    float u;
    float v;
    uint32_t pad;
} omv_hit;

/* Traces `n` rays given as 8 floats each (org xyz, tnear, dir xyz, tfar). */
omv_status omv_trace_rays(omv_scene* scene, int64_t n, const float* rays, omv_hit* hits);

/* Primary-hit (identification) pass: the validation modes pid/gid/mid
 * (FCSubject.h:189-240, main.cpp:261-270) as integer buffers.  One primary ray
 * per pixel; `jitter` = 2*W*H uniforms in [0,1) (dx+0.5, dy+0.5 per pixel) or
 * NULL for a Philox jitter keyed by `seed`.  Outputs (any may be NULL):
 * per-pixel omv_hit, and the global primitive id (face id + faces of all lower
 * meshes, BDPTRenderer.cpp:64). */
omv_status omv_render_ids(omv_scene* scene, const omv_camera* camera, const float* jitter,
                          uint64_t seed, omv_hit* hits, uint32_t* global_prim);

/* ------------------------------------------------ false-colour validation --- */

/* Subjects of the FC_VALIDATION build's -F option (FCSubject.h:189-470, chosen
 * by name in RenderScene::setFalseColorSubject, RenderScene.cpp:130-146).  An
 * unknown name is the EmptySubject (black). */
enum {
    OMV_FC_EMPTY = 0,
    OMV_FC_PID = 1, /* global primitive id, hashed colour */
    OMV_FC_GID = 2, /* mesh (geometry) id, hashed colour */
    OMV_FC_MID = 3, /* material id: (0, G, B) of its hashed colour; missing material pink */
    OMV_FC_MMP = 4, /* PBR metallic factor: white -> blue */
    OMV_FC_RMP = 5, /* PBR roughness factor: white -> green */
    OMV_FC_MD = 6,  /* relative mesh density (log of 1/area between the scene's extremes): white -> red */
    OMV_FC_SG = 7,  /* pointwise surface gradient (vertex normals vs the face normal): 1 - g grey */
    OMV_FC_MN = 8,  /* material kind: OpenMATERIAL green, PBR blue, missing pink */
    OMV_FC_IN = 9   /* inverted normal (ray direction along the face normal): red, else green */
};

/* Subject code of an -F name ("pid", "gid", "mid", "mmp", "rmp", "md", "sg",
 * "mn", "in"); OMV_FC_EMPTY for any other name, like fcSetSubject
 * (FCHandler.cpp:82-90). */
int32_t omv_fc_subject_from_name(const char* name);

/* The false-colour pass (main.cpp:261-270 with -F): one jittered primary ray
 * per pixel, the hit material paints the subject's argument
 * (PhysicallyBasedMaterial.cpp:202-240, OpenMaterial.cpp:165-210,
 * DiffuseColorMaterial.cpp:49-89) and the colour is the pixel's value
 * (BDPTRenderer.cpp:165-168); misses are black.
 *   uniforms  HOST, 4 floats per pixel: jitter dx+.5, dy+.5 and the two
 *             uniform-hemisphere draws a missing-material hit consumes
 *             (RenderMaterial.cpp:51-58); NULL: Philox keyed by `seed`
 *   palette   HOST 0xRRGGBB per category for pid/gid/mid (the reference
 *             draws them from an entropy-seeded generator, FCSubject.h:126-135);
 *             ids at or beyond palette_size paint black, as in the reference
 * Outputs (HOST, any may be NULL): image_rgba W*H*4 floats (alpha 1), args W*H
 * (the 4 bytes of GenericFCArgument: enumerator, clamped float bits, name
 * bytes or 0/1; 0 on a miss), hits W*H omv_hit.  The reference then applies
 * gammaCorrection to the image (omv_develop / omv_tonemap). */
omv_status omv_render_fc(omv_scene* scene, const omv_camera* camera, int32_t subject, const float* uniforms,
                         uint64_t seed, const uint32_t* palette, int32_t palette_size, float* image_rgba,
                         uint32_t* args, omv_hit* hits);

/* World bounding box of the scene's valid instances (every vertex of each
 * instanced mesh through its instance transform): AssetGeometry::getBBox
 * (AssetGeometry.cpp:230-236, Node.h:132-166, Mesh.cpp:56-65) for a scene
 * flattened without the CLI's centring transform. */
omv_status omv_scene_bounds(omv_scene* scene, float lo[3], float hi[3]);

/* The light-box views (-V, main.cpp:434-458): for each of the 8 corners p of
 * the box [lo, hi] (BoundingBox::getCorners order), a camera at 2p - C looking
 * at the centre C with up (0, 1, 0), and the default intrinsics
 * (adjustToResolution, setYFoV(60), PinholeCamera.cpp:156-174).  Host only. */
omv_status omv_lightbox_cameras(const float lo[3], const float hi[3], int32_t width, int32_t height,
                                omv_camera cameras[8]);

/* --------------------------------------------------- image development --- */

/* The tail of a render in the reference's main (main.cpp:505-521) on device
 * buffers: PinholeCamera::getImpression after stop() (PinholeCamera.cpp:70-78),
 * gammaCorrection (ToneMapping.cpp:24-53), saveImage's 8-bit conversion
 * (main.cpp:92) and SimpleDenoiserMedian (Denoiser.h:24-64).  Images are
 * row-major RGBA float (16 bytes per pixel) or RGBA uint8 in DEVICE memory of
 * the current device; `stream` is a cudaStream_t (NULL: the legacy default
 * stream).  Asynchronous; nothing is allocated.
 *
 * omv_develop: one pass over a film (sums and counts as omv_render_device
 * accumulates them): the normalised linear image (rgb / count, alpha 1), the
 * gamma-corrected image gammaCorrection(img, W, H, A, gamma) gives, and its
 * 8-bit rgba (rows flipped when `flip`, the order stb writes with
 * flipVerticallyOnWrite(true)).  Any of the three outputs may be NULL.
 * The reference's call is gammaCorrection(img, W, H, 1.0f, rparams.gamma),
 * gamma 0.5 by default (RendererParameters.h:95). */
omv_status omv_develop(const double* d_sum_rgb, const uint32_t* d_count, int32_t width, int32_t height, float A,
                       float gamma, float* d_linear_rgba, float* d_tonemapped_rgba, uint8_t* d_rgba8, int32_t flip,
                       void* stream);

/* gammaCorrection (ToneMapping.cpp:24-53) in place on `pixels` RGBA pixels. */
omv_status omv_tonemap(float* d_rgba, int64_t pixels, float A, float gamma, void* stream);

/* SimpleDenoiserMedian<half_size> (Denoiser.h:24-64): the per-channel median
 * of the (2 half_size + 1)^2 window for every pixel at least half_size from
 * each edge (alpha 1 there); border pixels are copied unchanged.  The reference
 * filters in place through a temporary image; here input and output must be
 * distinct buffers.  half_size 1 (the reference's), 2 or 3. */
omv_status omv_denoise_median(const float* d_in_rgba, float* d_out_rgba, int32_t width, int32_t height,
                              int32_t half_size, void* stream);

/* saveImage's conversion (main.cpp:92): unsigned char(255 f) per channel of an
 * image in [0, 1] (values outside are clamped), rows flipped when `flip`. */
omv_status omv_rgba8(const float* d_rgba, uint8_t* d_out, int32_t width, int32_t height, int32_t flip,
                     void* stream);

/* saveImage (main.cpp:86-120) of a HOST RGBA float image with
 * ImageSaver::flipVerticallyOnWrite(true): by extension, .pfm (ImageSaver::savePfm,
 * the float rgb as stored) or .png / .bmp / .tga (8 bits per channel, the
 * buffer's last row at the top).  The reference writes those three through
 * stb_image_write; these files hold the same pixels but are not compressed.
 * .jpg is not written (OMV_ERR_INVALID_ARGUMENT). */
omv_status omv_save_image(const char* path, const float* rgba, int32_t width, int32_t height);

/* ------------------------------------------------------ kernel test hooks --- */

/* Device evaluation of the material model on host SoA inputs, for parity tests
 * against the reference's BSDFModel<ndf::GGX> (BRDFModel.h:211-337) and
 * OpenMaterial (OpenMaterial.cpp:20-163).
 *
 * omv_brdf_eval_direct: BSDFModel::evaluateDirect.  Per case 17 floats in:
 *   I(3) O(3) N(3) color(4) metallness alpha pad pad; out: brdf(3).
 * omv_brdf_sample_indirect: BSDFModel::sampleIndirect with the three uniforms
 *   supplied.  Per case 24 floats in: I(3) N(3) T(3) color(4) metallness alpha
 *   eta isTransmissive u0 u1 u2 pad pad pad; out 6 floats: O(3) brdf(3).
 * omv_om_fresnel: OpenMaterial's per-channel brdf = 0.5*(Rp+Rs)/|cos| for complex
 *   IOR; per case in: n(3) k(3) cos; out 3 floats. */
omv_status omv_brdf_eval_direct(int64_t n, const float* in, float* out);
omv_status omv_brdf_sample_indirect(int64_t n, const float* in, float* out);
omv_status omv_om_fresnel(int64_t n, const float* in, float* out);

/* The float library calls of the reference's material and environment
 * arithmetic as the device evaluates them, correctly rounded: std::sin and
 * std::cos of the sampling angles (RandomSampler.h:87-103), std::asin and
 * std::acos of the background lookup (HdrBackground.cpp:61-63), std::pow(x, 5)
 * and std::pow(x, -2) of the Fresnel and GGX terms (BRDFModel.h:44-80).
 * `function` is one of OMV_FN_*; n floats in, n floats out (host buffers).
 * sin / cos take arguments in [0, 8] (the angles 2 pi u), asin / acos in
 * [-1, 1]. */
enum {
    OMV_FN_SIN = 0,
    OMV_FN_COS = 1,
    OMV_FN_ASIN = 2,
    OMV_FN_ACOS = 3,
    OMV_FN_POW5 = 4,
    OMV_FN_POW_M2 = 5
};
omv_status omv_library_function(int32_t function, int64_t n, const float* in, float* out);

/* BitmapTexture::texture(u, v, fvec4) (BitmapTexture.cpp:73-125) on the device:
 * one width x height RGBA8 image, n (u, v) pairs in, 4 floats each out. */
omv_status omv_texture_sample(int32_t width, int32_t height, const uint8_t* rgba, int64_t n, const float* uv,
                              float* out);

/* Camera rays for given jitter uniforms (2 per pixel, row-major), 6 floats per
 * pixel out (org, dir).  Device evaluation of PinholeCamera::getRay. */
omv_status omv_camera_rays(const omv_camera* camera, const float* jitter, float* rays);

/* HDRBackground::getRadiance on the device for n directions (3 floats each). */
omv_status omv_env_radiance(omv_scene* scene, int64_t n, const float* dirs, float* rgb);

/* -------------------------------------------------------------- errors --- */

const char* omv_last_error(void);
const char* omv_version(void);

/* Optional log callback: every failing call also reports its status and
 * message to `fn` (on the failing call's thread), as the reference collects
 * Embree's error callback messages in RenderScene::getRunErrors
 * (RenderScene.cpp:14-18).  Process-wide; NULL removes it.  Set it before
 * other threads call into the library. */
typedef void (*omv_log_fn)(void* user, omv_status status, const char* message);
omv_status omv_set_log_callback(omv_log_fn fn, void* user);

/* sizeof of the public structs in this order: omv_mesh_desc, omv_instance_desc,
 * omv_material_desc, omv_light_desc, omv_hdri_desc, omv_scene_desc,
 * omv_scene_info, omv_camera, omv_params, omv_stats, omv_hit, omv_job,
 * omv_texture_desc, omv_texture_ref, omv_adjoint_job -- for binding
 * layout checks (no reference counterpart).  With out == NULL returns the
 * count; otherwise writes min(n, count) sizes and returns that number. */
int32_t omv_struct_sizes(int64_t* out, int32_t n);

#ifdef __cplusplus
}
#endif

#endif /* OMV_H */
