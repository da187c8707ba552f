// Host-side scene handle (the object behind the opaque omv_scene*) and the
// entry points of the render path used by the C ABI layer (capi.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/omv.h"
#include "omv_types.h"

// A failed call throws; the runtime's non-sticky error state is cleared so
// that the next call on the handle starts clean (an allocation that does not
// fit is reported as out of memory and the handle stays usable).
#define OMV_CUDA(x)                                                                               \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) {                                                                  \
            (void)cudaGetLastError();                                                             \
            if (e_ == cudaErrorMemoryAllocation)                                                  \
                throw omv::DeviceOutOfMemory(std::string(#x) + ": " + cudaGetErrorString(e_));    \
            throw omv::CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));                \
        }                                                                                         \
    } while (0)

namespace omv {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct DeviceOutOfMemory : CudaError {
    using CudaError::CudaError;
};
struct ArgError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// reusable per-scene device work space of the wavefront renderer
struct RenderScratch {
    int64_t wave_cap = 0;
    int light_slots = 0;
    int shadow_slots = 0;
    void* base = nullptr;  // one allocation, carved into the arrays below
    size_t bytes = 0;
    float4* tp = nullptr;        // camera throughput (outFactor of the last vertex)
    float4* rad = nullptr;       // per-path radiance
    float4* ltp = nullptr;       // light throughput
    float4* lrad = nullptr;      // light Rad (xyz) and distance term (w)
    uint32_t* lmeta = nullptr;   // light index | (light vertex count << 16)
    float4* lv_pos = nullptr;    // [light_slots][wave_cap]
    float4* lv_rad = nullptr;    // [light_slots][wave_cap]
    float4* rq[2] = {nullptr, nullptr};  // ray queues: 2 float4 per entry
    uint4* hits = nullptr;       // per queue entry
    uint32_t* path_job = nullptr;  // batch: job of each path
    float4* sq = nullptr;        // shadow queue: 3 float4 per entry
    uint32_t* ctr = nullptr;     // per-wave queue and work counters
    unsigned long long* stats = nullptr;  // cumulative ray counters
};

constexpr int kMaxCounters = 512;

// One job of a batch render (device copy): its camera, samples, seed and
// material table, its film, and where its paths and pixels start in the
// batch's concatenated path and pixel ranges.
struct DevJob {
    omv_camera cam;
    int64_t path_base;
    uint32_t pixel_base;
    int32_t spp;
    int32_t sample_offset;
    int32_t part;             // scene of a group
    uint64_t seed;
    const DevMaterial* mats;
    double* sum;
    double* sumsq;
    uint32_t* count;
    uint32_t tlas_root;       // the scene's top-level tree
    int32_t light_base;       // the scene's lights: [light_base, light_base + light_count)
    int32_t light_count;
    float light_max;          // their total power (the light-pick CDF's last value)
};

// One scene of a group (omv_scene_create_group) within the group's arrays:
// its top-level tree, lights (a light-pick CDF of their own) and materials.
// A single scene is a group of one.
struct ScenePart {
    uint32_t tlas_root = 0xFFFFFFFFu;
    int32_t light_base = 0, light_count = 0;
    float light_max = 0.0f;
    int32_t mat_base = 0, mat_count = 0;  // without the shared missing material
};

struct SceneHost {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    DevScene dev{};
    std::vector<void*> allocs;
    uint32_t* tlas_items = nullptr;
    int num_meshes = 0;
    int num_instances = 0;
    int num_materials = 0;  // including the missing material
    int num_lights = 0;
    int num_textures = 0;
    int64_t num_triangles = 0;
    int64_t blas_nodes = 0;
    int64_t tlas_nodes = 0;
    int64_t device_bytes = 0;
    double build_ms = 0.0;
    std::vector<uint32_t> mesh_face_prefix;  // global primitive id base per mesh
    std::vector<uint32_t> mesh_vert_count;   // vertices per mesh (0: invalid mesh)
    bool fc_density_ready = false;           // triangle density extremes (the md validation subject)
    float fc_density_min = 0.0f, fc_density_max = 0.0f;
    uint32_t* d_face_prefix = nullptr;
    RenderScratch scratch;
    std::vector<DevMaterial> h_mats;         // the scene's materials (host copy)
    DevMaterial* mat_sets = nullptr;         // batch material sets: num_mat_sets x num_materials
    int num_mat_sets = 0;
    DevJob* d_jobs = nullptr;                // batch job table
    size_t jobs_cap = 0;
    cudaGraphExec_t batch_graph = nullptr;   // captured batch render, replayed for an identical job list
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;  // order `stream` after / before a caller's default stream
    std::vector<unsigned char> batch_key;    // what batch_graph was captured for
    int64_t batch_wave_paths = 0;            // autotuned wave size for batches (0: automatic)
    int batch_shade_threads = 0;             // autotuned threads per shading block for batches (0: 256)
    std::vector<ScenePart> parts;            // the scenes of a group (one for a single scene)

    ~SceneHost();
    void* alloc(size_t bytes);
    template <typename T>
    T* upload(const std::vector<T>& v)
    {
        T* p = static_cast<T*>(alloc(sizeof(T) * (v.empty() ? 1 : v.size())));
        if (!v.empty()) OMV_CUDA(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, stream));
        return p;
    }
};

// `parts` (optional): the scenes a merged description holds (instances of
// scene p have inst_part[i] == p; light and material ranges per scene)
SceneHost* scene_create(const omv_scene_desc& desc, int device, const std::vector<int>* inst_part = nullptr,
                        const std::vector<ScenePart>* parts = nullptr);
// several scenes in one handle: one device copy of all geometry, one
// top-level tree per scene; batch jobs pick their scene
SceneHost* scene_create_group(int num, const omv_scene_desc* descs, int device);

void render_frame(SceneHost& s, const omv_camera& cam, const omv_params& p, double* d_sum, double* d_sumsq,
                  uint32_t* d_count, cudaStream_t st, omv_stats* stats);
DevMaterial material_from_desc(const omv_material_desc& md, int num_textures);
DevMaterial missing_material();
// material sets for batch jobs: num_sets x (scene materials without the missing one)
void set_material_sets(SceneHost& s, int num_sets, const omv_material_desc* descs);
// all jobs through one wave pipeline (optionally captured once as a CUDA graph
// and replayed for an identical job list)
void render_batch(SceneHost& s, int num_jobs, const omv_job* jobs, const omv_params& p, cudaStream_t st,
                  omv_stats* stats, bool use_graph);
// times candidate wave sizes on the job list and keeps the fastest for batches
void autotune_batch(SceneHost& s, int num_jobs, const omv_job* jobs, const omv_params& p, cudaStream_t st,
                    int64_t* chosen, int32_t* chosen_threads);

// builds the environment's alias table (the MIS estimator) if not yet built
void ensure_env_sampler(SceneHost& s);
// replaces the scene's own materials (same count, same alpha-mask status)
void set_scene_materials(SceneHost& s, int num, const omv_material_desc* descs);
// path-replay gradient of an image loss with respect to the material parameters
void adjoint_frame(SceneHost& s, const omv_camera& cam, const omv_params& p, const float* d_adjoint, float* d_grad,
                   cudaStream_t st, int part = 0, const DevMaterial* mats = nullptr);
// the adjoint of every job of a list (each job's scene, material set, camera and samples)
void adjoint_batch(SceneHost& s, int n, const omv_adjoint_job* jobs, const omv_params& p, cudaStream_t st);

// render_frame on the fixed scratch array; makes no device allocation
void render_frame_static(SceneHost& s, const omv_camera& cam, const omv_params& p, double* d_sum, double* d_sumsq,
                         uint32_t* d_count, cudaStream_t st);
// largest wave of render_frame_static for these vertex-slot counts
int64_t static_wave_limit(int light_slots, int shadow_slots);
void render_ids(SceneHost& s, const omv_camera& cam, const float* d_jitter, uint64_t seed, omv_hit* d_hits,
                uint32_t* d_gprim, cudaStream_t st);
void trace_rays(SceneHost& s, int64_t n, const float* d_rays, omv_hit* d_hits, cudaStream_t st);
void env_radiance(SceneHost& s, int64_t n, const float* d_dirs, float* d_rgb, cudaStream_t st);

// kernel-level hooks (no scene)
// false-colour validation pass and light-box views (fc.cu)
int fc_subject_from_name(const char* name);
void render_fc(SceneHost& s, const omv_camera& cam, int subject, const float* uniforms, uint64_t seed,
               const uint32_t* palette, int palette_size, float* rgba, uint32_t* args, omv_hit* hits);
void scene_bounds(SceneHost& s, float lo[3], float hi[3]);
void lightbox_cameras(const float lo[3], const float hi[3], int width, int height, omv_camera out[8]);
// BitmapTexture::texture on the device for one image (d_table: 16 bytes of scratch)
void hook_texture_sample(int w, int h, const uint8_t* d_rgba, int64_t n, const float* d_uv, float* d_out,
                         void* d_table, cudaStream_t st);

// image development and writers (post.cu)
void develop_film(const double* d_sum, const uint32_t* d_count, int w, int h, float A, float gamma, float* d_linear,
                  float* d_toned, uint8_t* d_rgba8, bool flip, cudaStream_t st);
void tonemap(float* d_rgba, int64_t pixels, float A, float gamma, cudaStream_t st);
void denoise_median(const float* d_in, float* d_out, int w, int h, int half, cudaStream_t st);
void rgba8(const float* d_in, uint8_t* d_out, int w, int h, bool flip, cudaStream_t st);
void save_image(const char* path, const float* rgba, int w, int h);

void hook_eval_direct(int64_t n, const float* d_in, float* d_out, cudaStream_t st);
void hook_sample_indirect(int64_t n, const float* d_in, float* d_out, cudaStream_t st);
void hook_om_fresnel(int64_t n, const float* d_in, float* d_out, cudaStream_t st);
void hook_library_function(int fn, int64_t n, const float* d_in, float* d_out, cudaStream_t st);
void hook_camera_rays(const omv_camera& cam, const float* d_jitter, float* d_rays, cudaStream_t st);

}  // namespace omv
