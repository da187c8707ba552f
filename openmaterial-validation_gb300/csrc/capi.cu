// extern "C" boundary of the render path (declared in include/omv.h).  Every
// entry point converts C++ exceptions into an omv_status and records the
// message for omv_last_error(); nothing throws across the boundary.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <new>
#include <string>

#include "../../include/omv.h"
#include "scene.h"

struct omv_scene {
    std::unique_ptr<omv::SceneHost> h;
    double* sum = nullptr;
    double* sumsq = nullptr;
    uint32_t* count = nullptr;
    float4* image = nullptr;
    int64_t film_pixels = 0;
    ~omv_scene()
    {
        if (h) cudaSetDevice(h->device);
        cudaFree(sum);
        cudaFree(sumsq);
        cudaFree(count);
        cudaFree(image);
    }
};

namespace {

thread_local std::string g_last_error;
std::atomic<omv_log_fn> g_log_fn{nullptr};
std::atomic<void*> g_log_user{nullptr};

omv_status fail(omv_status code, const char* msg)
{
    g_last_error = msg ? msg : "unknown error";
    if (const omv_log_fn fn = g_log_fn.load()) fn(g_log_user.load(), code, g_last_error.c_str());
    return code;
}

template <typename F>
omv_status guarded(F&& f)
{
    try {
        f();
        g_last_error.clear();
        return OMV_OK;
    } catch (const omv::ArgError& e) {
        return fail(OMV_ERR_INVALID_ARGUMENT, e.what());
    } catch (const omv::DeviceOutOfMemory& e) {
        return fail(OMV_ERR_OUT_OF_MEMORY, e.what());
    } catch (const omv::CudaError& e) {
        return fail(OMV_ERR_CUDA, e.what());
    } catch (const std::bad_alloc&) {
        return fail(OMV_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        std::string m = e.what();
        if (m.find("no valid instance") != std::string::npos) return fail(OMV_ERR_EMPTY_SCENE, e.what());
        if (m.find("no CUDA device") != std::string::npos) return fail(OMV_ERR_NO_DEVICE, e.what());
        if (m.find("out of memory") != std::string::npos) return fail(OMV_ERR_OUT_OF_MEMORY, e.what());
        return fail(OMV_ERR_INTERNAL, e.what());
    } catch (...) {
        return fail(OMV_ERR_INTERNAL, "unknown exception");
    }
}

// PinholeCamera::stop (PinholeCamera.cpp:70-78): rgb / count, alpha 1
__global__ void k_resolve(int64_t n, const double* sum, const uint32_t* count, float4* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double c = (double)count[i];
    const double s = c < 0.5 ? 1.0 : 1.0 / c;
    out[i] = make_float4((float)(sum[3 * i] * s), (float)(sum[3 * i + 1] * s), (float)(sum[3 * i + 2] * s), 1.0f);
}

struct DevTmp {
    void* p = nullptr;
    explicit DevTmp(size_t bytes) { OMV_CUDA(cudaMalloc(&p, bytes ? bytes : 16)); }
    ~DevTmp() { cudaFree(p); }
    template <typename T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

void check_scene(const omv_scene* s)
{
    if (!s || !s->h) throw omv::ArgError("scene handle is NULL");
    OMV_CUDA(cudaSetDevice(s->h->device));
}

void check_camera(const omv_camera* c)
{
    if (!c) throw omv::ArgError("camera is NULL");
    if (c->width <= 0 || c->height <= 0) throw omv::ArgError("camera resolution must be positive");
    if ((int64_t)c->width * c->height > (int64_t)1 << 30) throw omv::ArgError("camera resolution too large");
}

}  // namespace

extern "C" {

void omv_params_default(omv_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->camera_bounces = 10;
    p->light_bounces = 10;
    p->max_path_length = 8;
    p->samples_per_pixel = 20;
    p->light_distance_attenuation = 1;
    p->light_scale = 100.0f;
    p->light_min_distance = 0.01f;
    p->ray_cut_value = 0.002f;
    p->seed = 0;
    p->estimator = OMV_ESTIMATOR_REFERENCE;
}

const char* omv_last_error(void) { return g_last_error.c_str(); }

omv_status omv_set_log_callback(omv_log_fn fn, void* user)
{
    g_log_user.store(user);
    g_log_fn.store(fn);
    return OMV_OK;
}

const char* omv_version(void) { return "omv-gb300 0.1 (sm_103a)"; }

int32_t omv_struct_sizes(int64_t* out, int32_t n)
{
    const int64_t sizes[] = {(int64_t)sizeof(omv_mesh_desc),  (int64_t)sizeof(omv_instance_desc),
                             (int64_t)sizeof(omv_material_desc), (int64_t)sizeof(omv_light_desc),
                             (int64_t)sizeof(omv_hdri_desc),  (int64_t)sizeof(omv_scene_desc),
                             (int64_t)sizeof(omv_scene_info), (int64_t)sizeof(omv_camera),
                             (int64_t)sizeof(omv_params),     (int64_t)sizeof(omv_stats),
                             (int64_t)sizeof(omv_hit),        (int64_t)sizeof(omv_job),
                             (int64_t)sizeof(omv_texture_desc), (int64_t)sizeof(omv_texture_ref),
                             (int64_t)sizeof(omv_adjoint_job)};
    const int32_t m = (int32_t)(sizeof(sizes) / sizeof(sizes[0]));
    if (!out) return m;
    const int32_t k = std::min(n, m);
    for (int32_t i = 0; i < k; ++i) out[i] = sizes[i];
    return k;
}

omv_status omv_scene_create(const omv_scene_desc* desc, int32_t device, omv_scene** out)
{
    return guarded([&] {
        if (!desc || !out) throw omv::ArgError("desc and out must not be NULL");
        *out = nullptr;
        std::unique_ptr<omv_scene> s(new omv_scene);
        s->h.reset(omv::scene_create(*desc, device));
        *out = s.release();
    });
}

omv_status omv_scene_destroy(omv_scene* scene)
{
    return guarded([&] { delete scene; });
}

omv_status omv_scene_get_info(const omv_scene* scene, omv_scene_info* info)
{
    return guarded([&] {
        if (!scene || !scene->h || !info) throw omv::ArgError("NULL argument");
        info->num_triangles = scene->h->num_triangles;
        info->num_blas_nodes = scene->h->blas_nodes;
        info->num_tlas_nodes = scene->h->tlas_nodes;
        info->device_bytes = scene->h->device_bytes;
        info->build_ms = scene->h->build_ms;
    });
}

omv_status omv_render_device(omv_scene* scene, const omv_camera* camera, const omv_params* params, double* d_sum_rgb,
                             double* d_sumsq_rgb, uint32_t* d_count, void* stream, omv_stats* stats)
{
    return guarded([&] {
        check_scene(scene);
        check_camera(camera);
        if (!params || !d_sum_rgb || !d_count) throw omv::ArgError("params, d_sum_rgb and d_count are required");
        if (params->accumulate_variance && !d_sumsq_rgb) throw omv::ArgError("accumulate_variance needs d_sumsq_rgb");
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
        omv::render_frame(*scene->h, *camera, *params, d_sum_rgb, params->accumulate_variance ? d_sumsq_rgb : nullptr,
                          d_count, st, stats);
    });
}

omv_status omv_render_device_static(omv_scene* scene, const omv_camera* camera, const omv_params* params,
                                    double* d_sum_rgb, double* d_sumsq_rgb, uint32_t* d_count, void* stream)
{
    return guarded([&] {
        check_scene(scene);
        check_camera(camera);
        if (!params || !d_sum_rgb || !d_count) throw omv::ArgError("params, d_sum_rgb and d_count are required");
        if (params->accumulate_variance && !d_sumsq_rgb) throw omv::ArgError("accumulate_variance needs d_sumsq_rgb");
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
        omv::render_frame_static(*scene->h, *camera, *params, d_sum_rgb,
                                 params->accumulate_variance ? d_sumsq_rgb : nullptr, d_count, st);
    });
}

omv_status omv_batch_set_materials(omv_scene* scene, int32_t num_sets, const omv_material_desc* sets)
{
    return guarded([&] {
        check_scene(scene);
        omv::set_material_sets(*scene->h, num_sets, sets);
    });
}

omv_status omv_render_batch(omv_scene* scene, int32_t num_jobs, const omv_job* jobs, const omv_params* params,
                            void* stream, int32_t flags, omv_stats* stats)
{
    return guarded([&] {
        check_scene(scene);
        if (!params) throw omv::ArgError("params is NULL");
        if (params->time_kernels && (flags & OMV_BATCH_GRAPH))
            throw omv::ArgError("time_kernels cannot be combined with OMV_BATCH_GRAPH");
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
        omv::render_batch(*scene->h, num_jobs, jobs, *params, st, stats, (flags & OMV_BATCH_GRAPH) != 0);
    });
}

omv_status omv_batch_autotune(omv_scene* scene, int32_t num_jobs, const omv_job* jobs, const omv_params* params,
                              void* stream, int64_t* chosen_wave_paths, int32_t* chosen_block_threads)
{
    return guarded([&] {
        check_scene(scene);
        if (!params) throw omv::ArgError("params is NULL");
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
        omv::autotune_batch(*scene->h, num_jobs, jobs, *params, st, chosen_wave_paths, chosen_block_threads);
    });
}

omv_status omv_scene_set_materials(omv_scene* scene, int32_t num_materials, const omv_material_desc* materials)
{
    return guarded([&] {
        check_scene(scene);
        omv::set_scene_materials(*scene->h, num_materials, materials);
    });
}

omv_status omv_scene_create_group(int32_t num_scenes, const omv_scene_desc* descs, int32_t device, omv_scene** out)
{
    return guarded([&] {
        if (!descs || !out) throw omv::ArgError("descs and out must not be NULL");
        if (num_scenes <= 0) throw omv::ArgError("a group needs at least one scene");
        *out = nullptr;
        std::unique_ptr<omv_scene> s(new omv_scene);
        s->h.reset(omv::scene_create_group(num_scenes, descs, device));
        *out = s.release();
    });
}

omv_status omv_adjoint_batch(omv_scene* scene, int32_t num_jobs, const omv_adjoint_job* jobs,
                             const omv_params* params, void* stream)
{
    return guarded([&] {
        check_scene(scene);
        if (!params) throw omv::ArgError("params is NULL");
        if (num_jobs < 0 || (num_jobs > 0 && !jobs)) throw omv::ArgError("invalid adjoint job list");
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
        omv::adjoint_batch(*scene->h, num_jobs, jobs, *params, st);
    });
}

omv_status omv_adjoint(omv_scene* scene, const omv_camera* camera, const omv_params* params,
                       const float* d_adjoint_rgb, float* d_grad, void* stream)
{
    return guarded([&] {
        check_scene(scene);
        check_camera(camera);
        if (!params) throw omv::ArgError("params is NULL");
        cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
        omv::adjoint_frame(*scene->h, *camera, *params, d_adjoint_rgb, d_grad, st);
    });
}

omv_status omv_render(omv_scene* scene, const omv_camera* camera, const omv_params* params, float* image_rgba,
                      double* sum_rgb, double* sumsq_rgb, uint32_t* count, omv_stats* stats)
{
    return guarded([&] {
        check_scene(scene);
        check_camera(camera);
        if (!params) throw omv::ArgError("params is NULL");
        if (sumsq_rgb && !params->accumulate_variance)
            throw omv::ArgError("sumsq_rgb requested without accumulate_variance");
        const int64_t npix = (int64_t)camera->width * camera->height;
        omv_scene& s = *scene;
        cudaStream_t st = s.h->stream;
        if (s.film_pixels < npix) {
            OMV_CUDA(cudaStreamSynchronize(st));
            cudaFree(s.sum);
            cudaFree(s.sumsq);
            cudaFree(s.count);
            cudaFree(s.image);
            s.sum = s.sumsq = nullptr;
            s.count = nullptr;
            s.image = nullptr;
            s.film_pixels = 0;
            OMV_CUDA(cudaMalloc(&s.sum, sizeof(double) * 3 * npix));
            OMV_CUDA(cudaMalloc(&s.sumsq, sizeof(double) * 3 * npix));
            OMV_CUDA(cudaMalloc(&s.count, sizeof(uint32_t) * npix));
            OMV_CUDA(cudaMalloc(&s.image, sizeof(float4) * npix));
            s.film_pixels = npix;
        }
        OMV_CUDA(cudaMemsetAsync(s.sum, 0, sizeof(double) * 3 * npix, st));
        OMV_CUDA(cudaMemsetAsync(s.count, 0, sizeof(uint32_t) * npix, st));
        if (params->accumulate_variance) OMV_CUDA(cudaMemsetAsync(s.sumsq, 0, sizeof(double) * 3 * npix, st));
        omv::render_frame(*s.h, *camera, *params, s.sum, params->accumulate_variance ? s.sumsq : nullptr, s.count, st,
                          stats);
        if (image_rgba) {
            k_resolve<<<(int)((npix + 255) / 256), 256, 0, st>>>(npix, s.sum, s.count, s.image);
            OMV_CUDA(cudaGetLastError());
            OMV_CUDA(cudaMemcpyAsync(image_rgba, s.image, sizeof(float4) * npix, cudaMemcpyDeviceToHost, st));
        }
        if (sum_rgb) OMV_CUDA(cudaMemcpyAsync(sum_rgb, s.sum, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, st));
        if (sumsq_rgb)
            OMV_CUDA(cudaMemcpyAsync(sumsq_rgb, s.sumsq, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, st));
        if (count) OMV_CUDA(cudaMemcpyAsync(count, s.count, sizeof(uint32_t) * npix, cudaMemcpyDeviceToHost, st));
        OMV_CUDA(cudaStreamSynchronize(st));
    });
}

omv_status omv_trace_rays(omv_scene* scene, int64_t n, const float* rays, omv_hit* hits)
{
    return guarded([&] {
        check_scene(scene);
        if (n < 0 || (n > 0 && (!rays || !hits))) throw omv::ArgError("invalid ray buffers");
        if (n == 0) return;
        cudaStream_t st = scene->h->stream;
        DevTmp dr(sizeof(float) * 8 * n), dh(sizeof(omv_hit) * n);
        OMV_CUDA(cudaMemcpyAsync(dr.p, rays, sizeof(float) * 8 * n, cudaMemcpyHostToDevice, st));
        omv::trace_rays(*scene->h, n, dr.as<float>(), dh.as<omv_hit>(), st);
        OMV_CUDA(cudaMemcpyAsync(hits, dh.p, sizeof(omv_hit) * n, cudaMemcpyDeviceToHost, st));
        OMV_CUDA(cudaStreamSynchronize(st));
    });
}

omv_status omv_render_ids(omv_scene* scene, const omv_camera* camera, const float* jitter, uint64_t seed,
                          omv_hit* hits, uint32_t* global_prim)
{
    return guarded([&] {
        check_scene(scene);
        check_camera(camera);
        const int64_t npix = (int64_t)camera->width * camera->height;
        cudaStream_t st = scene->h->stream;
        DevTmp dj(jitter ? sizeof(float) * 2 * npix : 16), dh(sizeof(omv_hit) * npix), dg(sizeof(uint32_t) * npix);
        if (jitter) OMV_CUDA(cudaMemcpyAsync(dj.p, jitter, sizeof(float) * 2 * npix, cudaMemcpyHostToDevice, st));
        omv::render_ids(*scene->h, *camera, jitter ? dj.as<float>() : nullptr, seed, dh.as<omv_hit>(),
                        dg.as<uint32_t>(), st);
        if (hits) OMV_CUDA(cudaMemcpyAsync(hits, dh.p, sizeof(omv_hit) * npix, cudaMemcpyDeviceToHost, st));
        if (global_prim)
            OMV_CUDA(cudaMemcpyAsync(global_prim, dg.p, sizeof(uint32_t) * npix, cudaMemcpyDeviceToHost, st));
        OMV_CUDA(cudaStreamSynchronize(st));
    });
}

omv_status omv_env_radiance(omv_scene* scene, int64_t n, const float* dirs, float* rgb)
{
    return guarded([&] {
        check_scene(scene);
        if (n < 0 || (n > 0 && (!dirs || !rgb))) throw omv::ArgError("invalid buffers");
        if (n == 0) return;
        cudaStream_t st = scene->h->stream;
        DevTmp dd(sizeof(float) * 3 * n), dr(sizeof(float) * 3 * n);
        OMV_CUDA(cudaMemcpyAsync(dd.p, dirs, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
        omv::env_radiance(*scene->h, n, dd.as<float>(), dr.as<float>(), st);
        OMV_CUDA(cudaMemcpyAsync(rgb, dr.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
        OMV_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C++" {  // a template inside the C block
template <typename Fn>
static omv_status run_hook(int64_t n, const float* in, float* out, int win, int wout, Fn fn)
{
    return guarded([&] {
        if (n < 0 || (n > 0 && (!in || !out))) throw omv::ArgError("invalid buffers");
        if (n == 0) return;
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw omv::CudaError("no CUDA device available");
        DevTmp di(sizeof(float) * win * n), dout(sizeof(float) * wout * n);
        OMV_CUDA(cudaMemcpy(di.p, in, sizeof(float) * win * n, cudaMemcpyHostToDevice));
        fn(n, di.as<float>(), dout.as<float>(), nullptr);
        OMV_CUDA(cudaMemcpy(out, dout.p, sizeof(float) * wout * n, cudaMemcpyDeviceToHost));
    });
}
}

omv_status omv_brdf_eval_direct(int64_t n, const float* in, float* out)
{
    return run_hook(n, in, out, 17, 3, omv::hook_eval_direct);
}

omv_status omv_brdf_sample_indirect(int64_t n, const float* in, float* out)
{
    return run_hook(n, in, out, 24, 6, omv::hook_sample_indirect);
}

omv_status omv_om_fresnel(int64_t n, const float* in, float* out)
{
    return run_hook(n, in, out, 7, 3, omv::hook_om_fresnel);
}

omv_status omv_library_function(int32_t function, int64_t n, const float* in, float* out)
{
    if (function < OMV_FN_SIN || function > OMV_FN_POW_M2) return guarded([] { throw omv::ArgError("unknown function"); });
    return run_hook(n, in, out, 1, 1, [function](int64_t m, const float* a, float* b, cudaStream_t st) {
        omv::hook_library_function(function, m, a, b, st);
    });
}

omv_status omv_texture_sample(int32_t width, int32_t height, const uint8_t* rgba, int64_t n, const float* uv,
                              float* out)
{
    return guarded([&] {
        if (width <= 0 || height <= 0 || !rgba) throw omv::ArgError("texture needs a positive size and texels");
        if (n < 0 || (n > 0 && (!uv || !out))) throw omv::ArgError("invalid buffers");
        if (n == 0) return;
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw omv::CudaError("no CUDA device available");
        const size_t tb = (size_t)width * height * 4;
        DevTmp dt(tb), du(sizeof(float) * 2 * n), dout(sizeof(float) * 4 * n), dtab(64);
        OMV_CUDA(cudaMemcpy(dt.p, rgba, tb, cudaMemcpyHostToDevice));
        OMV_CUDA(cudaMemcpy(du.p, uv, sizeof(float) * 2 * n, cudaMemcpyHostToDevice));
        omv::hook_texture_sample(width, height, dt.as<uint8_t>(), n, du.as<float>(), dout.as<float>(), dtab.p, nullptr);
        OMV_CUDA(cudaMemcpy(out, dout.p, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost));
    });
}

omv_status omv_camera_rays(const omv_camera* camera, const float* jitter, float* rays)
{
    return guarded([&] {
        check_camera(camera);
        if (!jitter || !rays) throw omv::ArgError("invalid buffers");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw omv::CudaError("no CUDA device available");
        const int64_t npix = (int64_t)camera->width * camera->height;
        DevTmp dj(sizeof(float) * 2 * npix), dr(sizeof(float) * 6 * npix);
        OMV_CUDA(cudaMemcpy(dj.p, jitter, sizeof(float) * 2 * npix, cudaMemcpyHostToDevice));
        omv::hook_camera_rays(*camera, dj.as<float>(), dr.as<float>(), nullptr);
        OMV_CUDA(cudaMemcpy(rays, dr.p, sizeof(float) * 6 * npix, cudaMemcpyDeviceToHost));
    });
}

/* ------------------------------------------------- false-colour validation */

int32_t omv_fc_subject_from_name(const char* name) { return omv::fc_subject_from_name(name); }

omv_status omv_render_fc(omv_scene* scene, const omv_camera* camera, int32_t subject, const float* uniforms,
                         uint64_t seed, const uint32_t* palette, int32_t palette_size, float* image_rgba,
                         uint32_t* args, omv_hit* hits)
{
    return guarded([&] {
        check_scene(scene);
        check_camera(camera);
        omv::render_fc(*scene->h, *camera, subject, uniforms, seed, palette, palette_size, image_rgba, args, hits);
    });
}

omv_status omv_scene_bounds(omv_scene* scene, float lo[3], float hi[3])
{
    return guarded([&] {
        check_scene(scene);
        if (!lo || !hi) throw omv::ArgError("lo and hi are required");
        omv::scene_bounds(*scene->h, lo, hi);
    });
}

omv_status omv_lightbox_cameras(const float lo[3], const float hi[3], int32_t width, int32_t height,
                                omv_camera cameras[8])
{
    return guarded([&] {
        if (!lo || !hi || !cameras) throw omv::ArgError("lo, hi and cameras are required");
        omv::lightbox_cameras(lo, hi, width, height, cameras);
    });
}

/* ------------------------------------------------------- image development */

omv_status omv_develop(const double* d_sum_rgb, const uint32_t* d_count, int32_t width, int32_t height, float A,
                       float gamma, float* d_linear_rgba, float* d_tonemapped_rgba, uint8_t* d_rgba8, int32_t flip,
                       void* stream)
{
    return guarded([&] {
        omv::develop_film(d_sum_rgb, d_count, width, height, A, gamma, d_linear_rgba, d_tonemapped_rgba, d_rgba8,
                          flip != 0, static_cast<cudaStream_t>(stream));
    });
}

omv_status omv_tonemap(float* d_rgba, int64_t pixels, float A, float gamma, void* stream)
{
    return guarded([&] { omv::tonemap(d_rgba, pixels, A, gamma, static_cast<cudaStream_t>(stream)); });
}

omv_status omv_denoise_median(const float* d_in_rgba, float* d_out_rgba, int32_t width, int32_t height,
                              int32_t half_size, void* stream)
{
    return guarded([&] {
        omv::denoise_median(d_in_rgba, d_out_rgba, width, height, half_size, static_cast<cudaStream_t>(stream));
    });
}

omv_status omv_rgba8(const float* d_rgba, uint8_t* d_out, int32_t width, int32_t height, int32_t flip, void* stream)
{
    return guarded([&] { omv::rgba8(d_rgba, d_out, width, height, flip != 0, static_cast<cudaStream_t>(stream)); });
}

omv_status omv_save_image(const char* path, const float* rgba, int32_t width, int32_t height)
{
    return guarded([&] { omv::save_image(path, rgba, width, height); });
}

}  // extern "C"
