// False-colour validation pass and light-box views (the FC_VALIDATION build's
// -F and -V options, main.cpp:261-270 and 434-458).
//
//   k_fc            one thread per pixel: jittered primary ray, alpha-mask-aware
//                   closest hit, the subject's argument from the hit surface
//                   point and material, GenericFCSubject::paint
//   k_density_range RenderMesh::getMinMaxDensity over every instance
//                   (RenderMesh.cpp:277-297), one block per instance
//   k_bounds        AssetGeometry::getBBox of the flattened scene, one block
//                   per instance
//
// The argument bits follow GenericFCArgument (FCSubject.h:41-86): an unsigned
// enumerator, a float clamped to [0, 1], four name bytes or a 0/1 flag.
// Float work is in the reference's operation order (this translation unit is
// compiled without FMA contraction); only logf / powf round differently.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "scene.h"
#include "shade.cuh"

namespace omv {
namespace {

constexpr int kFcThreads = 128;

__device__ __forceinline__ V3 xform_point(const float* m, float4 p)
{
    return v3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}

__device__ __forceinline__ float length3(V3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

// non-negative floats order like their bit patterns
__device__ __forceinline__ void atomic_min_pos(float* p, float v) { atomicMin((int*)p, __float_as_int(v)); }
__device__ __forceinline__ void atomic_max_pos(float* p, float v) { atomicMax((int*)p, __float_as_int(v)); }
__device__ __forceinline__ void atomic_min_f(float* p, float v)
{
    if (v >= 0.0f)
        atomicMin((int*)p, __float_as_int(v));
    else
        atomicMax((unsigned int*)p, __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* p, float v)
{
    if (v >= 0.0f)
        atomicMax((int*)p, __float_as_int(v));
    else
        atomicMin((unsigned int*)p, __float_as_uint(v));
}

__device__ __forceinline__ void face_world(const DevScene& S, const DevInstance* I, uint32_t face, V3& a, V3& b,
                                           V3& c)
{
    float m[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) m[k] = __ldg(&I->xf[k]);
    const uint32_t vb = __ldg(&I->vert_base);
    const uint32_t* F = S.faces + 3 * (size_t)(__ldg(&I->face_base) + face);
    a = xform_point(m, __ldg(S.verts + 3 * (size_t)(vb + __ldg(F))));
    b = xform_point(m, __ldg(S.verts + 3 * (size_t)(vb + __ldg(F + 1))));
    c = xform_point(m, __ldg(S.verts + 3 * (size_t)(vb + __ldg(F + 2))));
}

// out[0] = min density, out[1] = max density (densities are positive)
__global__ void k_density_range(DevScene S, const uint32_t* face_count, float* out)
{
    const DevInstance* I = S.insts + blockIdx.x;
    if (!__ldg(&I->valid)) return;
    const uint32_t n = face_count[__ldg(&I->mesh)];
    float lo = INFINITY, hi = 0.0f;
    for (uint32_t f = threadIdx.x; f < n; f += blockDim.x) {
        V3 a, b, c;
        face_world(S, I, f, a, b, c);
        const float area = length3(cross(b - a, c - a)) / 2.0f;
        if (area > kEps) {
            const float d = 1.0f / (0.0f + area);
            lo = fminf(lo, d);
            hi = fmaxf(hi, d);
        }
    }
    if (lo <= hi) {
        atomic_min_pos(out, lo);
        atomic_max_pos(out + 1, hi);
    }
}

__global__ void k_bounds(DevScene S, const uint32_t* vert_count, float* out)
{
    const DevInstance* I = S.insts + blockIdx.x;
    if (!__ldg(&I->valid)) return;
    float m[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) m[k] = __ldg(&I->xf[k]);
    const uint32_t n = vert_count[__ldg(&I->mesh)], vb = __ldg(&I->vert_base);
    V3 lo = v3(INFINITY, INFINITY, INFINITY), hi = v3(-INFINITY, -INFINITY, -INFINITY);
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const V3 p = xform_point(m, __ldg(S.verts + 3 * (size_t)(vb + k)));
        lo = v3(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
        hi = v3(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
    }
    if (n > threadIdx.x) {
        atomic_min_f(out + 0, lo.x);
        atomic_min_f(out + 1, lo.y);
        atomic_min_f(out + 2, lo.z);
        atomic_max_f(out + 3, hi.x);
        atomic_max_f(out + 4, hi.y);
        atomic_max_f(out + 5, hi.z);
    }
}

struct FcArgs {
    int subject;
    const float4* uniforms;  // per pixel, or null
    uint64_t seed;
    const uint32_t* palette;
    int palette_size;
    float dmin, dmax;
    const uint32_t* face_prefix;
    float4* rgba;
    uint32_t* args;
    omv_hit* hits;
};

__device__ __forceinline__ V3 hashed(const uint32_t* palette, int size, uint32_t id)
{
    const uint32_t n = (palette && id < (uint32_t)size) ? __ldg(palette + id) : 0u;
    return v3((float)((n >> 16) & 0xFFu) / 255.0f, (float)((n >> 8) & 0xFFu) / 255.0f, (float)(n & 0xFFu) / 255.0f);
}

__device__ __forceinline__ V3 lerp_paint(float t, V3 upper)
{
    return v3(lerpf(1.0f, upper.x, t), lerpf(1.0f, upper.y, t), lerpf(1.0f, upper.z, t));
}

__device__ __forceinline__ uint32_t float_bits(float f) { return __float_as_uint(f); }

__global__ void __launch_bounds__(kFcThreads) k_fc(DevScene S, const uint32_t* items, omv_camera cam, FcArgs a)
{
    __shared__ uint2 sstack[kStackShared * kFcThreads];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kFcThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    const int npix = cam.width * cam.height;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float4 u;
    if (a.uniforms) {
        u = a.uniforms[p];
    } else {
        const Rng4 r = rng4(a.seed, (uint32_t)p, 0u, 0u, kStreamCamera);
        u = make_float4(r.u[0], r.u[1], r.u[2], r.u[3]);
    }
    V3 O, R;
    camera_ray(cam, p % cam.width, p / cam.width, u.x, u.y, O, R);
    const V3 so = shifted_origin(O, R, 1.0f);
    float tnear = 0.0f;
    RayHit h;
    V3 col = v3(0.0f, 0.0f, 0.0f);
    uint32_t arg = 0;
    const bool hit = scene_intersect(S, items, so, R, tnear, kFltMax, h, st, tc);
    if (hit) {
        const DevMaterial& M = S.mats[__ldg(&S.insts[h.inst].material)];
        const Surf sp = surface_point(S, h.inst, h.prim, h.u, h.v, true, &M);  // includes modifyFrame
        const DevInstance* I = S.insts + h.inst;
        const uint32_t mesh = __ldg(&I->mesh);
        V3 inV = R;
        if (M.type == kMatMissing)  // getRayAndBrdf: hemisphere direction, then getBrdf(-out, -in)
            inV = -to_basis(sp.tan, sp.bin, sp.nrm, uniform_hemisphere(u.z, u.w));
        switch (a.subject) {
        case OMV_FC_PID:
            arg = __ldg(a.face_prefix + mesh) + h.prim;
            col = hashed(a.palette, a.palette_size, arg);
            break;
        case OMV_FC_GID:
            arg = mesh;
            col = hashed(a.palette, a.palette_size, arg);
            break;
        case OMV_FC_MID:
            if (M.type == kMatMissing) {
                arg = 0xFFFFFFFFu;
                col = v3(1000.0f, 0.0f, 1000.0f);
            } else {
                arg = sp.mat;
                const V3 c = hashed(a.palette, a.palette_size, arg);
                col = v3(0.0f, c.y, c.z);
            }
            break;
        case OMV_FC_MMP:
        case OMV_FC_RMP: {
            float f = 0.0f;
            if (M.type == kMatPbr) {  // getTextureOccMetRoughValues (PhysicallyBasedMaterial.cpp:54-90)
                const PbrParams P = pbr_params(S, M, sp);
                f = clamp01(a.subject == OMV_FC_MMP ? P.omr_metal : P.omr_rough);
            }
            arg = float_bits(f);
            col = lerp_paint(f, a.subject == OMV_FC_MMP ? v3(0.0f, 0.0f, 1.0f) : v3(0.0f, 1.0f, 0.0f));
            break;
        }
        case OMV_FC_MD:
        case OMV_FC_SG: {
            // RenderMesh.cpp:197-207 (pointwise gradient), BDPTRenderer.cpp:68-72
            V3 A, B, C;
            face_world(S, I, h.prim, A, B, C);
            V3 tfn = cross(B - A, C - A);
            float f;
            if (a.subject == OMV_FC_MD) {
                const float ref = 1.0f / (0.0f + length3(tfn) / 2.0f);
                f = clamp01(1.0f - logf(a.dmax / clampf(ref, a.dmin, a.dmax)) / logf(a.dmax / a.dmin));
                f = clamp01(f);
                col = lerp_paint(f, v3(1.0f, 0.0f, 0.0f));
            } else {
                tfn = normalize(tfn);
                float nm[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) nm[k] = __ldg(&I->nrm[k]);
                const uint32_t vb = __ldg(&I->vert_base);
                const uint32_t* F = S.faces + 3 * (size_t)(__ldg(&I->face_base) + h.prim);
                float ag = 0.0f;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float4* V = S.verts + 3 * (size_t)(vb + __ldg(F + k));
                    const float4 w0 = __ldg(V), w1 = __ldg(V + 1);
                    const V3 tvn = normalize_if_needed(m33(nm, v3(w0.w, w1.x, w1.y)));
                    ag = ag + sqrtf((1.0f - clampf(dot(tvn, tfn), -1.0f, 1.0f)) / 2.0f);
                }
                f = clamp01(powf(clampf(ag / 3.0f, 1e-6f, 1.0f), 0.286f));
                col = v3(1.0f - f, 1.0f - f, 1.0f - f);
            }
            arg = float_bits(f);
            break;
        }
        case OMV_FC_MN:
            if (M.type == kMatPbr) {
                arg = 'p' | ('b' << 8) | ('r' << 16);
                col = v3(0.0f, 0.0f, 1.0f);
            } else if (M.type == kMatOm) {
                arg = 'o' | ('m' << 8);
                col = v3(0.0f, 1.0f, 0.0f);
            } else {
                arg = 'm' | ('m' << 8);
                col = v3(1000.0f, 0.0f, 1000.0f);
            }
            break;
        case OMV_FC_IN: {
            const bool inv = dot(inV, face_normal(S, sp)) > 0.0f;
            arg = inv ? 1u : 0u;
            col = v3((float)inv, 1.0f - (float)inv, 0.0f);
            break;
        }
        default:
            break;
        }
    }
    if (a.rgba) a.rgba[p] = make_float4(col.x, col.y, col.z, 1.0f);
    if (a.args) a.args[p] = arg;
    if (a.hits) {
        omv_hit o;
        if (hit) {
            const DevInstance* I = S.insts + h.inst;
            o.inst = h.inst;
            o.geom = __ldg(&I->mesh);
            o.prim = h.prim;
            o.material = __ldg(&I->material);
            o.t = h.t;
            o.u = h.u;
            o.v = h.v;
        } else {
            o.inst = o.geom = o.prim = o.material = kInvalid;
            o.t = o.u = o.v = 0.0f;
        }
        o.pad = 0;
        a.hits[p] = o;
    }
}

struct DevBuf {
    void* p = nullptr;
    explicit DevBuf(size_t bytes) { OMV_CUDA(cudaMalloc(&p, bytes ? bytes : 16)); }
    ~DevBuf() { cudaFree(p); }
    template <typename T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

void ensure_density_range(SceneHost& s)
{
    if (s.fc_density_ready) return;
    DevBuf counts(sizeof(uint32_t) * std::max(1, s.num_meshes)), out(2 * sizeof(float));
    std::vector<uint32_t> fc(std::max(1, s.num_meshes), 0);
    for (int i = 0; i < s.num_meshes; ++i) fc[i] = s.mesh_face_prefix[i + 1] - s.mesh_face_prefix[i];
    const float init[2] = {INFINITY, 0.0f};
    OMV_CUDA(cudaMemcpyAsync(counts.p, fc.data(), sizeof(uint32_t) * fc.size(), cudaMemcpyHostToDevice, s.stream));
    OMV_CUDA(cudaMemcpyAsync(out.p, init, sizeof(init), cudaMemcpyHostToDevice, s.stream));
    if (s.num_instances > 0)
        k_density_range<<<s.num_instances, 256, 0, s.stream>>>(s.dev, counts.as<uint32_t>(), out.as<float>());
    OMV_CUDA(cudaGetLastError());
    float r[2];
    OMV_CUDA(cudaMemcpyAsync(r, out.p, sizeof(r), cudaMemcpyDeviceToHost, s.stream));
    OMV_CUDA(cudaStreamSynchronize(s.stream));
    s.fc_density_min = r[0];
    s.fc_density_max = r[1];
    s.fc_density_ready = true;
}

__global__ void k_texture_hook(DevScene S, int64_t n, const float2* uv, float4* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = tex_sample(S, 0, uv[i].x, uv[i].y);
}

}  // namespace

void hook_texture_sample(int w, int h, const uint8_t* d_rgba, int64_t n, const float* d_uv, float* d_out,
                         void* d_table, cudaStream_t st)
{
    DevScene S{};
    S.texels = reinterpret_cast<const uchar4*>(d_rgba);
    S.textures = static_cast<const DevTexture*>(d_table);
    S.num_textures = 1;
    const DevTexture t{0u, w, h, d_rgba ? 1 : 0};
    OMV_CUDA(cudaMemcpyAsync(d_table, &t, sizeof(t), cudaMemcpyHostToDevice, st));
    if (n > 0)
        k_texture_hook<<<(int)((n + 255) / 256), 256, 0, st>>>(S, n, reinterpret_cast<const float2*>(d_uv),
                                                             reinterpret_cast<float4*>(d_out));
    OMV_CUDA(cudaGetLastError());
}

int fc_subject_from_name(const char* name)
{
    static const char* names[] = {"pid", "gid", "mid", "mmp", "rmp", "md", "sg", "mn", "in"};
    if (!name) return OMV_FC_EMPTY;
    for (int i = 0; i < 9; ++i)
        if (std::strcmp(name, names[i]) == 0) return i + 1;
    return OMV_FC_EMPTY;
}

void render_fc(SceneHost& s, const omv_camera& cam, int subject, const float* uniforms, uint64_t seed,
               const uint32_t* palette, int palette_size, float* rgba, uint32_t* args, omv_hit* hits)
{
    if (subject < OMV_FC_EMPTY || subject > OMV_FC_IN) throw ArgError("unknown false-colour subject");
    if (palette_size < 0 || (palette_size > 0 && !palette)) throw ArgError("palette_size > 0 needs a palette");
    const int64_t npix = (int64_t)cam.width * cam.height;
    FcArgs a{};
    a.subject = subject;
    a.seed = seed;
    a.face_prefix = s.d_face_prefix;
    if (subject == OMV_FC_MD) {
        ensure_density_range(s);
        a.dmin = s.fc_density_min;
        a.dmax = s.fc_density_max;
    }
    DevBuf du(uniforms ? sizeof(float4) * npix : 0), dp(sizeof(uint32_t) * (size_t)std::max(palette_size, 1));
    DevBuf dimg(rgba ? sizeof(float4) * npix : 0), darg(args ? sizeof(uint32_t) * npix : 0),
        dhit(hits ? sizeof(omv_hit) * npix : 0);
    if (uniforms) {
        OMV_CUDA(cudaMemcpyAsync(du.p, uniforms, sizeof(float4) * npix, cudaMemcpyHostToDevice, s.stream));
        a.uniforms = du.as<float4>();
    }
    if (palette_size > 0) {
        OMV_CUDA(cudaMemcpyAsync(dp.p, palette, sizeof(uint32_t) * palette_size, cudaMemcpyHostToDevice, s.stream));
        a.palette = dp.as<uint32_t>();
        a.palette_size = palette_size;
    }
    a.rgba = rgba ? dimg.as<float4>() : nullptr;
    a.args = args ? darg.as<uint32_t>() : nullptr;
    a.hits = hits ? dhit.as<omv_hit>() : nullptr;
    k_fc<<<(int)((npix + kFcThreads - 1) / kFcThreads), kFcThreads, 0, s.stream>>>(s.dev, s.tlas_items, cam, a);
    OMV_CUDA(cudaGetLastError());
    if (rgba) OMV_CUDA(cudaMemcpyAsync(rgba, dimg.p, sizeof(float4) * npix, cudaMemcpyDeviceToHost, s.stream));
    if (args) OMV_CUDA(cudaMemcpyAsync(args, darg.p, sizeof(uint32_t) * npix, cudaMemcpyDeviceToHost, s.stream));
    if (hits) OMV_CUDA(cudaMemcpyAsync(hits, dhit.p, sizeof(omv_hit) * npix, cudaMemcpyDeviceToHost, s.stream));
    OMV_CUDA(cudaStreamSynchronize(s.stream));
}

void scene_bounds(SceneHost& s, float lo[3], float hi[3])
{
    DevBuf counts(sizeof(uint32_t) * std::max(1, s.num_meshes)), out(6 * sizeof(float));
    std::vector<uint32_t> vc(s.mesh_vert_count);
    vc.resize(std::max(1, s.num_meshes), 0);
    const float init[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    OMV_CUDA(cudaMemcpyAsync(counts.p, vc.data(), sizeof(uint32_t) * vc.size(), cudaMemcpyHostToDevice, s.stream));
    OMV_CUDA(cudaMemcpyAsync(out.p, init, sizeof(init), cudaMemcpyHostToDevice, s.stream));
    if (s.num_instances > 0)
        k_bounds<<<s.num_instances, 256, 0, s.stream>>>(s.dev, counts.as<uint32_t>(), out.as<float>());
    OMV_CUDA(cudaGetLastError());
    float r[6];
    OMV_CUDA(cudaMemcpyAsync(r, out.p, sizeof(r), cudaMemcpyDeviceToHost, s.stream));
    OMV_CUDA(cudaStreamSynchronize(s.stream));
    for (int k = 0; k < 3; ++k) {
        lo[k] = r[k];
        hi[k] = r[3 + k];
    }
}

// main.cpp:434-458 and 481-487, in the reference's float operation order
void lightbox_cameras(const float lo[3], const float hi[3], int width, int height, omv_camera out[8])
{
    if (width <= 0 || height <= 0) throw ArgError("camera resolution must be positive");
    for (int k = 0; k < 3; ++k)
        if (!(lo[k] <= hi[k])) throw ArgError("bounding box is empty");
    float C[3];
    for (int k = 0; k < 3; ++k) C[k] = (hi[k] - lo[k]) * 0.5f + lo[k];  // lerp(P0, P1, 0.5)
    const float half_h = 0.5f * (float)height, half_w = 0.5f * (float)width;
    // setYFoV(60): evaluated at run time through the C library's tanf, as the
    // reference does (a compile-time folded tan can differ in the last place)
    volatile float yfov = 60.0f;
    const float arg = 0.5f * yfov * 3.14159265358979323846f / 180.0f;
    const float focus = half_h / tanf(arg);
    for (int i = 0; i < 8; ++i) {
        const float p[3] = {(i & 4) ? hi[0] : lo[0], (i & 2) ? hi[1] : lo[1], (i & 1) ? hi[2] : lo[2]};
        float f[3], pos[3], up[3] = {0.0f, 1.0f, 0.0f}, left[3], up2[3];
        for (int k = 0; k < 3; ++k) f[k] = C[k] - p[k];
        for (int k = 0; k < 3; ++k) {
            const float t = f[k] * -2.0f;  // linearFunction(forward, C, -2)
            pos[k] = t + C[k];
        }
        const float L2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
        float L = std::sqrt(L2);
        if (L != 0.0f) {
            L = 1.0f / L;
            for (float& x : f) x = x * L;
        } else {
            f[0] = 1.0f;
            f[1] = f[2] = 0.0f;
        }
        auto cross = [](const float* a, const float* b, float* r) {
            r[0] = a[1] * b[2] - a[2] * b[1];
            r[1] = a[2] * b[0] - a[0] * b[2];
            r[2] = a[0] * b[1] - a[1] * b[0];
        };
        cross(f, up, left);
        cross(left, f, up2);
        omv_camera& c = out[i];
        std::memset(&c, 0, sizeof(c));
        c.width = width;
        c.height = height;
        for (int k = 0; k < 3; ++k) {
            c.position[k] = pos[k];
            c.rotation[k][0] = left[k];
            c.rotation[k][1] = up2[k];
            c.rotation[k][2] = f[k];
        }
        c.half_width = half_w;
        c.half_height = half_h;
        c.focus = focus;
    }
}

}  // namespace omv
