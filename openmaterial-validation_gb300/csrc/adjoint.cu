// Path-replay adjoint of the BDPT estimator (after Vicini, Speierer, Jakob,
// "Path replay backpropagation", SIGGRAPH 2021): gradients of an image loss
// with respect to the material parameters, given the loss's derivative with
// respect to every pixel (the adjoint image).
//
// One thread replays one path: it regenerates the light and camera subpaths
// from the path's Philox keys (the same random numbers as the forward render),
// traces their extension and shadow rays again, and keeps its few vertices
// in registers and local memory only while the path is processed.  The path's
// estimate is a sum of products of per-vertex factors (BDPTRenderer.cpp:
// 128-302 with weight 1); its derivative is taken with every sampled direction
// held fixed, which for the GGX-sampled branches adds the score d log D / d
// alpha of the half-vector density, so the result is an unbiased estimate of
// the gradient of the expected image (luminance cutoffs are treated as fixed).
// Two division-free backward recursions over the vertices give the factors'
// adjoints.  Gradients are summed per thread, reduced per warp with shuffles,
// per block in shared memory, and added to the output with one atomic per
// block and parameter.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "dual.cuh"
#include "scene.h"
#include "shade.cuh"

namespace omv {
namespace {

constexpr int kAdjThreads = 128;
constexpr int kAdjMaxVerts = 16;      // per subpath
constexpr int kAdjMaxMaterials = 16;  // materials with parameters
constexpr int kSlots = OMV_MATERIAL_PARAMS;

struct AdjArgs {
    DevScene S;
    const uint32_t* items;
    omv_camera cam;
    uint64_t seed;
    int64_t paths;
    int32_t spp, sample_offset;
    int32_t cam_bounces, light_bounces, max_len, atten_mode;
    float light_scale, min_dist, cut;
    const float* adj;  // W*H*3 adjoint image
    float* grad;       // num_user_materials * kSlots
    int32_t num_user_materials;
    uint32_t mat_base;  // first material of the scene (a scene of a group)
};

// derivatives of a vertex weight (or evaluation) with respect to the
// material's local parameters: PBR r,g,b, alpha, metallic; OpenMATERIAL
// n r,g,b, k r,g,b
struct LocalGrad {
    float d[3][6];
};
__device__ __forceinline__ void lg_zero(LocalGrad& g)
{
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int i = 0; i < 6; ++i) g.d[c][i] = 0.0f;
}

// material_sample's weight and its local derivatives (direction fixed)
__device__ __forceinline__ V3 sample_with_grad(const DevScene& S, const DevMaterial& M, const Surf& sp, V3 in, bool inv,
                                               const Rng4& u, V3& out, LocalGrad& g)
{
    lg_zero(g);
    SampleInfo info;
    const V3 w = material_sample(S, M, sp, in, inv, u, out, &info);
    if (M.type == kMatPbr) {
        if (info.kind < 0) return w;
        const PbrDual m = pbr_dual(M.color, M.alpha, M.metal);
        Dual<5> dw[3];
        d_bsdf_evaluate(in, out, info.N, m, info.kind, info.H, info.p, dw);
        const float score = info.kind != 0 ? ggx_log_pdf_dalpha(fabsf(dot(info.N, info.H)), M.alpha) : 0.0f;
        const float wv[3] = {w.x, w.y, w.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
#pragma unroll
            for (int i = 0; i < 5; ++i) g.d[c][i] = dw[c].d[i];
            g.d[c][3] += wv[c] * score;
        }
    } else if (M.type == kMatOm && M.om_valid) {
        const float cth = dot(out, sp.nrm);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const Dual<2> r = d_om_channel(M.om_n[c], M.om_k[c], cth);
            g.d[c][c] = r.d[0];
            g.d[c][3 + c] = r.d[1];
        }
    }
    return w;
}

// material_eval and its local derivatives
__device__ __forceinline__ V3 eval_with_grad(const DevMaterial& M, const Surf& sp, V3 in, V3 out, LocalGrad& g)
{
    lg_zero(g);
    const V3 f = material_eval(M, sp, in, out);
    if (M.type == kMatPbr) {
        V3 N = sp.nrm;
        if (dot(in, N) > 0.0f && M.transmissive) N = -N;
        const PbrDual m = pbr_dual(M.color, M.alpha, M.metal);
        Dual<5> df[3];
        d_bsdf_eval_direct(in, out, N, m, df);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int i = 0; i < 5; ++i) g.d[c][i] = df[c].d[i];
    } else if (M.type == kMatOm && M.om_valid) {
        const float cth = -dot(in, sp.nrm);
        if (!(fabsf(dot(out, sp.nrm) - cth) > 1e-6f)) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const Dual<2> r = d_om_channel(M.om_n[c], M.om_k[c], cth);
                g.d[c][c] = r.d[0];
                g.d[c][3 + c] = r.d[1];
            }
        }
    }
    return f;
}

// adds t to a gradient slot unless it is not finite: a degenerate path (an
// infinite sample of the forward estimator) must not poison the sum
__device__ __forceinline__ void add_finite(float& slot, float t)
{
    if (fabsf(t) <= kFltMax) slot += t;
}

// adds sum_c a[c] * g.d[c][i] to the material's parameter slots (`mat`:
// the material's number within the rendered scene)
__device__ __forceinline__ void accumulate(float* acc, const DevMaterial& M, uint32_t mat, int nmat, V3 a,
                                           const LocalGrad& g)
{
    if (mat >= (uint32_t)nmat) return;  // the missing material has no parameters
    const float av[3] = {a.x, a.y, a.z};
    float* o = acc + mat * kSlots;
    if (M.type == kMatPbr) {
        const float rough = sqrtf(M.alpha);  // alpha = roughness^2
        for (int c = 0; c < 3; ++c) {
            add_finite(o[0], av[c] * g.d[c][0]);
            add_finite(o[1], av[c] * g.d[c][1]);
            add_finite(o[2], av[c] * g.d[c][2]);
            add_finite(o[3], av[c] * g.d[c][3] * 2.0f * rough);
            add_finite(o[4], av[c] * g.d[c][4]);
        }
    } else if (M.type == kMatOm) {
        for (int c = 0; c < 3; ++c) {
            add_finite(o[5 + c], av[c] * g.d[c][c]);
            add_finite(o[8 + c], av[c] * g.d[c][3 + c]);
        }
    }
}

// BDPTRenderer::isConnected (BDPTRenderer.cpp:208-235)
__device__ __forceinline__ bool connected(const DevScene& S, const uint32_t* items, V3 A, V3 B, TraceStack& st,
                                          TraceCounters& tc)
{
    V3 dir = B - A;
    const float len = sqrtf(dot(dir, dir));
    const float safeD = 2.0f * kEpsAcc * kEps * max_abs(A, 1.0f);
    if (len <= safeD) return true;
    dir = v3(dir.x / len, dir.y / len, dir.z / len);
    float tnear = safeD;
    const float tfar = len + (0.1f * len > safeD ? 0.1f * len : safeD);
    RayHit h;
    if (!scene_intersect(S, items, A, dir, tnear, tfar, h, st, tc)) return true;
    const Surf sp = surface_point(S, h.inst, h.prim, h.u, h.v, false);
    const V3 dd = sp.pos - B;
    const float sb = 10.0f * kEps * max_abs(B, 1.0f);
    return dot(dd, dd) <= sb * sb;
}

struct LightVert {
    V3 pos, rad;   // connection end point and radiance (lv_pos, lv_rad)
    V3 w, pre;     // sampled weight (brdf x ct) and the product before it (x Rad0 x att)
    V3 q;          // adjoint of rad: sum over camera vertices of delta * tp * f * c
    uint32_t mat;
    LocalGrad g;   // d w / d params
};
struct CamVert {
    V3 tp, w, G;   // throughput at the vertex, sampled weight, local contribution
    uint32_t mat;
    bool has_w;    // the path continued from this vertex
    LocalGrad gw;  // d w / d params
    LocalGrad gG;  // d G / d params (through the connection evaluations)
};

// 4 resident blocks of 128 (128 registers, some spilled): 0.109 s per
// gradient of the 512x512x32 adjoint benchmark and 0.497 s per inverse-fit
// step, against 0.111 / 0.509 at the natural 168 registers (3 blocks) and
// 0.115 / 0.531 at 246 registers (2 blocks, no spills)
__global__ void __launch_bounds__(kAdjThreads, 4) k_adjoint(AdjArgs A)
{
    __shared__ uint2 sstack[kStackShared * kAdjThreads];
    __shared__ float sgrad[kAdjMaxMaterials * kSlots];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kAdjThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    for (int i = threadIdx.x; i < kAdjMaxMaterials * kSlots; i += blockDim.x) sgrad[i] = 0.0f;
    __syncthreads();
    const DevScene& S = A.S;
    const int nmat = A.num_user_materials;
    float acc[kAdjMaxMaterials * kSlots];
#pragma unroll 1
    for (int i = 0; i < kAdjMaxMaterials * kSlots; ++i) acc[i] = 0.0f;
    LightVert L[kAdjMaxVerts];
    CamVert Cv[kAdjMaxVerts];
    const float inv_spp = 1.0f / (float)A.spp;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < A.paths;
         g += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t pixel = (uint32_t)(g / A.spp);
        const uint32_t sample = (uint32_t)(A.sample_offset + g % A.spp);
        const float* ad = A.adj + 3 * (size_t)pixel;
        const V3 delta = v3(ad[0] * inv_spp, ad[1] * inv_spp, ad[2] * inv_spp);
        if (delta.x == 0.0f && delta.y == 0.0f && delta.z == 0.0f) continue;

        // ---- light subpath (k_light_gen, k_extend, k_light_shade)
        int nl = 0;  // light vertices on surfaces (lv[1..nl])
        V3 l0pos = v3(0, 0, 0);
        uint32_t li = 0;
        if (S.num_lights > 0) {
            const float d = rng4(A.seed, pixel, sample, 0u, kStreamLight).u[0] * S.light_max;
            const int N = S.num_lights;
            if (N > 1) {
                if (d <= S.light_cdf[0])
                    li = 0;
                else if (d >= S.light_cdf[N - 2])
                    li = N - 1;
                else {
                    int lo = 0, hi = N - 1;
                    while (lo < hi) {
                        int C = (lo + hi) / 2;
                        if (d <= S.light_cdf[C])
                            hi = C;
                        else
                            lo = C + 1;
                    }
                    li = (lo + hi) / 2;
                }
            }
            V3 R = light_direction(A.seed, pixel, sample);  // as k_light_gen
            const float4 lp = __ldg(S.light_pos + li);
            const float4 I = __ldg(S.light_int + li);
            l0pos = v3(lp.x, lp.y, lp.z);
            const V3 rad0 = v3(I.x * A.light_scale, I.y * A.light_scale, I.z * A.light_scale);
            V3 ltp = v3(1.0f, 1.0f, 1.0f);
            float att = 1.0f;
            V3 o = shifted_origin(l0pos, R, 1.0f);
            float tn = 0.0f;
            for (int b = 1; b <= A.light_bounces && b < kAdjMaxVerts; ++b) {
                RayHit h;
                if (!scene_intersect(S, A.items, o, R, tn, kFltMax, h, st, tc)) break;
                const Surf sp = surface_point(S, h.inst, h.prim, h.u, h.v, true);
                const DevMaterial M = S.mats[sp.mat];
                const Rng4 u = rng4(A.seed, pixel, sample, kDimLightBounce + (uint32_t)b, kStreamLight);
                V3 O;
                LightVert& lv = L[b];
                const V3 brdf = sample_with_grad(S, M, sp, R, false, u, O, lv.g);
                const float ct = fabsf(dot(R, sp.nrm));
                const V3 tp = v3(ltp.x * brdf.x * ct, ltp.y * brdf.y * ct, ltp.z * brdf.z * ct);
                if (b == 1) {
                    const V3 dd = sp.pos - l0pos;
                    att = light_attenuation(A.atten_mode, A.min_dist, sqrtf(dot(dd, dd)), lp.w);
                }
                const V3 orad = v3(tp.x * rad0.x * att, tp.y * rad0.y * att, tp.z * rad0.z * att);
                if (intensity(orad) < A.cut) break;
                lv.pos = sp.pos;
                lv.rad = orad;
                lv.w = v3(brdf.x * ct, brdf.y * ct, brdf.z * ct);
                lv.pre = v3(ltp.x * rad0.x * att, ltp.y * rad0.y * att, ltp.z * rad0.z * att);
                lv.q = v3(0, 0, 0);
                lv.mat = sp.mat;
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int i = 0; i < 6; ++i) lv.g.d[c][i] *= ct;
                nl = b;
                ltp = tp;
                if (!(b < A.light_bounces && (tp.x != 0.0f || tp.y != 0.0f || tp.z != 0.0f))) break;
                o = shifted_origin(sp.pos, O, 1.0f);
                R = O;
            }
        }
        const int lp_len = S.num_lights > 0 ? nl + 1 : 0;

        // ---- camera subpath (k_camera_gen, k_extend, k_camera_shade, k_shadow)
        int nc = 0;
        {
            const Rng4 r = rng4(A.seed, pixel, sample, 0u, kStreamCamera);
            V3 O0, D;
            camera_ray(A.cam, (int)(pixel % (uint32_t)A.cam.width), (int)(pixel / (uint32_t)A.cam.width), r.u[0],
                       r.u[1], O0, D);
            V3 o = shifted_origin(O0, D, 1.0f);
            float tn = 0.0f;
            V3 tp = v3(1.0f, 1.0f, 1.0f);
            for (int b = 1; b <= A.cam_bounces && nc < kAdjMaxVerts; ++b) {
                CamVert& cv = Cv[nc++];
                cv.tp = tp;
                cv.has_w = false;
                cv.mat = 0xFFFFFFFFu;
                cv.G = v3(0, 0, 0);
                lg_zero(cv.gG);
                RayHit h;
                if (!scene_intersect(S, A.items, o, D, tn, kFltMax, h, st, tc)) {
                    if (S.env.present && b <= A.max_len) cv.G = env_radiance(S.env, D);
                    break;
                }
                const Surf sp = surface_point(S, h.inst, h.prim, h.u, h.v, true);
                const DevMaterial M = S.mats[sp.mat];
                cv.mat = sp.mat;
                const Rng4 u = rng4(A.seed, pixel, sample, (uint32_t)b, kStreamCamera);
                V3 Onext;
                const V3 brdf = sample_with_grad(S, M, sp, D, true, u, Onext, cv.gw);
                const float ct = fabsf(dot(Onext, sp.nrm));
                const V3 outV = -D;
                for (int li_v = 0; li_v < lp_len && li_v + b <= A.max_len; ++li_v) {
                    const V3 lPos = li_v == 0 ? l0pos : L[li_v].pos;
                    V3 lRad;
                    const V3 LC = normalize(sp.pos - lPos);
                    if (li_v == 0) {
                        const float4 I = __ldg(S.light_int + li);
                        const float4 Lp = __ldg(S.light_pos + li);
                        const V3 dd = sp.pos - lPos;
                        const float lsc = light_attenuation(A.atten_mode, A.min_dist, sqrtf(dot(dd, dd)), Lp.w);
                        const float f = A.light_scale * lsc;
                        lRad = v3(I.x * f, I.y * f, I.z * f);
                    } else {
                        lRad = L[li_v].rad;
                    }
                    const float c = fabsf(dot(LC, sp.nrm));
                    V3 lc = v3(lRad.x * c * tp.x, lRad.y * c * tp.y, lRad.z * c * tp.z);
                    if (intensity(lc) < A.cut) continue;
                    LocalGrad ge;
                    const V3 f = eval_with_grad(M, sp, LC, outV, ge) * c;
                    lc = v3(f.x * tp.x * lRad.x, f.y * tp.y * lRad.y, f.z * tp.z * lRad.z);
                    if (intensity(lc) < A.cut) continue;
                    if (!connected(S, A.items, lPos, sp.pos, st, tc)) continue;
                    cv.G = cv.G + mul(f, lRad);
                    const float lr[3] = {lRad.x * c, lRad.y * c, lRad.z * c};
#pragma unroll
                    for (int cc = 0; cc < 3; ++cc)
#pragma unroll
                        for (int i = 0; i < 6; ++i) cv.gG.d[cc][i] += ge.d[cc][i] * lr[cc];
                    if (li_v > 0) L[li_v].q = L[li_v].q + mul(mul(delta, tp), f);
                }
                const V3 tpn = v3(tp.x * brdf.x * ct, tp.y * brdf.y * ct, tp.z * brdf.z * ct);
                cv.w = v3(brdf.x * ct, brdf.y * ct, brdf.z * ct);
#pragma unroll
                for (int cc = 0; cc < 3; ++cc)
#pragma unroll
                    for (int i = 0; i < 6; ++i) cv.gw.d[cc][i] *= ct;
                if (!(b < A.cam_bounces && (tpn.x != 0.0f || tpn.y != 0.0f || tpn.z != 0.0f))) break;
                cv.has_w = true;
                tp = tpn;
                o = shifted_origin(sp.pos, Onext, 1.0f);
                D = Onext;
            }
        }

        // ---- backward over the camera vertices: R = suffix radiance after a vertex
        V3 Rs = v3(0, 0, 0);
        for (int b = nc - 1; b >= 0; --b) {
            const CamVert& cv = Cv[b];
            if (cv.mat != 0xFFFFFFFFu) {
                const DevMaterial M = S.mats[cv.mat];
                // d/dparams of tp_b * (G_b + w_b * R_{b+1})
                const V3 a = mul(delta, cv.tp);
                accumulate(acc, M, cv.mat - A.mat_base, nmat, a, cv.gG);
                if (cv.has_w) accumulate(acc, M, cv.mat - A.mat_base, nmat, mul(a, Rs), cv.gw);
            }
            Rs = cv.has_w ? cv.G + mul(cv.w, Rs) : cv.G;
        }
        // ---- backward over the light vertices: S = suffix of q through the weights
        V3 Ss = v3(0, 0, 0);
        for (int j = nl; j >= 1; --j) {
            const LightVert& lv = L[j];
            Ss = (j == nl) ? lv.q : lv.q + mul(L[j + 1].w, Ss);
            accumulate(acc, S.mats[lv.mat], lv.mat - A.mat_base, nmat, mul(lv.pre, Ss), lv.g);
        }
    }
    // ---- reduce: warp shuffles, block shared memory, one atomic per block and slot
    const int lane = threadIdx.x & 31;
    for (int i = 0; i < nmat * kSlots; ++i) {
        float v = acc[i];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if (lane == 0 && v != 0.0f) atomicAdd(&sgrad[i], v);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nmat * kSlots; i += blockDim.x)
        if (sgrad[i] != 0.0f) atomicAdd(&A.grad[i], sgrad[i]);
}

}  // namespace

void adjoint_frame(SceneHost& s, const omv_camera& cam, const omv_params& p, const float* d_adjoint, float* d_grad,
                   cudaStream_t st, int part, const DevMaterial* mats)
{
    if (part < 0 || part >= (int)s.parts.size()) throw ArgError("adjoint scene (part) out of range");
    const ScenePart& P = s.parts[part];
    if (cam.width <= 0 || cam.height <= 0) throw ArgError("camera resolution must be positive");
    if (p.samples_per_pixel <= 0) throw ArgError("the adjoint needs at least one sample per pixel");
    if (p.camera_bounces < 0 || p.light_bounces < 0) throw ArgError("negative bounce count");
    if (p.camera_bounces >= kAdjMaxVerts || p.light_bounces >= kAdjMaxVerts)
        throw ArgError("the adjoint supports at most 15 camera and 15 light bounces");
    const int nmat = P.mat_count;
    if (nmat > kAdjMaxMaterials) throw ArgError("the adjoint supports at most 16 materials per scene");
    if (!d_adjoint || !d_grad) throw ArgError("adjoint image and gradient buffers are required");
    if (p.estimator != OMV_ESTIMATOR_REFERENCE) throw ArgError("the adjoint replays the reference estimator only");
    for (const DevMaterial& m : s.h_mats)
        if (m.type == kMatPbr && (m.textured || m.emissive_on))
            throw ArgError("the adjoint differentiates untextured materials only");
    AdjArgs A;
    A.S = s.dev;
    // the scene of the group: its top-level tree, its lights, the job's materials
    A.S.tlas_root = P.tlas_root;
    A.S.light_pos += P.light_base;
    A.S.light_int += P.light_base;
    A.S.light_cdf += P.light_base;
    A.S.num_lights = P.light_count;
    A.S.light_max = P.light_max;
    if (mats) A.S.mats = mats;
    A.mat_base = (uint32_t)P.mat_base;
    A.items = s.tlas_items;
    A.cam = cam;
    A.seed = p.seed;
    A.paths = (int64_t)cam.width * cam.height * p.samples_per_pixel;
    A.spp = p.samples_per_pixel;
    A.sample_offset = p.sample_offset;
    A.cam_bounces = p.camera_bounces;
    A.light_bounces = p.light_bounces;
    A.max_len = p.max_path_length;
    A.atten_mode = p.light_distance_attenuation;
    A.light_scale = p.light_scale;
    A.min_dist = p.light_min_distance;
    A.cut = p.ray_cut_value;
    A.adj = d_adjoint;
    A.grad = d_grad;
    A.num_user_materials = nmat;
    int occ = 0;
    OMV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_adjoint, kAdjThreads, 0));
    const int64_t want = (A.paths + kAdjThreads - 1) / kAdjThreads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)std::max(1, occ) * s.num_sms * 4));
    k_adjoint<<<grid, kAdjThreads, 0, st>>>(A);
    OMV_CUDA(cudaGetLastError());
}

void adjoint_batch(SceneHost& s, int n, const omv_adjoint_job* jobs, const omv_params& p, cudaStream_t st)
{
    for (int i = 0; i < n; ++i) {  // checked before anything is enqueued
        const omv_job& j = jobs[i].job;
        if (j.material_set < -1 || j.material_set >= s.num_mat_sets)
            throw ArgError("adjoint job material set out of range");
        if (j.part < 0 || j.part >= (int)s.parts.size()) throw ArgError("adjoint job scene (part) out of range");
        if (j.samples_per_pixel <= 0 || j.camera.width <= 0 || j.camera.height <= 0)
            throw ArgError("adjoint job without samples or pixels");
        if (!jobs[i].d_adjoint_rgb || !jobs[i].d_grad) throw ArgError("adjoint job without adjoint image or gradient");
    }
    for (int i = 0; i < n; ++i) {
        const omv_job& j = jobs[i].job;
        omv_params q = p;
        q.samples_per_pixel = j.samples_per_pixel;
        q.sample_offset = j.sample_offset;
        q.seed = j.seed;
        const DevMaterial* mats = j.material_set < 0 ? nullptr : s.mat_sets + (size_t)j.material_set * s.num_materials;
        adjoint_frame(s, j.camera, q, jobs[i].d_adjoint_rgb, jobs[i].d_grad, st, j.part, mats);
    }
}

}  // namespace omv
