// Per-vertex shading shared by the wavefront kernels and the path-replay
// adjoint: surface point of a hit, material sampling and evaluation, and the
// alpha-mask-aware closest-hit query of the reference.
#pragma once

#include "omv_device.cuh"
#include "omv_types.h"
#include "trace.cuh"

namespace omv {

struct Surf {
    V3 pos, nrm, tan, bin;
    float tw;
    uint32_t mat;
    uint32_t inst;
    uint32_t face;
    uint32_t vert_base;
    uint32_t face_base;
    float bu, bv;       // hit barycentrics (u, v); the first weight is 1 - u - v
    uint32_t uv_mask;   // coordinate sets of the mesh
};

// ------------------------------------------------------------ textures ---

// what a texture lookup needs of a hit, passed by value to the out-of-line
// texture helpers (a Surf passed by reference would live in local memory)
struct TexHit {
    uint32_t face, vert_base, face_base, uv_mask;
    float bu, bv;
};
__device__ __forceinline__ TexHit tex_hit(const Surf& sp)
{
    return TexHit{sp.face, sp.vert_base, sp.face_base, sp.uv_mask, sp.bu, sp.bv};
}

// BitmapTexture::getPixCoords + texture(u, v, fvec4) (BitmapTexture.cpp:73-125):
// bilinear over the four wrapped neighbours, texels scaled by 1/255
__device__ __forceinline__ float4 tex_sample(const DevScene& S, int t, float u, float v)
{
    const DevTexture T = S.textures[t];
    if (!T.present) return make_float4(0.5f, 0.5f, 0.5f, 1.0f);
    const int W = T.width, H = T.height;
    const float upage = floorf(u - 0.5f / (float)W);
    const float vpage = floorf(v - 0.5f / (float)H);
    u -= upage;
    v -= vpage;
    u *= (float)W;
    v *= (float)H;
    const int iu = (int)u, iv = (int)v;
    const float kui = u - (float)iu, kvi = v - (float)iv;
    const float ku = 1.0f - kui, kv = 1.0f - kvi;
    const int l = iu % W, r = (iu + 1) % W, b = iv % H, tp = (iv + 1) % H;
    const uchar4* px = S.texels + T.offset;
    const uchar4 c0 = __ldg(px + b * W + l), c1 = __ldg(px + b * W + r);
    const uchar4 c2 = __ldg(px + tp * W + l), c3 = __ldg(px + tp * W + r);
    const float w0 = ku * kv, w1 = kui * kv, w2 = ku * kvi, w3 = kui * kvi;
    constexpr float sc = 1.0f / 255.0f;
    return make_float4((float)c0.x * w0 * sc + (float)c1.x * w1 * sc + (float)c2.x * w2 * sc + (float)c3.x * w3 * sc,
                       (float)c0.y * w0 * sc + (float)c1.y * w1 * sc + (float)c2.y * w2 * sc + (float)c3.y * w3 * sc,
                       (float)c0.z * w0 * sc + (float)c1.z * w1 * sc + (float)c2.z * w2 * sc + (float)c3.z * w3 * sc,
                       (float)c0.w * w0 * sc + (float)c1.w * w1 * sc + (float)c2.w * w2 * sc + (float)c3.w * w3 * sc);
}

__device__ __forceinline__ float2 vertex_uv(const DevScene& S, int ch, uint32_t vi)
{
    if (ch == 0) {
        const float4 w = __ldg(S.verts + 3 * (size_t)vi + 2);
        return make_float2(w.z, w.w);
    }
    return __ldg(S.uv1 + vi);
}

// SurfacePoint::getTexCoords -> RenderMesh::getTexCoord (RenderMesh.cpp:146-157):
// (0, 0) and false when the mesh lacks the coordinate set
__device__ __forceinline__ bool tex_coords(const DevScene& S, const TexHit& sp, int ch, float2& tc)
{
    tc = make_float2(0.0f, 0.0f);
    if (ch < 0 || ch > 1 || !(sp.uv_mask & (1u << ch))) return false;
    const uint32_t* F = S.faces + 3 * (size_t)(sp.face_base + sp.face);
    const float2 a = vertex_uv(S, ch, sp.vert_base + __ldg(F));
    const float2 b = vertex_uv(S, ch, sp.vert_base + __ldg(F + 1));
    const float2 c = vertex_uv(S, ch, sp.vert_base + __ldg(F + 2));
    const float b0 = 1.0f - sp.bu - sp.bv, b1 = sp.bu, b2 = sp.bv;
    tc = make_float2(a.x * b0 + b.x * b1 + c.x * b2, a.y * b0 + b.y * b1 + c.y * b2);
    return true;
}

// multVector3(TM, (u, v, 1)) then the bitmap lookup
__device__ __forceinline__ float4 tex_transformed(const DevScene& S, const DevTexRef& t, float2 uv)
{
    const float uu = t.m[0] * uv.x + t.m[1] * uv.y + t.m[2] * 1.0f;
    const float vv = t.m[3] * uv.x + t.m[4] * uv.y + t.m[5] * 1.0f;
    return tex_sample(S, t.tex, uu, vv);
}

// a slot as PhysicallyBasedMaterial::Helper reads it: only when the image
// exists and the mesh has the slot's coordinate set
__device__ __forceinline__ bool tex_slot(const DevScene& S, const DevMaterial& M, int slot, const TexHit& sp,
                                         float4& out)
{
    const DevTexRef& t = M.tex[slot];
    float2 uv;
    if (t.tex < 0 || !tex_coords(S, sp, t.ch, uv)) return false;
    out = tex_transformed(S, t, uv);
    return true;
}

// per-vertex PBR values: getTextureRGBA, getTextureOccMetRoughValues and
// occluseColor (PhysicallyBasedMaterial.cpp:27-95, 178-200, 261-276)
struct PbrParams {
    float color[4];
    float metal, alpha;
    bool transmissive;
    float omr_metal, omr_rough;  // before the roughness clamp (the validation subjects)
};

static __device__ __noinline__ PbrParams pbr_params_textured(const DevScene& S, const DevMaterial& M, TexHit sp)
{
    PbrParams P;
    float4 rgba = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    tex_slot(S, M, kTexBase, sp, rgba);
    P.color[0] = rgba.x * M.factor[0];
    P.color[1] = rgba.y * M.factor[1];
    P.color[2] = rgba.z * M.factor[2];
    P.color[3] = M.alpha_mode != OMV_ALPHA_BLEND ? 1.0f : rgba.w * M.factor[3];
    P.transmissive = M.double_sided || P.color[3] < 1.0f;
    float o0 = 1.0f, o1 = M.metal, o2 = M.rough;
    float4 tb;
    if (tex_slot(S, M, kTexMetRough, sp, tb)) {
        o0 *= tb.x;
        o1 *= tb.z;
        o2 *= tb.y;
    }
    if (M.tex[kTexOcclusion].tex != M.tex[kTexMetRough].tex && tex_slot(S, M, kTexOcclusion, sp, tb)) o0 = tb.x;
    for (int i = 0; i < 3; ++i) P.color[i] = lerpf(P.color[i], o0 * P.color[i], M.occl_strength);
    P.omr_metal = o1;
    P.omr_rough = o2;
    P.metal = o1;
    const float rough = clampf(o2, 0.00001f, 0.99999f);
    P.alpha = __fmul_rn(rough, rough);  // std::pow(roughness, 2.0f)
    return P;
}

__device__ __forceinline__ PbrParams pbr_params(const DevScene& S, const DevMaterial& M, const Surf& sp)
{
    if (M.textured) return pbr_params_textured(S, M, tex_hit(sp));
    PbrParams P;
#pragma unroll
    for (int i = 0; i < 4; ++i) P.color[i] = M.color[i];
    P.metal = M.metal;
    P.alpha = M.alpha;
    P.transmissive = M.transmissive != 0;
    P.omr_metal = M.metal;
    P.omr_rough = M.rough;
    return P;
}

// PhysicallyBasedMaterial::modifyFrame (:147-167): the normal map's tangent-space
// normal, or (0, 0, 1) without one
static __device__ __noinline__ V3 normal_map(const DevScene& S, const DevMaterial& M, TexHit sp)
{
    float4 t;
    if (!tex_slot(S, M, kTexNormal, sp, t)) return v3(0.0f, 0.0f, 1.0f);
    if (t.z <= 0.5f) t.z = 0.5f + kEps;
    V3 tn = v3(2.0f * t.x + -1.0f, 2.0f * t.y + -1.0f, 2.0f * t.z + -1.0f);
    tn.x = M.normal_scale * tn.x;
    tn.y = M.normal_scale * tn.y;
    return normalize(tn);
}

// PhysicallyBasedMaterial::getEmissivity + Helper::getTextureEmissivity
// (:96-117, 280-287, 293-299); only called for an emissive material
static __device__ __noinline__ V3 pbr_emission(const DevScene& S, const DevMaterial& M, TexHit sp)
{
    float2 euv;
    tex_coords(S, sp, M.tex[kTexEmissive].ch, euv);
    const float4 t = tex_transformed(S, M.tex[kTexEmissive], euv);
    return v3(t.x * M.emissive[0], t.y * M.emissive[1], t.z * M.emissive[2]);
}

__device__ __forceinline__ V3 m33(const float* m, V3 v)
{
    return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

// BDPTRenderer::computeSurfacePoint -> RenderMesh::computeSurfacePoint
// (RenderMesh.cpp:159-196), then SurfacePoint::applyTextureNormal((0,0,1))
// (SurfacePoint.cpp:19-34) as every material's modifyFrame without a normal map
__device__ __forceinline__ Surf surface_point(const DevScene& S, uint32_t inst, uint32_t prim, float u, float v,
                                              bool frame, const DevMaterial* M = nullptr)
{
    const DevInstance* I = S.insts + inst;
    Surf sp;
    sp.inst = inst;
    sp.face = prim;
    sp.mat = __ldg(&I->material);
    sp.vert_base = __ldg(&I->vert_base);
    sp.face_base = __ldg(&I->face_base);
    sp.bu = u;
    sp.bv = v;
    sp.uv_mask = __ldg(&I->uv_mask);
    const uint32_t* F = S.faces + 3 * (size_t)(sp.face_base + prim);
    const uint32_t f0 = __ldg(F), f1 = __ldg(F + 1), f2 = __ldg(F + 2);
    const float b0 = 1.0f - u - v, b1 = u, b2 = v;
    const float4* V0 = S.verts + 3 * (size_t)(sp.vert_base + f0);
    const float4* V1 = S.verts + 3 * (size_t)(sp.vert_base + f1);
    const float4* V2 = S.verts + 3 * (size_t)(sp.vert_base + f2);
    const float4 a0 = __ldg(V0), a1 = __ldg(V1), a2 = __ldg(V2);
    V3 pp = v3(b0 * a0.x + b1 * a1.x + b2 * a2.x, b0 * a0.y + b1 * a1.y + b2 * a2.y, b0 * a0.z + b1 * a1.z + b2 * a2.z);
    float m[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) m[k] = __ldg(&I->xf[k]);
    sp.pos = v3(m[0] * pp.x + m[1] * pp.y + m[2] * pp.z + m[3], m[4] * pp.x + m[5] * pp.y + m[6] * pp.z + m[7],
                m[8] * pp.x + m[9] * pp.y + m[10] * pp.z + m[11]);
    if (!frame) return sp;
    const float4 c0 = __ldg(V0 + 1), c1 = __ldg(V1 + 1), c2 = __ldg(V2 + 1);
    const float4 d0 = __ldg(V0 + 2), d1 = __ldg(V1 + 2), d2 = __ldg(V2 + 2);
    V3 pn = v3(b0 * a0.w + b1 * a1.w + b2 * a2.w, b0 * c0.x + b1 * c1.x + b2 * c2.x, b0 * c0.y + b1 * c1.y + b2 * c2.y);
    V3 pt = v3(b0 * c0.z + b1 * c1.z + b2 * c2.z, b0 * c0.w + b1 * c1.w + b2 * c2.w, b0 * d0.x + b1 * d1.x + b2 * d2.x);
    float tw = b0 * d0.y + b1 * d1.y + b2 * d2.y;
    tw = tw >= 0.0f ? 1.0f : -1.0f;
    pn = normalize_if_needed(pn);
    const float tn = dot(pn, pt);
    pt = normalize_if_needed(pt - pn * tn);
    V3 pbn = cross(pn, pt) * tw;
    float nm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) nm[k] = __ldg(&I->nrm[k]);
    V3 n = normalize_if_needed(m33(nm, pn));
    V3 t = normalize_if_needed(m33(nm, pt));
    V3 b = normalize_if_needed(m33(nm, pbn));
    // modifyFrame -> applyTextureNormal(tn): nn = tn.x t + tn.y b + tn.z n, with
    // tn = (0, 0, 1) unless the material (given) has a normal map
    const V3 tnm = (M && M->type == kMatPbr && M->tex[kTexNormal].tex >= 0) ? normal_map(S, *M, tex_hit(sp))
                                                                          : v3(0.0f, 0.0f, 1.0f);
    n = normalize_if_needed(t * tnm.x + b * tnm.y + n * tnm.z);
    t = normalize_if_needed(cross(b, n));
    b = cross(n, t) * tw;
    sp.nrm = n;
    sp.tan = t;
    sp.bin = b;
    sp.tw = tw;
    return sp;
}

// triangleNormal of the hit face through the normal matrix, normalised
// (OpenMaterial.cpp:76-86)
__device__ __forceinline__ V3 face_normal(const DevScene& S, const Surf& sp)
{
    const uint32_t* F = S.faces + 3 * (size_t)(sp.face_base + sp.face);
    const float4 p0 = __ldg(S.verts + 3 * (size_t)(sp.vert_base + __ldg(F)));
    const float4 p1 = __ldg(S.verts + 3 * (size_t)(sp.vert_base + __ldg(F + 1)));
    const float4 p2 = __ldg(S.verts + 3 * (size_t)(sp.vert_base + __ldg(F + 2)));
    V3 e1 = v3(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z);
    V3 e2 = v3(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z);
    float nm[9];
    const DevInstance* I = S.insts + sp.inst;
#pragma unroll
    for (int k = 0; k < 9; ++k) nm[k] = __ldg(&I->nrm[k]);
    return normalize(m33(nm, cross(e1, e2)));
}

// RenderMaterial::getRayAndBrdf of each material kind; u = the vertex's
// uniforms, P = the vertex's PBR values (pbr_params)
__device__ __forceinline__ V3 material_sample(const DevScene& S, const DevMaterial& M, const PbrParams& P,
                                              const Surf& sp, V3 in, bool inv, const Rng4& u, V3& out,
                                              SampleInfo* info = nullptr)
{
    if (M.type == kMatPbr) {  // PhysicallyBasedMaterial::getRayAndBrdf (:248-291)
        BsdfIn d;
        d.I = in;
        d.N = sp.nrm;
        d.T = sp.tan;
#pragma unroll
        for (int i = 0; i < 4; ++i) d.color[i] = P.color[i];
        d.metal = P.metal;
        d.alpha = P.alpha;
        d.eta = M.eta;
        d.transmissive = P.transmissive;
        return bsdf_sample_indirect(d, u.u[0], u.u[1], u.u[2], out, info);
    }
    if (M.type == kMatOm) {  // OpenMaterial::defineNextDirection + getRayAndBrdf (:72-93, :165-232)
        out = reflect3(in, sp.nrm);
        V3 tfn = face_normal(S, sp);
        float corr = dot(out, tfn);
        if (corr < 0.1f) out = normalize(tfn * (0.1f - corr) + out);
        if (!M.om_valid) return v3(0.0f, 0.0f, 0.0f);
        float c = dot(out, sp.nrm);
        return v3(om_channel(M.om_n[0], M.om_k[0], c), om_channel(M.om_n[1], M.om_k[1], c),
                  om_channel(M.om_n[2], M.om_k[2], c));
    }
    // missing material: DiffuseColorMaterial (uniform hemisphere, brdf = albedo)
    out = to_basis(sp.tan, sp.bin, sp.nrm, uniform_hemisphere(u.u[0], u.u[1]));
    (void)inv;
    return v3(M.color[0], M.color[1], M.color[2]);
}

// RenderMaterial::getBrdf (impSmpScale = false) for a connection
__device__ __forceinline__ V3 material_eval(const DevMaterial& M, const PbrParams& P, const Surf& sp, V3 in, V3 out)
{
    if (M.type == kMatPbr) {  // PhysicallyBasedMaterial::getBrdf (:178-245)
        V3 N = sp.nrm;
        if (dot(in, N) > 0.0f && P.transmissive) N = -N;
        return bsdf_eval_direct(in, out, N, P.color, P.metal, P.alpha);
    }
    if (M.type == kMatOm) {  // OpenMaterial::getBrdf (:95-163): mirror directions only
        if (!M.om_valid) return v3(0.0f, 0.0f, 0.0f);
        float c = -dot(in, sp.nrm);
        if (fabsf(dot(out, sp.nrm) - c) > 1e-6f) return v3(0.0f, 0.0f, 0.0f);
        return v3(om_channel(M.om_n[0], M.om_k[0], c), om_channel(M.om_n[1], M.om_k[1], c),
                  om_channel(M.om_n[2], M.om_k[2], c));
    }
    return v3(M.color[0], M.color[1], M.color[2]);
}

// the BsdfIn material_sample builds for a PBR vertex
__device__ __forceinline__ BsdfIn pbr_bsdf_in(const DevMaterial& M, const PbrParams& P, const Surf& sp, V3 in)
{
    BsdfIn d;
    d.I = in;
    d.N = sp.nrm;
    d.T = sp.tan;
#pragma unroll
    for (int i = 0; i < 4; ++i) d.color[i] = P.color[i];
    d.metal = P.metal;
    d.alpha = P.alpha;
    d.eta = M.eta;
    d.transmissive = P.transmissive;
    return d;
}

// the same without textures (the material's constants)
__device__ __forceinline__ V3 material_sample(const DevScene& S, const DevMaterial& M, const Surf& sp, V3 in, bool inv,
                                              const Rng4& u, V3& out, SampleInfo* info = nullptr)
{
    return material_sample(S, M, pbr_params(S, M, sp), sp, in, inv, u, out, info);
}
__device__ __forceinline__ V3 material_eval(const DevMaterial& M, const Surf& sp, V3 in, V3 out)
{
    PbrParams P;
#pragma unroll
    for (int i = 0; i < 4; ++i) P.color[i] = M.color[i];
    P.metal = M.metal;
    P.alpha = M.alpha;
    P.transmissive = M.transmissive != 0;
    return material_eval(M, P, sp, in, out);
}

// PhysicallyBasedMaterial::isMasked (:301-316) for a MASK material with a base
// colour texture: factor alpha x the texture's alpha at the untransformed
// coordinates (1 where the mesh lacks the set, BitmapTexture.cpp:142-156)
static __device__ __noinline__ bool texture_masked(const DevScene& S, const DevMaterial& M, uint32_t inst,
                                                   uint32_t prim, float u, float v)
{
    const DevInstance* I = S.insts + inst;
    const TexHit sp{prim, __ldg(&I->vert_base), __ldg(&I->face_base), __ldg(&I->uv_mask), u, v};
    float2 uv;
    float a = 1.0f;
    if (tex_coords(S, sp, M.tex[kTexBase].ch, uv)) a = tex_sample(S, M.tex[kTexBase].tex, uv.x, uv.y).w;
    return M.factor[3] * a < M.cutoff;
}

// whether sceneIntersect skips this hit: an alpha-masked material (BLEND or
// MASK below the cutoff), or a texture-masked one whose texel is transparent
__device__ __forceinline__ bool hit_masked(const DevScene& S, const RayHit& h)
{
    const uint32_t mat = __ldg(&S.insts[h.inst].material);
    const int masked = S.mats[mat].masked;
    if (!masked) return false;
    return masked != 2 || texture_masked(S, S.mats[mat], h.inst, h.prim, h.u, h.v);
}

// tnear of sceneIntersect's next try after a skipped hit at t
__device__ __forceinline__ float masked_retry_tnear(V3 o, V3 d, float t)
{
    V3 org = v3(o.x + t * d.x, o.y + t * d.y, o.z + t * d.z);
    float vv = max_abs(org, 1.0f);
    vv = vv > t ? vv : t;
    const float delta = kEpsAcc * kEps * vv;
    return t + delta;
}

constexpr int kMaskedTries = 10;

// BDPTRenderer::sceneIntersect (BDPTRenderer.cpp:75-102): closest hit, skipping
// alpha-masked materials up to 10 times; tnear persists like the reference's
// RTCRayHit does across the bounces of one path
__device__ __forceinline__ bool scene_intersect(const DevScene& S, const uint32_t* items, V3 o, V3 d, float& tnear,
                                                float tfar, RayHit& h, TraceStack& st, TraceCounters& tc,
                                                uint32_t root = kInvalid)
{
    const float t1 = tfar;
    for (int itr = 0; itr < kMaskedTries; ++itr) {
        if (!trace_closest(S, items, o, d, tnear, tfar, h, st, tc, root)) return false;
        if (!hit_masked(S, h)) return true;
        tnear = masked_retry_tnear(o, d, h.t);
        tfar = t1;
        if (tfar <= tnear) return false;
    }
    return false;
}

}  // namespace omv
