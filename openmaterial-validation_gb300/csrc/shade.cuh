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
};

__device__ __forceinline__ V3 m33(const float* m, V3 v)
{
    return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

// BDPTRenderer::computeSurfacePoint -> RenderMesh::computeSurfacePoint
// (RenderMesh.cpp:159-196), then SurfacePoint::applyTextureNormal((0,0,1))
// (SurfacePoint.cpp:19-34) as every material's modifyFrame without a normal map
__device__ __forceinline__ Surf surface_point(const DevScene& S, uint32_t inst, uint32_t prim, float u, float v,
                                              bool frame)
{
    const DevInstance* I = S.insts + inst;
    Surf sp;
    sp.inst = inst;
    sp.face = prim;
    sp.mat = __ldg(&I->material);
    sp.vert_base = __ldg(&I->vert_base);
    sp.face_base = __ldg(&I->face_base);
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
    // applyTextureNormal((0,0,1)): nn = 0*t + 0*b + 1*n
    n = normalize_if_needed(t * 0.0f + b * 0.0f + n * 1.0f);
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

// RenderMaterial::getRayAndBrdf of each material kind; u = the vertex's uniforms
__device__ __forceinline__ V3 material_sample(const DevScene& S, const DevMaterial& M, const Surf& sp, V3 in, bool inv,
                                              const Rng4& u, V3& out, SampleInfo* info = nullptr)
{
    if (M.type == kMatPbr) {  // PhysicallyBasedMaterial::getRayAndBrdf (:248-291)
        BsdfIn d;
        d.I = in;
        d.N = sp.nrm;
        d.T = sp.tan;
#pragma unroll
        for (int i = 0; i < 4; ++i) d.color[i] = M.color[i];
        d.metal = M.metal;
        d.alpha = M.alpha;
        d.eta = M.eta;
        d.transmissive = M.transmissive != 0;
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
__device__ __forceinline__ V3 material_eval(const DevMaterial& M, const Surf& sp, V3 in, V3 out)
{
    if (M.type == kMatPbr) {  // PhysicallyBasedMaterial::getBrdf (:178-245)
        V3 N = sp.nrm;
        if (dot(in, N) > 0.0f && M.transmissive) N = -N;
        return bsdf_eval_direct(in, out, N, M.color, M.metal, M.alpha);
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

// BDPTRenderer::sceneIntersect (BDPTRenderer.cpp:75-102): closest hit, skipping
// alpha-masked materials up to 10 times; tnear persists like the reference's
// RTCRayHit does across the bounces of one path
__device__ __forceinline__ bool scene_intersect(const DevScene& S, const uint32_t* items, V3 o, V3 d, float& tnear,
                                                float tfar, RayHit& h, TraceStack& st, TraceCounters& tc)
{
    const float t1 = tfar;
    for (int itr = 0; itr < 10; ++itr) {
        if (!trace_closest(S, items, o, d, tnear, tfar, h, st, tc)) return false;
        const uint32_t mat = __ldg(&S.insts[h.inst].material);
        if (!S.mats[mat].masked) return true;
        V3 org = v3(o.x + h.t * d.x, o.y + h.t * d.y, o.z + h.t * d.z);
        float vv = max_abs(org, 1.0f);
        vv = vv > h.t ? vv : h.t;
        const float delta = kEpsAcc * kEps * vv;
        tnear = h.t + delta;
        tfar = t1;
        if (tfar <= tnear) return false;
    }
    return false;
}

}  // namespace omv
