// Device-side math of the render path: vector helpers, the counter-based RNG,
// and the per-vertex material model of the reference renderer.
//
// Functions whose results are compared bit for bit with the CPU oracle (ray
// setup, camera rays, instance transforms, the triangle test) use explicit
// round-to-nearest intrinsics (__fmul_rn/__fadd_rn/...), which the compiler
// never fuses into FMAs.  Everything else may be contracted; it is checked
// against the oracle within 1e-5 relative.  The reference's float library
// calls on that path (sin, cos, pow, acos, asin) are evaluated correctly
// rounded (crmath.cuh).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "crmath.cuh"
#include "omv_types.h"

namespace omv {

constexpr float kPi = 3.14159265358979323846f;      // M_PIf (Constants.h:20)
constexpr float kEps = 1.1920928955078125e-07f;     // fEpsilon (Constants.h:30)
constexpr float kEpsAcc = 3.0f;                     // BDPTRenderer::m_fEpsAcc (BDPTRenderer.h:43)
constexpr float kFltMax = 3.402823466e+38f;
constexpr float kOneMinusUlp = 0.99999994039535522461f;  // nextafter(1, 0)
constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// ------------------------------------------------------------ vectors ---
struct V3 {
    float x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// exact-order variants (no contraction)
__device__ __forceinline__ float dot_rn(V3 a, V3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

// normalize3 (UtilityFunctions.h:202-217): L = 1/|a|, a*L; (1,0,0) for zero
__device__ __forceinline__ V3 normalize_rn(V3 a)
{
    float L = __fsqrt_rn(dot_rn(a, a));
    if (L != 0.0f) {
        L = __fdiv_rn(1.0f, L);
        return v3(__fmul_rn(a.x, L), __fmul_rn(a.y, L), __fmul_rn(a.z, L));
    }
    return v3(1.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ V3 normalize(V3 a)
{
    float L = sqrtf(dot(a, a));
    if (L != 0.0f) {
        L = 1.0f / L;
        return a * L;
    }
    return v3(1.0f, 0.0f, 0.0f);
}
// normalizeIfNeeded3 (UtilityFunctions.h:222-238), eps = 10*FLT_EPSILON
__device__ __forceinline__ V3 normalize_if_needed(V3 a)
{
    const float eps = 10.0f * kEps;
    float sL = dot(a, a);
    if (sL < 1.0f + eps && sL > 1.0f - eps) return a;
    float L = sqrtf(sL);
    if (L != 0.0f) {
        L = 1.0f / L;
        return a * L;
    }
    return v3(1.0f, 0.0f, 0.0f);
}

__device__ __forceinline__ float clampf(float v, float lo, float hi)
{
    float m = v < hi ? v : hi;  // min(value, upper)
    return lo > m ? lo : m;     // max(lower, ...)
}
__device__ __forceinline__ float clamp01(float v) { return clampf(v, 0.0f, 1.0f); }
// lerp(lower, upper, value) = (upper - lower) * value + lower
__device__ __forceinline__ float lerpf(float lo, float up, float v) { return (up - lo) * v + lo; }

// maxAbsInVector (BDPTRenderer.cpp:35-40)
__device__ __forceinline__ float max_abs(V3 v, float th)
{
    float a0 = fabsf(v.x), a1 = fabsf(v.y), a2 = fabsf(v.z);
    float mv = a0 > a1 && a0 > a2 ? a0 : a1 > a2 ? a1 : a2;
    return mv < th ? th : mv;
}
// intensity (BDPTRenderer.cpp:52-55)
__device__ __forceinline__ float intensity(V3 r) { return 0.299f * r.x + 0.587f * r.y + 0.114f * r.z; }

__device__ __forceinline__ V3 ld3(const float* p) { return v3(p[0], p[1], p[2]); }

// ------------------------------------------------------------ Philox ---
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw:
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011), multipliers and
// Weyl key increments as published there.
struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// the reference's uniform float: float(x) / 2^32, kept below 1
// (std::uniform_real_distribution<float> over std::mt19937, RandomSampler.h:59)
__device__ __forceinline__ float u01(uint32_t x)
{
    float r = __fmul_rn(__uint2float_rn(x), 2.3283064365386963e-10f);
    return r >= 1.0f ? kOneMinusUlp : r;
}

// four uniforms for (path, sample, dimension, stream)
struct Rng4 {
    float u[4];
};
__device__ __forceinline__ Rng4 rng4(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim, uint32_t stream)
{
    U4 c{pixel, sample, dim, stream};
    U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    Rng4 o;
    o.u[0] = u01(r.x);
    o.u[1] = u01(r.y);
    o.u[2] = u01(r.z);
    o.u[3] = u01(r.w);
    return o;
}

enum : uint32_t { kStreamCamera = 0u, kStreamLight = 1u };
constexpr uint32_t kDimLightBounce = 1024u;

// The direction of a light path's first ray.  RandomSampler::uniformSphere
// (RandomSampler.h:75-84) draws v uniformly in [0,1)^3 until eps <= |v|^2 <= 1
// and returns v / |v|: a direction uniform over the positive octant of the unit
// sphere (the ball is invariant under rotations).  Drawn here without the
// rejection loop, in which a warp waits for its slowest lane's draws: z
// uniform in [0, 1) (on a sphere, slices of equal height have equal areas) and
// the azimuth uniform in [0, pi/2).
__device__ __forceinline__ V3 light_direction(uint64_t seed, uint32_t pixel, uint32_t sample)
{
    const Rng4 r = rng4(seed, pixel, sample, 1u, kStreamLight);
    const float z = r.u[0];
    const float rxy = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincosf(0.5f * kPi * r.u[1], &s, &c);
    return v3(rxy * c, rxy * s, z);
}

// ------------------------------------------------------ camera / ray ---

// PinholeCamera::getRay (PinholeCamera.cpp:80-95), exact float order
__device__ __forceinline__ void camera_ray(const omv_camera& cam, int x, int y, float ux, float uy, V3& O, V3& R)
{
    float px = __fsub_rn(__fadd_rn((float)x, 0.5f), cam.half_width);
    float py = __fsub_rn(__fadd_rn((float)y, 0.5f), cam.half_height);
    float dx = __fadd_rn(__fmul_rn(1.0f, ux), -0.5f);  // lerp(-0.5, 0.5, u)
    float dy = __fadd_rn(__fmul_rn(1.0f, uy), -0.5f);
    V3 c = normalize_rn(v3(__fadd_rn(px, dx), __fadd_rn(py, dy), cam.focus));
    const float(*M)[3] = cam.rotation;
    R = v3(__fadd_rn(__fadd_rn(__fmul_rn(M[0][0], c.x), __fmul_rn(M[0][1], c.y)), __fmul_rn(M[0][2], c.z)),
           __fadd_rn(__fadd_rn(__fmul_rn(M[1][0], c.x), __fmul_rn(M[1][1], c.y)), __fmul_rn(M[1][2], c.z)),
           __fadd_rn(__fadd_rn(__fmul_rn(M[2][0], c.x), __fmul_rn(M[2][1], c.y)), __fmul_rn(M[2][2], c.z)));
    O = v3(cam.position[0], cam.position[1], cam.position[2]);
}

// setRay + shiftRayAlongDirection (BDPTRenderer.cpp:42-50, 309-321):
// origin moved by (3*eps_shift*FLT_EPSILON) * max(|O|inf, 1) along R
__device__ __forceinline__ V3 shifted_origin(V3 O, V3 R, float eps_shift)
{
    float v = max_abs(O, 1.0f);
    float delta = __fmul_rn(__fmul_rn(__fmul_rn(kEpsAcc, eps_shift), kEps), v);
    return v3(__fadd_rn(O.x, __fmul_rn(delta, R.x)), __fadd_rn(O.y, __fmul_rn(delta, R.y)),
              __fadd_rn(O.z, __fmul_rn(delta, R.z)));
}

// computeLightAttenuation (BDPTRenderer.cpp:104-126)
__device__ __forceinline__ float light_attenuation(int mode, float min_d, float d, float attD)
{
    if (attD >= kFltMax) {
        d = d < min_d ? min_d : d;
        switch (mode) {
            case 1: return 1.0f / d;
            case 2: return 1.0f / (d * d);
            default: return 1.0f;
        }
    }
    float q = 1.0f - d / attD;
    float rD = q > 0.0f ? q : 0.0f;
    switch (mode) {
        case 1: return rD;
        case 2: return sqrtf(rD);
        default: return d < attD ? 1.0f : 0.0f;
    }
}

// ------------------------------------------------------------- BRDF ---

// ndf::GGX and SmithG (BRDFModel.h:40-80)
__device__ __forceinline__ float ggx_pdf(float c, float alpha)
{
    float c2 = c * c;
    float a2 = alpha * alpha;
    float l = lerpf(1.0f, a2, c2);
    return a2 / (kPi * (l * l));
}
// std::pow(a, -2.0f) (BRDFModel.h:55) correctly rounded
__device__ __forceinline__ float ggx_lambda(float a) { return 0.5f * (sqrtf(1.0f + cr::rcp_sq_cr(a)) - 1.0f); }
__device__ __forceinline__ float smith_g1(float c, float alpha)
{
    float a = c / (alpha * sqrtf(1.0f - c * c));
    return (alpha > 0.0f || c < 0.99f) ? 1.0f / (1.0f + ggx_lambda(a)) : 1.0f;
}
__device__ __forceinline__ float smith_g2(float s, float m)
{
    float p = s * m;
    return p / (s + m - p);
}
// std::pow(x, 5.0f) (BRDFModel.h:180, 231) correctly rounded for x >= 2^-20
// (below, x^5 < 2^-100 and the Schlick term it feeds does not see it)
__device__ __forceinline__ float pow5(float x) { return cr::pow5_cr(x); }

struct BsdfIn {
    V3 I, N, T;
    float color[4];
    float metal, alpha, eta;
    bool transmissive;
};

// BSDFModel::evaluate (BRDFModel.h:139-207): kind 0 diffuse, 1 specular, 2 transmitted
__device__ __forceinline__ V3 bsdf_evaluate(V3 vIn, V3 vOut, V3 norm, const float* color, float metal, float alpha,
                                            int kind, V3 Hext, float p)
{
    V3 H = kind == 2 ? Hext : normalize(vOut - vIn);
    float VdotN = clampf(fabsf(dot(vIn, norm)), 0.0001f, 1.0f);
    float LdotN = clampf(fabsf(dot(vOut, norm)), 0.0001f, 1.0f);
    float NdotH = fabsf(dot(norm, H));
    float VdotH = fabsf(dot(vIn, H));
    float LdotH = fabsf(dot(vOut, H));
    float P = pow5(clamp01(1.0f - VdotH));
    float out[3];
    if (kind == 0) {
        float k = kPi / LdotN / p;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float F0 = lerpf(0.04f, color[i], metal);
            float F = lerpf(P, 1.0f, F0);
            float cd = (1.0f - metal) * color[i];
            out[i] = k * ((1.0f - F) * cd / kPi);
        }
    } else {
        float G = smith_g2(smith_g1(VdotN, alpha), smith_g1(LdotN, alpha));
        float k = 4.0f * LdotH * VdotN / NdotH / LdotN / (kind == 1 ? (1.0f - p) : p);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float F0 = lerpf(0.04f, color[i], metal);
            float F = lerpf(P, 1.0f, F0);
            float fs = clampf(0.25f * (kind == 2 ? 1.0f - F : F) * G / (VdotN * LdotN), 0.0f, kFltMax);
            out[i] = k * fs;
        }
    }
    return v3(out[0], out[1], out[2]);
}

// BSDFModel::evaluateDirect (BRDFModel.h:211-261)
__device__ __forceinline__ V3 bsdf_eval_direct(V3 I, V3 O, V3 N, const float* color, float metal, float alpha)
{
    float VdotN = -dot(I, N);
    float LdotN = dot(O, N);
    if (!(VdotN > 0.0f && LdotN > 0.0f)) return v3(0.0f, 0.0f, 0.0f);
    V3 H = normalize(O - I);
    float VdotH = fabsf(dot(I, H));
    float NdotH = fabsf(dot(N, H));
    float P = pow5(clamp01(1.0f - VdotH));
    float D = ggx_pdf(clamp01(NdotH), alpha);
    float G = smith_g2(smith_g1(VdotN, alpha), smith_g1(LdotN, alpha));
    float out[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float F0 = lerpf(0.04f, color[i], metal);
        float F = lerpf(P, 1.0f, F0);
        float cd = (1.0f - metal) * color[i];
        float fd = (1.0f - F) * cd / kPi;
        float fs = clampf(0.25f * F * D * G / (VdotN * LdotN), 0.0f, kFltMax);
        out[i] = fd + fs;
    }
    return v3(out[0], out[1], out[2]);
}

// RandomSampler::GGXHemisphere / cosineSqrtHemisphere / uniformHemisphere (RandomSampler.h:66-103)
__device__ __forceinline__ V3 ggx_hemisphere(float alpha2, float uphi, float rnd)
{
    float phi = (2.0f * kPi) * uphi;
    float cth = sqrtf((1.f - rnd) / (1.f - (1.0f - alpha2) * rnd));
    float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
    float s, c;
    cr::sincos_cr(phi, s, c);
    return v3(sth * c, sth * s, cth);
}
__device__ __forceinline__ V3 cosine_hemisphere(float uphi, float rnd)
{
    float phi = (2.0f * kPi) * uphi;
    float sth = sqrtf(rnd);
    float s, c;
    cr::sincos_cr(phi, s, c);
    return v3(sth * c, sth * s, sqrtf(1.0f - rnd));
}
__device__ __forceinline__ V3 uniform_hemisphere(float uphi, float cth)
{
    float phi = (2.0f * kPi) * uphi;
    float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
    float s, c;
    cr::sincos_cr(phi, s, c);
    return v3(sth * c, sth * s, cth);
}
// transformToNormalSpace (BRDFModel.h:25-34)
__device__ __forceinline__ V3 to_basis(V3 b0, V3 b1, V3 b2, V3 c) { return b0 * c.x + b1 * c.y + b2 * c.z; }

__device__ __forceinline__ V3 reflect3(V3 I, V3 N)
{
    float w = 2.0f * dot(I, N);
    return I - N * w;
}
__device__ __forceinline__ bool refract3(V3 I, V3 N, float eta, V3& R)
{
    float NI = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - NI * NI);
    if (k < 0.0f) {
        R = -I;
        return false;
    }
    k = eta * NI + sqrtf(k);
    R = I * eta - N * k;
    return true;
}

// What bsdf_sample_indirect decided, for differentiating its weight with the
// sampled direction held fixed: the evaluate kind (-1: zero weight), half
// vector, branch probability and the normal it used.
struct SampleInfo {
    int kind;
    V3 H, N;
    float p;
};

// BSDFModel::sampleIndirect (BRDFModel.h:265-337) with the three uniforms
// (branch, phi, radial) supplied; returns the weight, writes the direction.
__device__ __forceinline__ V3 bsdf_sample_indirect(BsdfIn d, float u0, float u1, float u2, V3& O,
                                                   SampleInfo* info = nullptr)
{
    if (info) info->kind = -1;
    float VdotN = -dot(d.I, d.N);
    V3 binorm = cross(d.N, d.T);
    V3 b0 = d.T, b1 = binorm;
    O = v3(0.0f, 0.0f, 0.0f);
    if (VdotN < 0.0f) {
        if (d.transmissive) {
            b0 = binorm;
            b1 = d.T;
            d.N = -d.N;
        } else {
            return v3(0.0f, 0.0f, 0.0f);
        }
    }
    const float p = 0.8f * fabsf(VdotN) + 0.1f;
    if (u0 < p) {
        if (u0 < p * (1.0f - d.color[3])) {
            float eta = VdotN < 0.0f ? 1.0f / d.eta : d.eta;
            V3 H = normalize(to_basis(b0, b1, d.N, ggx_hemisphere(d.alpha * d.alpha, u1, u2)));
            if (refract3(d.I, H, eta, O) && dot(d.N, O) < 0.0f) {
                O = normalize(O);
                if (info) *info = SampleInfo{2, H, d.N, p};
                return bsdf_evaluate(d.I, O, d.N, d.color, d.metal, d.alpha, 2, H, p);
            }
            return v3(0.0f, 0.0f, 0.0f);
        }
        O = normalize(to_basis(b0, b1, d.N, cosine_hemisphere(u1, u2)));
        if (info) *info = SampleInfo{0, O, d.N, p};
        return bsdf_evaluate(d.I, O, d.N, d.color, d.metal, d.alpha, 0, O, p);
    }
    V3 H = normalize(to_basis(b0, b1, d.N, ggx_hemisphere(d.alpha * d.alpha, u1, u2)));
    O = reflect3(d.I, H);
    if (dot(d.N, O) > 0.0f) {
        O = normalize(O);
        if (info) *info = SampleInfo{1, H, d.N, p};
        return bsdf_evaluate(d.I, O, d.N, d.color, d.metal, d.alpha, 1, H, p);
    }
    return v3(0.0f, 0.0f, 0.0f);
}

// ---------------------------------------------------- OpenMATERIAL ---
struct Cf {
    float re, im;
};
__device__ __forceinline__ Cf cmul(Cf a, Cf b) { return Cf{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Cf cdiv(Cf a, Cf b)
{
    // Smith's algorithm (R. L. Smith, "Algorithm 116: Complex division", CACM 1962)
    if (fabsf(b.re) >= fabsf(b.im)) {
        float r = b.im / b.re, den = b.re + b.im * r;
        return Cf{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
    }
    float r = b.re / b.im, den = b.re * r + b.im;
    return Cf{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
}
// principal square root, branch cut on the negative real axis
__device__ __forceinline__ Cf csqrt(Cf z)
{
    float m = hypotf(z.re, z.im);
    if (m == 0.0f) return Cf{0.0f, z.im};
    float t = sqrtf(0.5f * (m + fabsf(z.re)));
    if (z.re >= 0.0f) return Cf{t, 0.5f * z.im / t};
    return Cf{0.5f * fabsf(z.im) / t, copysignf(t, z.im)};
}

// fresnelReflection (OpenMaterial.cpp:20-38), then lerp(P,S,0.5)/|cos| (:147-155)
__device__ __forceinline__ float om_channel(float n, float k, float cosTheta)
{
    Cf N{n, k};
    Cf N2 = cmul(N, N);
    float c = fabsf(cosTheta);
    float s2 = 1.0f - c * c;
    Cf root = csqrt(Cf{N2.re - s2, N2.im});
    Cf N2c{N2.re * c, N2.im * c};
    Cf rp = cdiv(Cf{N2c.re - root.re, N2c.im - root.im}, Cf{N2c.re + root.re, N2c.im + root.im});
    Cf rs = cdiv(Cf{c - root.re, -root.im}, Cf{c + root.re, root.im});
    float P = rp.re * rp.re + rp.im * rp.im;
    float S = rs.re * rs.re + rs.im * rs.im;
    return lerpf(P, S, 0.5f) / fabsf(cosTheta);
}

// Density of the reflection branches of bsdf_sample_indirect at direction O and
// the integrand they estimate: sum over branches b of P_b w_b(O) |N.O| pdf_b(O),
// w_b the branch's weight (bsdf_evaluate).  A direction another strategy
// samples then carries the same expected contribution as the sampler's own
// (the MIS estimator's environment connection).  Diffuse: cosine hemisphere,
// P = p color.a; specular: GGX half vector with alpha^2 = (alpha)^2 reflected,
// pdf D(H) (N.H) / (4 |O.H|), P = 1 - p.  Transmission is not covered (zero).
__device__ __forceinline__ float bsdf_reflection_mix(BsdfIn d, V3 O, float ct, V3& feff)
{
    feff = v3(0.0f, 0.0f, 0.0f);
    const float VdotN = -dot(d.I, d.N);
    if (VdotN < 0.0f) {
        if (!d.transmissive) return 0.0f;
        d.N = -d.N;
    }
    const float cosO = dot(d.N, O);
    if (!(cosO > 0.0f)) return 0.0f;
    const float p = 0.8f * fabsf(VdotN) + 0.1f;
    const float Pd = p * d.color[3], Ps = 1.0f - p;
    const float pdf_d = cosO / kPi;
    float pdf_s = 0.0f;
    // the sampler reflects I about H and normalises, so the half vector of O is
    // taken with the unit incoming direction (camera rays need not be unit)
    const V3 H = normalize(O - normalize(d.I));
    const float NdotH = dot(d.N, H);
    if (NdotH > 0.0f) {
        const float a2 = d.alpha * d.alpha;
        const float den = 1.0f + (a2 - 1.0f) * NdotH * NdotH;
        const float D = a2 / (kPi * den * den);
        const float OdotH = fabsf(dot(O, H));
        if (OdotH > 0.0f) pdf_s = D * NdotH / (4.0f * OdotH);
    }
    const float pdf = Pd * pdf_d + Ps * pdf_s;
    if (!(pdf > 0.0f)) return 0.0f;
    if (Pd > 0.0f) feff = feff + bsdf_evaluate(d.I, O, d.N, d.color, d.metal, d.alpha, 0, O, p) * (Pd * pdf_d);
    if (pdf_s > 0.0f) feff = feff + bsdf_evaluate(d.I, O, d.N, d.color, d.metal, d.alpha, 1, H, p) * (Ps * pdf_s);
    feff = feff * ct;
    return pdf;
}

// ------------------------------------------------------ environment ---
// HDRBackground::getRadiance (HdrBackground.cpp:55-97)
__device__ __forceinline__ V3 env_radiance(const DevEnv& e, V3 dir)
{
    const float* R = e.rot;
    V3 rd = v3(R[0] * dir.x + R[3] * dir.y + R[6] * dir.z, R[1] * dir.x + R[4] * dir.y + R[7] * dir.z,
               R[2] * dir.x + R[5] * dir.y + R[8] * dir.z);
    V3 rxy = normalize(v3(rd.x, rd.y, 0.0f));
    float xang = cr::acos_cr(clampf(rxy.x, -1.0f, 1.0f));
    xang = rxy.y < 0.0f ? 2.0f * kPi - xang : xang;
    float yang = cr::asin_cr(clampf(rd.z, -1.0f, 1.0f)) + 0.5f * kPi;
    float u = xang / (2.0f * kPi);
    float v = 1.0f - yang / kPi;
    const int W = e.width, H = e.height;
    u -= floorf(u - e.half_u);
    v -= floorf(v - e.half_v);
    u *= e.fwidth;
    v *= e.fheight;
    int iu = (int)u, iv = (int)v;
    float kui = u - (float)iu, kvi = v - (float)iv;
    float ku = 1.0f - kui, kv = 1.0f - kvi;
    // u is in [0, 1] here (an angle over 2 pi), so iu is in [0, W]: the
    // reference's iu % W and (iu + 1) % W by one conditional subtraction
    const int l = iu >= W ? iu - W : iu, r = iu + 1 >= W ? iu + 1 - W : iu + 1;
    const int b = iv >= H ? iv - H : iv, t = iv + 1 >= H ? iv + 1 - H : iv + 1;
    float4 c0 = __ldg(e.rgb + b * W + l), c1 = __ldg(e.rgb + b * W + r);
    float4 c2 = __ldg(e.rgb + t * W + l), c3 = __ldg(e.rgb + t * W + r);
    float w0 = ku * kv, w1 = kui * kv, w2 = ku * kvi, w3 = kui * kvi;
    V3 val = v3(c0.x * w0 + c1.x * w1 + c2.x * w2 + c3.x * w3, c0.y * w0 + c1.y * w1 + c2.y * w2 + c3.y * w3,
                c0.z * w0 + c1.z * w1 + c2.z * w2 + c3.z * w3);
    return val * e.scale;
}

// lookup coordinates of a world direction (the first half of env_radiance)
__device__ __forceinline__ void env_uv(const DevEnv& e, V3 dir, float& u, float& v)
{
    const float* R = e.rot;
    V3 rd = v3(R[0] * dir.x + R[3] * dir.y + R[6] * dir.z, R[1] * dir.x + R[4] * dir.y + R[7] * dir.z,
               R[2] * dir.x + R[5] * dir.y + R[8] * dir.z);
    V3 rxy = normalize(v3(rd.x, rd.y, 0.0f));
    float xang = cr::acos_cr(clampf(rxy.x, -1.0f, 1.0f));
    xang = rxy.y < 0.0f ? 2.0f * kPi - xang : xang;
    float yang = cr::asin_cr(clampf(rd.z, -1.0f, 1.0f)) + 0.5f * kPi;
    u = xang / (2.0f * kPi);
    v = 1.0f - yang / kPi;
}

// density per steradian with which env_sample draws `dir`
__device__ __forceinline__ float env_pdf(const DevEnv& e, V3 dir)
{
    if (e.smp.cells <= 0) return 0.0f;
    float u, v;
    env_uv(e, dir, u, v);
    const int i = min(max((int)(u * e.fwidth), 0), e.width - 1);
    const int j = min(max((int)(v * e.fheight), 0), e.height - 1);
    return __ldg(e.smp.pdf + (size_t)j * e.width + i);
}

// a direction from the environment's alias table (u0: cell, u1: alias
// choice, u2/u3: position in the cell, uniform in solid angle); returns its
// density per steradian (0: nothing to sample)
__device__ __forceinline__ float env_sample(const DevEnv& e, float u0, float u1, float u2, float u3, V3& dir)
{
    const int n = e.smp.cells;
    if (n <= 0) return 0.0f;
    int c = min((int)(u0 * (float)n), n - 1);
    if (!(u1 < __ldg(e.smp.prob + c))) c = (int)__ldg(e.smp.alias + c);
    const float pdf = __ldg(e.smp.pdf + c);
    if (!(pdf > 0.0f)) return 0.0f;
    const int i = c % e.width, j = c / e.width;
    const float u = ((float)i + u2) / (float)e.width;
    const float c0 = cospif((float)j / (float)e.height), c1 = cospif((float)(j + 1) / (float)e.height);
    const float z = c0 - u3 * (c0 - c1);  // cos(pi v), uniform in solid angle over the cell's rows
    const float sxy = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float sn, cs;
    sincospif(2.0f * u, &sn, &cs);
    const V3 rd = v3(sxy * cs, sxy * sn, z);
    const float* R = e.rot;  // rd = dir R, R a rotation: dir = R rd
    dir = normalize(v3(R[0] * rd.x + R[1] * rd.y + R[2] * rd.z, R[3] * rd.x + R[4] * rd.y + R[5] * rd.z,
                       R[6] * rd.x + R[7] * rd.y + R[8] * rd.z));
    return pdf;
}

}  // namespace omv
