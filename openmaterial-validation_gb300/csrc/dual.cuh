// Forward-mode derivatives of the material functions with respect to their
// parameters, for the path-replay adjoint.  A Dual<K> carries a value and its
// derivatives with respect to K parameters; the functions below restate the
// BRDF and Fresnel code of omv_device.cuh (same formulas and operation order
// for the value part) on duals.
#pragma once

#include "omv_device.cuh"

namespace omv {

template <int K>
struct Dual {
    float v;
    float d[K];
};

template <int K>
__device__ __forceinline__ Dual<K> dconst(float v)
{
    Dual<K> r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = 0.0f;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dvar(float v, int i)
{
    Dual<K> r = dconst<K>(v);
    r.d[i] = 1.0f;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(Dual<K> a, Dual<K> b)
{
    Dual<K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(Dual<K> a, Dual<K> b)
{
    Dual<K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(Dual<K> a)
{
    Dual<K> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(Dual<K> a, Dual<K> b)
{
    Dual<K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(Dual<K> a, float s)
{
    Dual<K> r;
    r.v = a.v * s;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = a.d[i] * s;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(float s, Dual<K> a)
{
    Dual<K> r;
    r.v = s * a.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = s * a.d[i];
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(Dual<K> a, Dual<K> b)
{
    Dual<K> r;
    r.v = a.v / b.v;
    const float ib = 1.0f / b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(Dual<K> a, float s)
{
    Dual<K> r;
    r.v = a.v / s;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = a.d[i] / s;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(float s, Dual<K> b)
{
    return dconst<K>(s) / b;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(Dual<K> a, float s)
{
    a.v = a.v + s;
    return a;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(float s, Dual<K> a)
{
    a.v = s + a.v;
    return a;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(Dual<K> a, float s)
{
    a.v = a.v - s;
    return a;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(float s, Dual<K> a)
{
    return dconst<K>(s) - a;
}
template <int K>
__device__ __forceinline__ Dual<K> dsqrt(Dual<K> a)
{
    Dual<K> r;
    r.v = sqrtf(a.v);
    const float g = r.v > 0.0f ? 0.5f / r.v : 0.0f;
#pragma unroll
    for (int i = 0; i < K; ++i) r.d[i] = a.d[i] * g;
    return r;
}
template <int K>
__device__ __forceinline__ Dual<K> dabs(Dual<K> a)
{
    return a.v < 0.0f ? -a : a;
}
// clamp: the derivative is zero where the value is clamped
template <int K>
__device__ __forceinline__ Dual<K> dclamp(Dual<K> a, float lo, float hi)
{
    if (a.v < lo) return dconst<K>(lo);
    if (a.v > hi) return dconst<K>(hi);
    return a;
}
// lerp(lo, up, v) = (up - lo) * v + lo, as lerpf
template <int K>
__device__ __forceinline__ Dual<K> dlerp(Dual<K> lo, Dual<K> up, Dual<K> v)
{
    return (up - lo) * v + lo;
}

// ----------------------------------------------------------- GGX / Smith ---
template <int K>
__device__ __forceinline__ Dual<K> d_ggx_pdf(float c, Dual<K> alpha)
{
    const float c2 = c * c;
    const Dual<K> a2 = alpha * alpha;
    const Dual<K> l = dlerp(dconst<K>(1.0f), a2, dconst<K>(c2));
    return a2 / ((l * l) * kPi);
}
template <int K>
__device__ __forceinline__ Dual<K> d_smith_g1(float c, Dual<K> alpha)
{
    if (!(alpha.v > 0.0f || c < 0.99f)) return dconst<K>(1.0f);
    const float s = sqrtf(1.0f - c * c);
    if (!(s > 0.0f)) return dconst<K>(1.0f);  // c = 1: the float code's limit (a infinite, G1 = 1)
    const Dual<K> a = c / (alpha * s);
    const Dual<K> lam = (dsqrt(1.0f + 1.0f / (a * a)) - 1.0f) * 0.5f;
    return 1.0f / (1.0f + lam);
}
template <int K>
__device__ __forceinline__ Dual<K> d_smith_g2(Dual<K> s, Dual<K> m)
{
    const Dual<K> p = s * m;
    return p / (s + m - p);
}

// PBR parameters as duals: colour r,g,b (0-2), GGX alpha (3), metallic (4)
struct PbrDual {
    Dual<5> color[3];
    Dual<5> alpha, metal;
};
__device__ __forceinline__ PbrDual pbr_dual(const float* color, float alpha, float metal)
{
    PbrDual m;
#pragma unroll
    for (int i = 0; i < 3; ++i) m.color[i] = dvar<5>(color[i], i);
    m.alpha = dvar<5>(alpha, 3);
    m.metal = dvar<5>(metal, 4);
    return m;
}

// bsdf_evaluate on duals (directions fixed)
__device__ __forceinline__ void d_bsdf_evaluate(V3 vIn, V3 vOut, V3 norm, const PbrDual& m, int kind, V3 Hext,
                                                float p, Dual<5> out[3])
{
    const V3 H = kind == 2 ? Hext : normalize(vOut - vIn);
    const float VdotN = clampf(fabsf(dot(vIn, norm)), 0.0001f, 1.0f);
    const float LdotN = clampf(fabsf(dot(vOut, norm)), 0.0001f, 1.0f);
    const float NdotH = fabsf(dot(norm, H));
    const float VdotH = fabsf(dot(vIn, H));
    const float LdotH = fabsf(dot(vOut, H));
    const float P = pow5(clamp01(1.0f - VdotH));
    if (kind == 0) {
        const float k = kPi / LdotN / p;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const Dual<5> F0 = dlerp(dconst<5>(0.04f), m.color[i], m.metal);
            const Dual<5> F = dlerp(dconst<5>(P), dconst<5>(1.0f), F0);
            const Dual<5> cd = (1.0f - m.metal) * m.color[i];
            out[i] = ((1.0f - F) * cd / kPi) * k;
        }
    } else {
        const Dual<5> G = d_smith_g2(d_smith_g1(VdotN, m.alpha), d_smith_g1(LdotN, m.alpha));
        const float k = 4.0f * LdotH * VdotN / NdotH / LdotN / (kind == 1 ? (1.0f - p) : p);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const Dual<5> F0 = dlerp(dconst<5>(0.04f), m.color[i], m.metal);
            const Dual<5> F = dlerp(dconst<5>(P), dconst<5>(1.0f), F0);
            const Dual<5> fs = dclamp((0.25f * (kind == 2 ? 1.0f - F : F) * G) / (VdotN * LdotN), 0.0f, kFltMax);
            out[i] = fs * k;
        }
    }
}

// bsdf_eval_direct on duals
__device__ __forceinline__ void d_bsdf_eval_direct(V3 I, V3 O, V3 N, const PbrDual& m, Dual<5> out[3])
{
    const float VdotN = -dot(I, N);
    const float LdotN = dot(O, N);
    if (!(VdotN > 0.0f && LdotN > 0.0f)) {
#pragma unroll
        for (int i = 0; i < 3; ++i) out[i] = dconst<5>(0.0f);
        return;
    }
    const V3 H = normalize(O - I);
    const float VdotH = fabsf(dot(I, H));
    const float NdotH = fabsf(dot(N, H));
    const float P = pow5(clamp01(1.0f - VdotH));
    const Dual<5> D = d_ggx_pdf(clamp01(NdotH), m.alpha);
    const Dual<5> G = d_smith_g2(d_smith_g1(VdotN, m.alpha), d_smith_g1(LdotN, m.alpha));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const Dual<5> F0 = dlerp(dconst<5>(0.04f), m.color[i], m.metal);
        const Dual<5> F = dlerp(dconst<5>(P), dconst<5>(1.0f), F0);
        const Dual<5> cd = (1.0f - m.metal) * m.color[i];
        const Dual<5> fd = (1.0f - F) * cd / kPi;
        const Dual<5> fs = dclamp((0.25f * F * D * G) / (VdotN * LdotN), 0.0f, kFltMax);
        out[i] = fd + fs;
    }
}

// d/dalpha of log D_alpha(c) for the GGX half-vector density the sampler draws
// from (RandomSampler::GGXHemisphere): the score of a GGX-sampled direction
__device__ __forceinline__ float ggx_log_pdf_dalpha(float c, float alpha)
{
    const float c2 = c * c, a2 = alpha * alpha;
    const float l = (a2 - 1.0f) * c2 + 1.0f;
    return 2.0f / alpha - 4.0f * alpha * c2 / l;
}

// --------------------------------------------------- OpenMATERIAL Fresnel ---
struct DC {
    Dual<2> re, im;
};
__device__ __forceinline__ DC dcmul(DC a, DC b) { return DC{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ DC dcdiv(DC a, DC b)
{
    if (fabsf(b.re.v) >= fabsf(b.im.v)) {
        const Dual<2> r = b.im / b.re, den = b.re + b.im * r;
        return DC{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
    }
    const Dual<2> r = b.re / b.im, den = b.re * r + b.im;
    return DC{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
}
__device__ __forceinline__ DC dcsqrt(DC z)
{
    const Dual<2> m = dsqrt(z.re * z.re + z.im * z.im);
    if (m.v == 0.0f) return DC{dconst<2>(0.0f), z.im};
    const Dual<2> t = dsqrt((m + dabs(z.re)) * 0.5f);
    if (z.re.v >= 0.0f) return DC{t, (z.im * 0.5f) / t};
    return DC{(dabs(z.im) * 0.5f) / t, z.im.v < 0.0f ? -t : t};
}
// om_channel with n (slot 0) and k (slot 1) as duals
__device__ __forceinline__ Dual<2> d_om_channel(float n, float k, float cosTheta)
{
    const DC N{dvar<2>(n, 0), dvar<2>(k, 1)};
    const DC N2 = dcmul(N, N);
    const float c = fabsf(cosTheta);
    const float s2 = 1.0f - c * c;
    const DC root = dcsqrt(DC{N2.re - s2, N2.im});
    const DC N2c{N2.re * c, N2.im * c};
    const DC rp = dcdiv(DC{N2c.re - root.re, N2c.im - root.im}, DC{N2c.re + root.re, N2c.im + root.im});
    const DC rs = dcdiv(DC{c - root.re, -root.im}, DC{c + root.re, root.im});
    const Dual<2> P = rp.re * rp.re + rp.im * rp.im;
    const Dual<2> S = rs.re * rs.re + rs.im * rs.im;
    return dlerp(P, S, dconst<2>(0.5f)) / fabsf(cosTheta);
}

}  // namespace omv
