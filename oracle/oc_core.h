/*
 * ORACLE -- test infrastructure only.  CPU restatement of the reference
 * renderer's hot path (LudwigFriedmann/OpenMATERIAL-Validation, pathtracer/src).
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this code, as the checker / the timed CPU reference; the product never links it.
 *
 * Every helper below restates a reference function with the SAME floating-point
 * operation order, so that, compiled without FMA contraction
 * (-ffp-contract=off), the oracle reproduces the reference bit for bit:
 *   dot3/cross3/length3/normalize3/normalizeIfNeeded3  UtilityFunctions.h:128-238
 *   multVector3 (3 overloads)                           UtilityFunctions.h:286-307
 *   inverseMatrix3 / detMatrix3                         UtilityFunctions.h:334-349
 *   reflect3 / refract3                                 UtilityFunctions.h:473-495
 *   clamp/min/max/lerp/linearFunction                   UtilityFunctions.h:430-469
 */
#ifndef OMV_ORACLE_CORE_H
#define OMV_ORACLE_CORE_H

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#define OC_PI 3.14159265358979323846f /* M_PIf, Constants.h:20 */
#define OC_EPS FLT_EPSILON            /* fEpsilon, Constants.h:30 */

static inline float oc_min(float a, float b) { return a < b ? a : b; }
static inline float oc_max(float a, float b) { return a > b ? a : b; }
static inline float oc_clamp(float v, float lo, float hi) { return oc_max(lo, oc_min(v, hi)); }
static inline float oc_clamp01(float v) { return oc_clamp(v, 0.0f, 1.0f); }
/* linearFunction(k, c, x) = k*x + c */
static inline float oc_linf(float k, float c, float x) { return k * x + c; }
/* lerp(lower, upper, value) = linearFunction(upper-lower, lower, value) */
static inline float oc_lerp(float lo, float up, float v) { return oc_linf(up - lo, lo, v); }

static inline float oc_dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void oc_cross3(const float* a, const float* b, float* r)
{
    float r0 = a[1] * b[2] - a[2] * b[1];
    float r1 = a[2] * b[0] - a[0] * b[2];
    float r2 = a[0] * b[1] - a[1] * b[0];
    r[0] = r0; r[1] = r1; r[2] = r2;
}
static inline float oc_length3(const float* a) { return sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
static inline float oc_distance3(const float* a, const float* b)
{
    float c[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    return oc_length3(c);
}
static inline float oc_sqdistance3(const float* a, const float* b)
{
    float c[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    return oc_dot3(c, c);
}
static inline void oc_normalize3(float* a)
{
    float L = oc_length3(a);
    if (L != 0.0f) {
        L = 1.0f / L;
        a[0] = a[0] * L; a[1] = a[1] * L; a[2] = a[2] * L;
    } else {
        a[0] = 1.0f; a[1] = 0.0f; a[2] = 0.0f;
    }
}
static inline void oc_normalize_if_needed3_to(const float* a, float* r)
{
    const float eps = 10.0f * FLT_EPSILON;
    float sL = oc_dot3(a, a);
    if (sL < 1.0f + eps && sL > 1.0f - eps) {
        r[0] = a[0]; r[1] = a[1]; r[2] = a[2];
        return;
    }
    float L = sqrtf(sL);
    if (L != 0.0f) {
        L = 1.0f / L;
        float x = a[0] * L, y = a[1] * L, z = a[2] * L;
        r[0] = x; r[1] = y; r[2] = z;
    } else {
        r[0] = 1.0f; r[1] = 0.0f; r[2] = 0.0f;
    }
}
static inline void oc_normalize_if_needed3(float* a) { oc_normalize_if_needed3_to(a, a); }

/* multVector3(const T A[][4], V, R): affine point transform */
static inline void oc_xform_point(const float A[4][4], const float* V, float* R)
{
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = A[i][0] * V[0] + A[i][1] * V[1] + A[i][2] * V[2] + A[i][3];
    R[0] = r[0]; R[1] = r[1]; R[2] = r[2];
}
/* multVector3(const T A[][3], V, R) */
static inline void oc_mat3_vec(const float A[3][3], const float* V, float* R)
{
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = A[i][0] * V[0] + A[i][1] * V[1] + A[i][2] * V[2];
    R[0] = r[0]; R[1] = r[1]; R[2] = r[2];
}
/* multVector3(const T V[], const T A[][3], R) */
static inline void oc_vec_mat3(const float* V, const float A[3][3], float* R)
{
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = A[0][i] * V[0] + A[1][i] * V[1] + A[2][i] * V[2];
    R[0] = r[0]; R[1] = r[1]; R[2] = r[2];
}

static inline float oc_det3(const float M[3][3])
{
    return M[0][0] * M[1][1] * M[2][2] + M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
           M[0][2] * M[1][1] * M[2][0] - M[0][1] * M[1][0] * M[2][2] - M[0][0] * M[1][2] * M[2][1];
}
/* inverseMatrix3: k = 1.0 / det is evaluated in double (double literal) */
static inline void oc_inverse3(const float M[3][3], float R[3][3])
{
    float k = (float)(1.0 / (double)oc_det3(M));
    R[0][0] = k * (M[1][1] * M[2][2] - M[1][2] * M[2][1]);
    R[0][1] = k * (-M[0][1] * M[2][2] + M[0][2] * M[2][1]);
    R[0][2] = k * (M[0][1] * M[1][2] - M[0][2] * M[1][1]);
    R[1][0] = k * (-M[1][0] * M[2][2] + M[1][2] * M[2][0]);
    R[1][1] = k * (M[0][0] * M[2][2] - M[0][2] * M[2][0]);
    R[1][2] = k * (-M[0][0] * M[1][2] + M[0][2] * M[1][0]);
    R[2][0] = k * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    R[2][1] = k * (-M[0][0] * M[2][1] + M[0][1] * M[2][0]);
    R[2][2] = k * (M[0][0] * M[1][1] - M[0][1] * M[1][0]);
}

static inline void oc_reflect3(const float* I, const float* N, float* O)
{
    const float w = 2.0f * oc_dot3(I, N);
    float o[3];
    for (int i = 0; i < 3; ++i) o[i] = I[i] - w * N[i];
    O[0] = o[0]; O[1] = o[1]; O[2] = o[2];
}
static inline int oc_refract3(const float* I, const float* N, float eta, float* R)
{
    float N_I = oc_dot3(N, I);
    float k = 1.0f - eta * eta * (1.0f - N_I * N_I);
    if (k < 0.0f) {
        R[0] = -I[0]; R[1] = -I[1]; R[2] = -I[2];
        return 0;
    }
    k = eta * N_I + sqrtf(k);
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = eta * I[i] - k * N[i];
    R[0] = r[0]; R[1] = r[1]; R[2] = r[2];
    return 1;
}

/* transformToNormalSpace (BRDFModel.h:25-34): R = b0*c0 + R, then b1*c1 + R, b2*c2 + R */
static inline void oc_to_normal_space(const float* b0, const float* b1, const float* b2, const float* c, float* R)
{
    float r[3] = {0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 3; ++i) r[i] = oc_linf(b0[i], r[i], c[0]);
    for (int i = 0; i < 3; ++i) r[i] = oc_linf(b1[i], r[i], c[1]);
    for (int i = 0; i < 3; ++i) r[i] = oc_linf(b2[i], r[i], c[2]);
    R[0] = r[0]; R[1] = r[1]; R[2] = r[2];
}

/* BDPTRenderer::maxAbsInVector (BDPTRenderer.cpp:35-40) */
static inline float oc_max_abs(const float* v, float th)
{
    float a0 = fabsf(v[0]), a1 = fabsf(v[1]), a2 = fabsf(v[2]);
    float mv = a0 > a1 && a0 > a2 ? a0 : a1 > a2 ? a1 : a2;
    return mv < th ? th : mv;
}
/* BDPTRenderer::intensity (BDPTRenderer.cpp:52-55) */
static inline float oc_intensity(const float* r) { return 0.299f * r[0] + 0.587f * r[1] + 0.114f * r[2]; }

/* ------------------------------------------------------------------ RNG --- */
/* std::mt19937 (Matsumoto & Nishimura 1998) + libstdc++'s
 * uniform_real_distribution<float>(0,1): generate_canonical<float,24> takes one
 * 32-bit draw, r = float(x) / 2^32, clamped below 1 (RandomSampler.h:38-60). */
typedef struct oc_mt {
    uint32_t s[624];
    int idx;
} oc_mt;

static inline void oc_mt_seed(oc_mt* m, uint32_t seed)
{
    m->s[0] = seed;
    for (uint32_t i = 1; i < 624; ++i) m->s[i] = 1812433253u * (m->s[i - 1] ^ (m->s[i - 1] >> 30)) + i;
    m->idx = 624;
}
static inline uint32_t oc_mt_next(oc_mt* m)
{
    if (m->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            uint32_t y = (m->s[i] & 0x80000000u) | (m->s[(i + 1) % 624] & 0x7fffffffu);
            m->s[i] = m->s[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        m->idx = 0;
    }
    uint32_t y = m->s[m->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}
static inline float oc_mt_uniform(oc_mt* m)
{
    float sum = (float)oc_mt_next(m) * 1.0f;
    float r = sum / 4294967296.0f;
    if (r >= 1.0f) r = nextafterf(1.0f, 0.0f);
    return r * (1.0f - 0.0f) + 0.0f;
}

#endif
