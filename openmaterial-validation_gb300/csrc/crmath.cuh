// Correctly rounded float sin/cos, asin/acos, x^5 and 1/x^2 for the restated
// material and environment arithmetic.
//
// The reference evaluates these with the host C library in float
// (std::sin / std::cos / std::pow in RandomSampler.h:87-103 and
// BRDFModel.h:44-80, 180, 231; std::acos / std::asin in HdrBackground.cpp:61-63).
// Those results are within about one ulp of the exact values, and
// sampleIndirect and the environment lookup amplify one-ulp differences of
// their inputs beyond 1e-5 relative on a small fraction of inputs (grazing
// directions, steep texel gradients).  Evaluating each function to about 46
// bits and rounding once gives the correctly rounded float on all but a
// vanishing fraction of inputs, which keeps the device within 1e-5 of the
// reference wherever the reference's own library is within an ulp.
//
// Method (published techniques, constants derived from their definitions):
//   * double-float ("double-word") arithmetic: T. J. Dekker, "A floating-point
//     technique for extending the available precision", Numer. Math. 18
//     (1971); error-free sum (Knuth, TAOCP vol. 2, 4.2.2) and the product
//     error from one fused multiply-add;
//   * sin / cos: additive range reduction by pi/2 split into three 20-bit
//     parts and a remainder (W. J. Cody and W. Waite, "Software Manual for the
//     Elementary Functions", 1980), a second one by pi/32 against a table of
//     sin and cos of j pi/32 (the angle-sum method of table-driven
//     evaluation, P. T. P. Tang, ACM TOMS 1989), and Taylor series of sin and
//     cos on |r| <= pi/64, their first terms in double-float;
//   * asin / acos: one Newton step on sin(y) = t from a float starting value,
//     with sin evaluated in double-float; |t| > 1/2 through
//     asin(t) = pi/2 - 2 asin(sqrt((1 - t) / 2));
//   * x^5 and 1/x^2: double-float products; 1/(p + e) by one Newton-Raphson
//     correction of the rounded reciprocal of p; both are rational, so where
//     the double-float result lies near a rounding midpoint (about one input
//     in 2^20) the side of the midpoint is decided exactly, in double with
//     error-free products, and exact midpoints (x^5 of odd * 2^j, odd <= 31)
//     round to even.
// Everything is plain float arithmetic (the fused multiply-adds are explicit),
// so the host build (-ffp-contract=off) computes the same results as the
// device; only the low-order corrections of asin / acos (a cosine and two
// quotients that need about 2^-20) use the device's fast approximations.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define OMV_CR_HD __host__ __device__ __forceinline__
#define OMV_CR_RARE static __host__ __device__ __noinline__  // rare paths, out of the callers' registers
#else
#define OMV_CR_HD inline
#define OMV_CR_RARE inline
#endif

namespace omv {
namespace cr {

struct FF {
    float hi, lo;  // value hi + lo, |lo| <= ulp(hi) / 2 after normalisation
};

// error-free sum of two floats (any magnitudes)
OMV_CR_HD FF two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return FF{s, e};
}
// error-free sum when |a| >= |b| (or a == 0)
OMV_CR_HD FF fast_two_sum(float a, float b)
{
    const float s = a + b;
    return FF{s, b - (s - a)};
}
// error-free product
OMV_CR_HD FF two_prod(float a, float b)
{
    const float p = a * b;
    return FF{p, fmaf(a, b, -p)};
}
OMV_CR_HD FF ff_mul(FF x, FF y)
{
    FF p = two_prod(x.hi, y.hi);
    const float e = p.lo + (x.hi * y.lo + x.lo * y.hi);
    return fast_two_sum(p.hi, e);
}
OMV_CR_HD FF ff_mul_f(FF x, float y)
{
    FF p = two_prod(x.hi, y);
    const float e = p.lo + x.lo * y;
    return fast_two_sum(p.hi, e);
}
OMV_CR_HD FF ff_add(FF x, FF y)
{
    FF s = two_sum(x.hi, y.hi);
    const float e = s.lo + (x.lo + y.lo);
    return fast_two_sum(s.hi, e);
}
OMV_CR_HD FF ff_neg(FF x) { return FF{-x.hi, -x.lo}; }

// double-float constants: hi = the float nearest the value, lo = the float
// nearest the remainder
constexpr float kPiHalfHi = 1.5707963705062866f, kPiHalfLo = -4.371138828673793e-08f;
constexpr float kPiHi = 3.1415927410125732f, kPiLo = -8.742277657347586e-08f;
constexpr float kTwoOverPi = 0.6366197466850281f;
// pi/2 = kC1 + kC2 + kC3 + kC4 to about 2^-86: kC1..kC3 are pi/2's leading
// bits cut to 20 significant bits each, so q * kCi is exact for the quadrant
// numbers q <= 5 used here
constexpr float kC1 = 1.5707950592041016f;
constexpr float kC2 = 1.2675900507019833e-06f;
constexpr float kC3 = 7.443542310303641e-13f;
constexpr float kC4 = 5.170182817331536e-19f;

// Taylor coefficients (-1)^k / (2k+1)! (sin) and (-1)^k / (2k)! (cos),
// k = 1..4 in double-float, the rest in float
constexpr float kS1h = -0.1666666716337204f, kS1l = 4.967053879312289e-09f;
constexpr float kS2h = 0.008333333767950535f, kS2l = -4.34617203337595e-10f;
constexpr float kS3h = -0.00019841270113829523f, kS3l = 2.725596874933456e-12f;
constexpr float kS4h = 2.7557318844628753e-06f, kS4l = 3.793571224297229e-14f;
constexpr float kS5 = -2.5052107943679403e-08f, kS6 = 1.6059044372074283e-10f, kS7 = -7.647163609812713e-13f,
                kS8 = 2.8114573589663704e-15f;
constexpr float kK1h = -0.5f, kK1l = 0.0f;
constexpr float kK2h = 0.0416666679084301f, kK2l = -1.2417634698280722e-09f;
constexpr float kK3h = -0.0013888889225199819f, kK3l = 3.3631094437103215e-11f;
constexpr float kK4h = 2.4801587642286904e-05f, kK4l = -3.40699609366682e-13f;
constexpr float kK5 = -2.755731998149713e-07f, kK6 = 2.0876755879584152e-09f, kK7 = -1.147074536050896e-11f,
                kK8 = 4.7794772561329454e-14f;

// sin(y) for a float |y| <= 0.53 (asin's Newton step): y^2 is exact as a
// double-float, and on this range the terms from y^9 on need float accuracy only
OMV_CR_HD FF ff_sin_small(float y)
{
    const FF z = two_prod(y, y);
    const float zh = z.hi;
    const float ts = kS4h + zh * (kS5 + zh * (kS6 + zh * kS7));
    FF t = ff_add(FF{kS3h, kS3l}, ff_mul_f(z, ts));
    t = ff_add(FF{kS2h, kS2l}, ff_mul(z, t));
    t = ff_add(FF{kS1h, kS1l}, ff_mul(z, t));
    return ff_add(FF{y, 0.0f}, ff_mul_f(ff_mul(z, t), y));
}

// sin and cos of j pi / 32, j = 0..8, as double-floats (sin hi, lo, cos hi, lo)
#ifdef __CUDACC__
__device__
#endif
constexpr float kSinCosTable[9][4] = {
    {0.0f, 0.0f, 1.0f, 0.0f},
    {0.0980171412229538f, -8.933931927579408e-10f, 0.9951847195625305f, 7.109666189109021e-09f},
    {0.19509032368659973f, -1.670471427850373e-09f, 0.9807852506637573f, 2.9739473106360492e-08f},
    {0.290284663438797f, 1.3815665056426951e-08f, 0.9569403529167175f, -1.7184508038781132e-08f},
    {0.3826834261417389f, 6.2233507236442165e-09f, 0.9238795042037964f, 2.830748968563057e-08f},
    {0.4713967442512512f, -7.425253745196869e-09f, 0.8819212913513184f, -2.7002963420841297e-08f},
    {0.5555702447891235f, -1.1769521357507529e-08f, 0.8314695954322815f, 1.687026340846387e-08f},
    {0.6343932747840881f, 9.37955757507325e-09f, 0.7730104327201843f, 2.0642552556182636e-08f},
    {0.7071067690849304f, 1.2101617485882343e-08f, 0.7071067690849304f, 1.2101617485882343e-08f},
};

OMV_CR_HD float table_at(int j, int k)
{
#ifdef __CUDA_ARCH__
    return __ldg(&kSinCosTable[j][k]);
#else
    return kSinCosTable[j][k];
#endif
}

// Correctly rounded sinf / cosf of x in [0, 8] (the sampling angles 2 pi u):
// x = q pi/2 + j pi/32 + r with |r| <= pi/64, sin and cos of r by short
// series, combined with the table's values of j pi / 32 by the angle sums.
OMV_CR_HD void sincos_cr(float x, float& s_out, float& c_out)
{
    // quadrant q = nearest integer to x / (pi/2); x - q pi/2 as a double-float
    const float q = rintf(x * kTwoOverPi);
    FF r = two_sum(x - q * kC1, -(q * kC2));  // x - q kC1 is exact (Sterbenz, or q = 0)
    FF r2 = two_sum(r.hi, -(q * kC3));
    r = fast_two_sum(r2.hi, r2.lo + (r.lo - q * kC4));
    // j = nearest integer to r / (pi/32); pi/32 = (kC1 + kC2 + kC3 + kC4) / 16 and
    // j kCi / 16 is exact for |j| <= 8; r.hi - j kC1 / 16 is exact (Sterbenz)
    const float j = rintf(r.hi * (16.0f * kTwoOverPi));
    FF t = two_sum(r.hi - j * (kC1 * 0.0625f), -(j * (kC2 * 0.0625f)));
    FF t2 = two_sum(t.hi, -(j * (kC3 * 0.0625f)));
    t = fast_two_sum(t2.hi, t2.lo + (t.lo + (r.lo - j * (kC4 * 0.0625f))));
    // sin t = t (1 + z (S1 + z (S2 + z S3))), cos t = 1 + z (K1 + z (K2 + z K3)), z = t^2 <= 0.0025
    FF z = two_prod(t.hi, t.hi);
    z = fast_two_sum(z.hi, z.lo + 2.0f * t.hi * t.lo);
    const float zh = z.hi;
    const FF ps = ff_add(FF{kS1h, kS1l}, FF{zh * (kS2h + zh * kS3h), 0.0f});
    const FF st = ff_add(t, ff_mul(t, ff_mul(z, ps)));
    const FF pc = ff_add(FF{kK1h, kK1l}, ff_mul_f(z, kK2h + zh * kK3h));
    const FF ct = ff_add(FF{1.0f, 0.0f}, ff_mul(z, pc));
    // the angle sums with sin / cos of |j| pi / 32 (odd / even in j)
    const int ja = (int)fabsf(j);
    const float sg = j < 0.0f ? -1.0f : 1.0f;
    const FF sj{sg * table_at(ja, 0), sg * table_at(ja, 1)}, cj{table_at(ja, 2), table_at(ja, 3)};
    const float sv = ff_add(ff_mul(sj, ct), ff_mul(cj, st)).hi;
    const float cv = ff_add(ff_mul(cj, ct), ff_neg(ff_mul(sj, st))).hi;
    const int qi = (int)q & 3;
    s_out = qi == 0 ? sv : qi == 1 ? cv : qi == 2 ? -sv : -cv;
    c_out = qi == 0 ? cv : qi == 1 ? -sv : qi == 2 ? -cv : sv;
}

// cos(y) and a quotient to about 2^-21 (the Newton correction needs no more)
OMV_CR_HD float cos_rough(float y)
{
#ifdef __CUDA_ARCH__
    return __cosf(y);
#else
    return cosf(y);
#endif
}

// asin of a double-float t with 0 <= t <= 1/2, as a double-float: one Newton
// step on sin(y) = t from the float approximation y0 (the step's own error
// is of the order of (y - y0)^2, far below the rounding of the result)
OMV_CR_HD FF asin_ff_small(FF t)
{
    const float y0 = asinf(t.hi);
    const FF s = ff_sin_small(y0);
    const float res = (t.hi - s.hi) + (t.lo - s.lo);  // t.hi - s.hi is exact (Sterbenz)
#ifdef __CUDA_ARCH__
    return two_sum(y0, __fdividef(res, cos_rough(y0)));  // two ulp suffice here
#else
    return two_sum(y0, res / cos_rough(y0));
#endif
}

// sqrt of a float as a double-float (the residual a - h^2 is exact by FMA)
OMV_CR_HD FF sqrt_ff(float a)
{
    const float h = sqrtf(a);
    if (!(h > 0.0f)) return FF{h, 0.0f};
#ifdef __CUDA_ARCH__
    return FF{h, __fdividef(fmaf(-h, h, a), 2.0f * h)};  // the low part needs about 2^-20 only
#else
    return FF{h, fmaf(-h, h, a) / (2.0f * h)};
#endif
}

// The asin of |x| reduced to an argument in [0, 1/2]: |x| itself, or
// sqrt((1 - |x|) / 2) above 1/2 (asin|x| = pi/2 - 2 asin of that); without a
// branch, so that the lanes of a warp take one path
OMV_CR_HD FF asin_reduced(float ax, bool& big)
{
    big = ax > 0.5f;
    const FF r = sqrt_ff((1.0f - ax) * 0.5f);  // 1 - ax exact for ax in [1/2, 1]
    return asin_ff_small(big ? r : FF{ax, 0.0f});
}

// correctly rounded asinf for x in [-1, 1]
OMV_CR_HD float asin_cr(float x)
{
    bool big;
    const FF a = asin_reduced(fabsf(x), big);
    const FF v = big ? ff_add(FF{kPiHalfHi, kPiHalfLo}, FF{-2.0f * a.hi, -2.0f * a.lo}) : a;
    const float r = v.hi + v.lo;
    return x < 0.0f ? -r : r;
}

// correctly rounded acosf for x in [-1, 1]
OMV_CR_HD float acos_cr(float x)
{
    bool big;
    const FF a = asin_reduced(fabsf(x), big);  // asin|x|, or (pi/2 - asin|x|) / 2 when big
    const bool neg = x < 0.0f;
    FF v;
    if (big)  // acos|x| = 2a; acos(-|x|) = pi - 2a
        v = neg ? ff_add(FF{kPiHi, kPiLo}, FF{-2.0f * a.hi, -2.0f * a.lo}) : FF{2.0f * a.hi, 2.0f * a.lo};
    else  // acos(x) = pi/2 - asin(x)
        v = ff_add(FF{kPiHalfHi, kPiHalfLo}, neg ? a : ff_neg(a));
    return v.hi + v.lo;
}

OMV_CR_HD uint32_t f2u(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
OMV_CR_HD float u2f(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

// A double-float value h + lo (h = RN(h + lo)) whose exact value is within
// about 2^-44 |h| of it can round the other way only when h + lo lies near the
// midpoint between h and its neighbour on lo's side, i.e. |lo| near half that
// gap: ulp(h) / 2, or ulp(h) / 4 below a power of two.  A few instructions,
// conservative (true also for |h| < 2^-100, which the callers pass on).
OMV_CR_HD bool maybe_midpoint(float h, float lo)
{
    const uint32_t e = f2u(h) & 0x7F800000u;
    if (e < (27u << 23)) return true;
    const float u = u2f(e - (23u << 23));  // ulp(h)
    const float a = fabsf(lo), t = 0x1p-40f * fabsf(h);
    return fabsf(a - 0.5f * u) <= t || fabsf(a - 0.25f * u) <= t;
}

// the correctly rounded choice between h and nb, given the sign of
// (exact value - midpoint of h and nb); ties to even
OMV_CR_HD float round_by_side(float h, float nb, double side)
{
    if (side == 0.0) {
        return (f2u(h) & 1u) ? nb : h;
    }
    return ((nb > h) == (side > 0.0)) ? nb : h;
}

// correctly rounded x^5 (std::pow(x, 5.0f) of a float) for x^5 in the normal
// range: a double-float product, and near a rounding midpoint (about one
// input in 2^20) an exact decision: x^5 = p1 + e1 + p2 + e2 exactly in double
// (x^2 exact, x^4 = d4h + d4l and d4h x, d4l x split by fused multiply-adds)
// the neighbour of h on lo's side
OMV_CR_HD float side_neighbour(float h, float lo)
{
    return nextafterf(h, lo > 0.0f ? 3.402823466e+38f : -3.402823466e+38f);
}

OMV_CR_RARE float pow5_decide(float x, float h, float lo)
{
    const float nb = side_neighbour(h, lo);
    const double d = (double)x, d2 = d * d;
    const double d4h = d2 * d2, d4l = fma(d2, d2, -d4h);
    const double p1 = d4h * d, e1 = fma(d4h, d, -p1);
    const double p2 = d4l * d, e2 = fma(d4l, d, -p2);
    const double m = 0.5 * ((double)h + (double)nb);  // exact
    return round_by_side(h, nb, (((p1 - m) + e1) + p2) + e2);  // p1 - m exact (Sterbenz)
}
OMV_CR_HD float pow5_cr(float x)
{
    const FF x2 = two_prod(x, x);
    const FF x4 = ff_mul(x2, x2);
    const FF x5 = ff_mul_f(x4, x);
    if (!maybe_midpoint(x5.hi, x5.lo)) return x5.hi;
    return pow5_decide(x, x5.hi, x5.lo);
}

OMV_CR_RARE float rcp_sq_decide(float x, float h, float lo)
{
    if (!(fabsf(h) >= 0x1p-125f)) return h;  // subnormal results: not decided
    const float nb = side_neighbour(h, lo);
    const double m = 0.5 * ((double)h + (double)nb);  // exact
    const double x2 = (double)x * (double)x;            // exact
    const double mh = m * x2, ml = fma(m, x2, -mh);     // m x^2 = mh + ml exactly
    return round_by_side(h, nb, -((mh - 1.0) + ml));    // sign of 1/x^2 - m = sign of 1 - m x^2
}

// correctly rounded 1 / x^2 (std::pow(x, -2.0f) of a float): the rounded
// reciprocal of x^2 = p.hi + p.lo with one Newton-Raphson correction, and near
// a rounding midpoint m an exact decision by the sign of 1 - m x^2 (m x^2 is
// a 73-bit product, split exactly by a fused multiply-add)
OMV_CR_HD float rcp_sq_cr(float x)
{
    const FF p = two_prod(x, x);  // x^2 = p.hi + p.lo exactly
    const float q = 1.0f / p.hi;
    if (q == 0.0f || !(q <= 3.402823466e+38f)) return q;  // x = 0 (inf), x^2 overflows (0), NaN
    const float r = fmaf(-q, p.hi, 1.0f);  // exact residual of the rounded reciprocal
    const float c = q * (r - q * p.lo);
    const FF v = fast_two_sum(q, c);
    if (!maybe_midpoint(v.hi, v.lo)) return v.hi;
    return rcp_sq_decide(x, v.hi, v.lo);
}

}  // namespace cr
}  // namespace omv
