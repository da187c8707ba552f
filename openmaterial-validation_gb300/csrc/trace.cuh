// Closest-hit traversal of the two-level 8-wide BVH: the device replacement of
// Embree's rtcIntersect1 as the reference calls it (BDPTRenderer.cpp:84).
//
// Hit contract (identical to the CPU oracle, oracle/oc_bvh.c):
//   * the ray is moved into instance object space with the float inverse of the
//     3x4 instance matrix, in a fixed operation order (t is preserved);
//   * Woop/Benthin/Wald watertight triangle test, fixed order, double-precision
//     retry of the edge functions when one is exactly zero;
//   * accept tnear <= t <= tfar; equal t -> lowest (instance, primitive).
// Every box test is conservative (quantised boxes rounded outward plus a
// relative margin on t), so the result does not depend on the tree layout.
#pragma once

#include "omv_device.cuh"
#include "omv_types.h"

namespace omv {

constexpr int kStackShared = 16;  // entries per thread kept in shared memory
constexpr int kStackTotal = 64;   // further entries spill to local memory
constexpr uint32_t kInstTag = 0x80000000u;

struct TraceStack {
    uint2* sh;  // this thread's first shared entry; entry i at sh[i * stride]
    int stride;
    int sp;
    int overflow;
    uint2 spill[kStackTotal - kStackShared];

    __device__ __forceinline__ void push(uint32_t id, float t)
    {
        uint2 e = make_uint2(id, __float_as_uint(t));
        if (sp < kStackShared)
            sh[sp * stride] = e;
        else if (sp < kStackTotal)
            spill[sp - kStackShared] = e;
        else {
            overflow = 1;
            return;
        }
        ++sp;
    }
    __device__ __forceinline__ uint2 pop()
    {
        --sp;
        return sp < kStackShared ? sh[sp * stride] : spill[sp - kStackShared];
    }
};

struct RayHit {
    uint32_t inst, prim;
    float t, u, v;
};

struct Shear {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ float pick3(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ float pick4(float4 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// oc_bvh.c wt_setup: false for a zero or non-finite direction
__device__ __forceinline__ bool shear_setup(V3 d, Shear& w)
{
    const float F = kFltMax;
    if (!(fabsf(d.x) <= F && fabsf(d.y) <= F && fabsf(d.z) <= F)) return false;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    float m = ax;
    if (ay > m) {
        kz = 1;
        m = ay;
    }
    if (az > m) {
        kz = 2;
        m = az;
    }
    if (!(m > 0.0f)) return false;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    float dz = pick3(d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    w.kx = kx;
    w.ky = ky;
    w.kz = kz;
    w.Sx = __fdiv_rn(pick3(d, kx), dz);
    w.Sy = __fdiv_rn(pick3(d, ky), dz);
    w.Sz = __fdiv_rn(1.0f, dz);
    return true;
}

// oc_bvh.c wt_triangle, same operation order
__device__ __forceinline__ bool tri_hit(const Shear& w, V3 o, float4 p0, float4 p1, float4 p2, float tnear, float tfar,
                                        float& t, float& u, float& v)
{
    const float okx = pick3(o, w.kx), oky = pick3(o, w.ky), okz = pick3(o, w.kz);
    const float Akx = __fsub_rn(pick4(p0, w.kx), okx), Aky = __fsub_rn(pick4(p0, w.ky), oky),
                Akz = __fsub_rn(pick4(p0, w.kz), okz);
    const float Bkx = __fsub_rn(pick4(p1, w.kx), okx), Bky = __fsub_rn(pick4(p1, w.ky), oky),
                Bkz = __fsub_rn(pick4(p1, w.kz), okz);
    const float Ckx = __fsub_rn(pick4(p2, w.kx), okx), Cky = __fsub_rn(pick4(p2, w.ky), oky),
                Ckz = __fsub_rn(pick4(p2, w.kz), okz);
    const float Ax = __fsub_rn(Akx, __fmul_rn(w.Sx, Akz));
    const float Ay = __fsub_rn(Aky, __fmul_rn(w.Sy, Akz));
    const float Bx = __fsub_rn(Bkx, __fmul_rn(w.Sx, Bkz));
    const float By = __fsub_rn(Bky, __fmul_rn(w.Sy, Bkz));
    const float Cx = __fsub_rn(Ckx, __fmul_rn(w.Sx, Ckz));
    const float Cy = __fsub_rn(Cky, __fmul_rn(w.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
        V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
        W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(w.Sz, Akz);
    const float Bz = __fmul_rn(w.Sz, Bkz);
    const float Cz = __fmul_rn(w.Sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float rcp = __fdiv_rn(1.0f, det);
    const float tt = __fmul_rn(T, rcp);
    if (!(tt >= tnear && tt <= tfar)) return false;
    t = tt;
    u = __fmul_rn(V, rcp);
    v = __fmul_rn(W, rcp);
    return true;
}

// Reciprocal for box tests only (the triangle test uses the true direction):
// zero components become +-1e-20 so that no 0 * inf NaN can appear.  The fast
// reciprocal (__fdividef: within 2 ulp for divisors up to 2^126, so the
// component is quartered first and the result quartered after, exactly while
// the result is a normal float) scales the slab distances of its axis by at
// most 1 +- 2^-22; with the roundings of the distance itself (about 2^-22
// more) that stays inside the box test's relative margins (1 -+ 2^-21), so
// the test remains conservative for direction components up to 2^126 in
// magnitude (beyond, the subnormal result adds up to 2^-22 more).  38.17
// instead of 38.55 ms per benchmark frame against the correctly rounded
// division (PTX rcp.approx.f32, subnormal results included: 38.40).
__device__ __forceinline__ float box_rcp(float d)
{
    const float x = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return __fdividef(1.0f, 0.25f * x) * 0.25f;
}

// Whether the ray (origin o, box reciprocal rid) meets the box [lo, hi] within
// [tnear, tfar]: slab distances with the node test's relative margins, so
// conservative in the same way.
__device__ __forceinline__ bool object_box_hit(float4 lo, float4 hi, V3 o, V3 rid, float tnear, float tfar)
{
    const float ax = (lo.x - o.x) * rid.x, bx = (hi.x - o.x) * rid.x;
    const float ay = (lo.y - o.y) * rid.y, by = (hi.y - o.y) * rid.y;
    const float az = (lo.z - o.z) * rid.z, bz = (hi.z - o.z) * rid.z;
    const float tin = fmaxf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)) * 0.99999952f, tnear);
    const float tout = fminf(fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz)) * 1.00000048f, tfar);
    return tin <= tout;
}

// world -> object space, 3x4 row-major inverse, fixed order
__device__ __forceinline__ void to_object(const float* m, V3 o, V3 d, V3& ro, V3& rd)
{
    ro = v3(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], o.x), __fmul_rn(m[1], o.y)), __fmul_rn(m[2], o.z)), m[3]),
            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], o.x), __fmul_rn(m[5], o.y)), __fmul_rn(m[6], o.z)), m[7]),
            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], o.x), __fmul_rn(m[9], o.y)), __fmul_rn(m[10], o.z)), m[11]));
    rd = v3(__fadd_rn(__fadd_rn(__fmul_rn(m[0], d.x), __fmul_rn(m[1], d.y)), __fmul_rn(m[2], d.z)),
            __fadd_rn(__fadd_rn(__fmul_rn(m[4], d.x), __fmul_rn(m[5], d.y)), __fmul_rn(m[6], d.z)),
            __fadd_rn(__fadd_rn(__fmul_rn(m[8], d.x), __fmul_rn(m[9], d.y)), __fmul_rn(m[10], d.z)));
}

// Quantised plane of slot s (two 16-bit planes per word, each 0x8000 | q) as
// the float Q = 1 + q * 2^-15: one byte permute places the plane under the
// byte 0x3F and above a zero byte, and the flag bit completes the exponent 127.
// A plane's slab distance (p + q s - o) / d is then Q A + (b - A) with
// A = 2^15 s / d and b = (p - o) / d: one fused multiply-add per plane.
__device__ __forceinline__ float qplane(uint4 w, int s)
{
    const uint32_t x = (s >> 1) == 0 ? w.x : (s >> 1) == 1 ? w.y : (s >> 1) == 2 ? w.z : w.w;
    return __uint_as_float(__byte_perm(x, 0x3F000000u, (s & 1) ? 0x7324u : 0x7104u));
}

// Offset b - k A of the near (kNear) or far plane distances of one axis.  The
// rounding of b - A is at most 2^-24 (|b| + |A|): the |b| part is of the size
// of b's own rounding, which the relative margins of the box test cover, and
// the |A| part (2^-9 of a quantum's distance) is covered by moving the near
// planes 2^-21 |A| (2^-6 of a quantum) closer and the far planes as much
// farther (k = 1 -+ 2^-21, exact; A has the sign of 1/d).
template <bool kNear>
__device__ __forceinline__ float plane_offset(float b, float A)
{
    const float up = 1.0f + 0x1p-21f, down = 1.0f - 0x1p-21f;
    return fmaf(-((A >= 0.0f) == kNear ? up : down), A, b);
}

__device__ __forceinline__ void cswap(uint32_t& a, uint32_t& b)
{
    uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

struct TraceCounters {
    uint32_t nodes;
    uint32_t tris;
};

// Traversal state of one ray: trace_begin, then trace_step until it returns
// false, then trace_end (trace_closest runs the three in a row).  Keeping the
// state in one struct and one stack entry per step also compiles to a faster
// loop than the single-function form (38.5 vs 38.9 ms per benchmark frame).
struct TraceState {
    V3 o, d, idw;      // world ray and box reciprocal
    V3 ro, rid;        // the ray in the current space (world or instance object space)
    Shear rs;          // shear of the current space's direction
    float tnear, best_t, bu, bv;
    uint32_t best_inst, best_prim, cur_inst, guard;
    int blas_base;     // stack depth at which the current instance's tree started
    bool in_blas, found;
};

// false when the ray cannot hit anything (empty interval, zero or non-finite direction)
__device__ __forceinline__ bool trace_begin(const DevScene& S, V3 o, V3 d, float tnear, float tfar, TraceState& T,
                                           TraceStack& st, uint32_t root = kInvalid)
{
    if (!(tnear <= tfar) || S.num_instances == 0) return false;
    if (!shear_setup(d, T.rs)) return false;
    T.o = o;
    T.d = d;
    T.idw = v3(box_rcp(d.x), box_rcp(d.y), box_rcp(d.z));
    T.ro = o;
    T.rid = T.idw;
    T.tnear = tnear;
    T.best_t = tfar;
    T.bu = T.bv = 0.0f;
    T.best_inst = T.best_prim = kInvalid;
    T.cur_inst = 0;
    T.guard = 0;
    T.blas_base = 0;
    T.in_blas = false;
    T.found = false;
    st.sp = 0;
    st.push(root == kInvalid ? S.tlas_root : root, tnear);  // root: one scene of a group
    return true;
}

// Processes one stack entry (an instance or a node); false when the traversal is
// over.  kStop: also over as soon as a hit with t < stop_below is taken (an
// occlusion query stops at any hit: stop_below = infinity).
template <bool kStop = false>
__device__ __forceinline__ bool trace_step(const DevScene& S, const uint32_t* __restrict__ tlas_items, TraceState& T,
                                          TraceStack& st, TraceCounters& tc, float stop_below = 0.0f)
{
    if (T.guard++ > (1u << 22)) {  // a malformed tree can never spin a warp forever
        st.overflow = 1;
        return false;
    }
    if (T.in_blas && st.sp == T.blas_base) {
        T.in_blas = false;
        T.ro = T.o;
        T.rid = T.idw;
    }
    if (st.sp == 0) return false;
    const uint2 e = st.pop();
    if (__uint_as_float(e.y) > T.best_t) return true;
    if (e.x & kInstTag) {
        const uint32_t ii = e.x & ~kInstTag;
        const DevInstance* I = S.insts + ii;
        float m[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) m[k] = __ldg(&I->inv[k]);
        V3 rd;
        to_object(m, T.o, T.d, T.ro, rd);
        const V3 rid = v3(box_rcp(rd.x), box_rcp(rd.y), box_rcp(rd.z));
        // the object's own bounds first: most rays that cross an instance's
        // world box (the box of a rotated object) miss the object's box
        if (!object_box_hit(__ldg(&I->olo), __ldg(&I->ohi), T.ro, rid, T.tnear, T.best_t) || !shear_setup(rd, T.rs)) {
            T.ro = T.o;
            return true;
        }
        T.rid = rid;
        T.in_blas = true;
        T.blas_base = st.sp;
        T.cur_inst = ii;
        st.push(__ldg(&I->blas_root), __uint_as_float(e.y));
        return true;
    }
    ++tc.nodes;
    const uint4* N = S.nodes + 8 * (size_t)e.x;
    const uint4 w0 = __ldg(N + 0), w1 = __ldg(N + 1);
    const uint4 qlx = __ldg(N + 2), qly = __ldg(N + 3), qlz = __ldg(N + 4);
    const uint4 qhx = __ldg(N + 5), qhy = __ldg(N + 6), qhz = __ldg(N + 7);
    const float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    const uint32_t exps = w0.w;
    const uint32_t imask = exps >> 24;
    const uint32_t child_base = w1.x, prim_base = w1.y, meta_lo = w1.z, meta_hi = w1.w;
    // 2^15 times the quantum 2^(e-127) of each axis (e <= 239)
    const float sx = __uint_as_float(((exps & 0xFFu) + 15u) << 23);
    const float sy = __uint_as_float((((exps >> 8) & 0xFFu) + 15u) << 23);
    const float sz = __uint_as_float((((exps >> 16) & 0xFFu) + 15u) << 23);
    const V3 rid = T.rid, ro = T.ro;
    const float ax = sx * rid.x, ay = sy * rid.y, az = sz * rid.z;
    const float bx = (px - ro.x) * rid.x, by = (py - ro.y) * rid.y, bz = (pz - ro.z) * rid.z;
    const float bnx = plane_offset<true>(bx, ax), bfx = plane_offset<false>(bx, ax);
    const float bny = plane_offset<true>(by, ay), bfy = plane_offset<false>(by, ay);
    const float bnz = plane_offset<true>(bz, az), bfz = plane_offset<false>(bz, az);
    // entry and exit planes per axis from the ray direction: for a child with
    // qlo <= qhi these are exactly min() and max() of the two slab distances
    const uint4 nx = rid.x >= 0.0f ? qlx : qhx, fx = rid.x >= 0.0f ? qhx : qlx;
    const uint4 ny = rid.y >= 0.0f ? qly : qhy, fy = rid.y >= 0.0f ? qhy : qly;
    const uint4 nz = rid.z >= 0.0f ? qlz : qhz, fz = rid.z >= 0.0f ? qhz : qlz;
    const float lim = T.best_t, tnear = T.tnear;
    uint32_t key[8];
    uint32_t leafmask = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xFFu;
        const bool internal = (imask >> s) & 1u;
        const bool valid = internal || meta != 0u;
        const float tnx = fmaf(qplane(nx, s), ax, bnx), tfx = fmaf(qplane(fx, s), ax, bfx);
        const float tny = fmaf(qplane(ny, s), ay, bny), tfy = fmaf(qplane(fy, s), ay, bfy);
        const float tnz = fmaf(qplane(nz, s), az, bnz), tfz = fmaf(qplane(fz, s), az, bfz);
        const float tin = fmaxf(fmaxf(fmaxf(tnx, tny), tnz) * 0.99999952f, tnear);
        const float tout = fminf(fminf(fminf(tfx, tfy), tfz) * 1.00000048f, lim);
        key[s] = 0xFFFFFFFFu;
        if (valid && tin <= tout) {
            if (!internal && T.in_blas)
                leafmask |= 1u << s;
            else  // entry distance rounded down to 8 ulp | slot
                key[s] = (__float_as_uint(fmaxf(tin, 0.0f)) & ~7u) | (uint32_t)s;
        }
    }
    // leaf triangles first: they can shrink best_t before children are pushed
    for (uint32_t m = leafmask; m; m &= m - 1u) {
        const int s = __ffs(m) - 1;
        const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xFFu;
        const uint32_t cnt = meta >> 5, off = meta & 31u;
        for (uint32_t k = 0; k < cnt; ++k) {
            const float4* Tp = S.tris + 3 * (size_t)(prim_base + off + k);
            const float4 a = __ldg(Tp), b = __ldg(Tp + 1), c = __ldg(Tp + 2);
            ++tc.tris;
            float t, u, v;
            if (tri_hit(T.rs, T.ro, a, b, c, tnear, T.best_t, t, u, v)) {
                const uint32_t prim = __float_as_uint(a.w);
                const bool take = !T.found || t < T.best_t ||
                                  (t == T.best_t && (T.cur_inst < T.best_inst ||
                                                     (T.cur_inst == T.best_inst && prim < T.best_prim)));
                if (take) {
                    T.found = true;
                    T.best_t = t;
                    T.bu = u;
                    T.bv = v;
                    T.best_inst = T.cur_inst;
                    T.best_prim = prim;
                    if (kStop && t < stop_below) return false;
                }
            }
        }
    }
    // 19-comparator sorting network (Knuth, TAOCP vol. 3, 5.3.4), ascending entry t
    cswap(key[0], key[2]); cswap(key[1], key[3]); cswap(key[4], key[6]); cswap(key[5], key[7]);
    cswap(key[0], key[4]); cswap(key[1], key[5]); cswap(key[2], key[6]); cswap(key[3], key[7]);
    cswap(key[0], key[1]); cswap(key[2], key[3]); cswap(key[4], key[5]); cswap(key[6], key[7]);
    cswap(key[2], key[4]); cswap(key[3], key[5]);
    cswap(key[1], key[4]); cswap(key[3], key[6]);
    cswap(key[1], key[2]); cswap(key[3], key[4]); cswap(key[5], key[6]);
#pragma unroll
    for (int j = 7; j >= 0; --j) {
        const uint32_t k = key[j];
        if (k == 0xFFFFFFFFu) continue;
        const float te = __uint_as_float(k & ~7u);
        if (te > T.best_t) continue;
        const uint32_t s = k & 7u;
        const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xFFu;
        if ((imask >> s) & 1u)
            st.push(child_base + meta, te);
        else
            st.push(kInstTag | __ldg(tlas_items + prim_base + (meta & 31u)), te);
    }
    return true;
}

__device__ __forceinline__ bool trace_end(const TraceState& T, RayHit& hit)
{
    if (!T.found) return false;
    hit.inst = T.best_inst;
    hit.prim = T.best_prim;
    hit.t = T.best_t;
    hit.u = T.bu;
    hit.v = T.bv;
    return true;
}

// Whether any triangle is hit in [tnear, tfar] (the closest-hit query's answer
// to "is there a hit", without finding the closest).
__device__ __forceinline__ bool trace_any(const DevScene& S, const uint32_t* __restrict__ tlas_items, V3 o, V3 d,
                                          float tnear, float tfar, TraceStack& st, TraceCounters& tc,
                                          uint32_t root = kInvalid)
{
    TraceState T;
    if (!trace_begin(S, o, d, tnear, tfar, T, st, root)) return false;
    while (trace_step<true>(S, tlas_items, T, st, tc, __int_as_float(0x7F800000))) {
    }
    return T.found;
}

// Closest hit, except that the traversal stops at the first hit found with
// t < stop_below (then `hit` is that hit, not necessarily the closest).
__device__ __forceinline__ bool trace_closest_or_below(const DevScene& S, const uint32_t* __restrict__ tlas_items, V3 o,
                                                       V3 d, float tnear, float tfar, float stop_below, RayHit& hit,
                                                       TraceStack& st, TraceCounters& tc, uint32_t root = kInvalid)
{
    TraceState T;
    if (!trace_begin(S, o, d, tnear, tfar, T, st, root)) return false;
    while (trace_step<true>(S, tlas_items, T, st, tc, stop_below)) {
    }
    return trace_end(T, hit);
}

// Closest hit; returns true and fills `hit` when a triangle is found.
__device__ __forceinline__ bool trace_closest(const DevScene& S, const uint32_t* __restrict__ tlas_items, V3 o, V3 d,
                                           float tnear, float tfar, RayHit& hit, TraceStack& st, TraceCounters& tc,
                                           uint32_t root = kInvalid)
{
    TraceState T;
    if (!trace_begin(S, o, d, tnear, tfar, T, st, root)) return false;
    while (trace_step(S, tlas_items, T, st, tc)) {
    }
    return trace_end(T, hit);
}

}  // namespace omv
