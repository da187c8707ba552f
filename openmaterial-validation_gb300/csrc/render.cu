// Wavefront bidirectional render loop: the device form of
// BDPTRenderer::render -> renderRow -> computePaths (BDPTRenderer.cpp:237-393).
//
// A frame of W*H*spp paths is processed in waves of up to `wave_cap` paths.
// Per wave (all launches on one stream, queue sizes stay on the device):
//   light stage  (only with point lights)
//     k_light_gen       light pick + uniformSphere emission (tryComputeLightPath)
//     k_extend          closest hit of every queued ray
//     k_light_shade     surface point, BRDF sample, light-vertex store, cut-off
//   camera stage
//     k_camera_gen      jittered pinhole rays (PinholeCamera::getRay)
//     k_extend
//     k_camera_shade    surface point, BRDF sample, environment on escape,
//                       light/camera vertex connections (and, with the MIS
//                       estimator, environment rays) -> shadow queue
//     k_shadow          isConnected (closest hit + end-point test), add
//   k_film              per-path radiance into the FP64 film (PinholeCamera::hit)
// Queues are SoA-packed float4 records appended with warp-aggregated atomics
// (ballot + popc); the tracing kernels are persistent and fetch 32 rays per
// warp from an atomic work counter.  Random numbers are Philox4x32-10 keyed by
// (pixel, sample, vertex) so any partition of the work gives the same image.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "omv_device.cuh"
#include "scene.h"
#include "trace.cuh"
#include "shade.cuh"

namespace omv {

namespace {

constexpr int kTraceThreads = 128;
// 6 resident blocks of the trace kernels per SM (80 registers, a few spilled
// stack words): more warps in flight for the latency-bound traversal than the
// 5 blocks its unconstrained 96 registers allow (measured 3.18 -> 3.06 ms per
// extension launch on the 1920x1080x64 frame; 7 and 8 blocks spill more)
constexpr int kTraceMinBlocks = 6;
constexpr int kShadeThreads = 256;

// counter slots within RenderScratch::ctr (reset per wave)
constexpr int kCtrLight = 0;     // + bounce (0..light_bounces)
constexpr int kCtrCam = 64;      // + bounce (0..camera_bounces)
constexpr int kCtrShadow = 128;  // + bounce
constexpr int kCtrWork = 192;    // + launch index
constexpr int kCtrEnv = 448;     // + bounce: MIS environment rays
enum {
    kStatExt = 0, kStatShadow = 1, kStatLight = 2, kStatNodes = 3, kStatTris = 4, kStatOverflow = 5,
    kStatShadowNodes = 6, kStatShadowTris = 7, kStatTailNodes = 8, kStatTailTris = 9, kStatTailCam = 10
};
// Tail kernel (k_camera_tail): once at most kTailPaths camera paths
// are alive at a bounce (from bounce kTailMin on), one launch takes each of
// them to its end, one thread per path, instead of a launch pair (or three)
// per remaining bounce, each of which costs the latency of its slowest ray.
// The decision is made on the device from the bounce's queue count, so the
// host launches the tail kernel before every bounce from kTailMin on; it returns
// at once while more paths are alive, and after it has run, the queue count
// it leaves at zero makes the bounce's wavefront kernels return at once.
// Only for scenes without point lights: with vertex connections, one thread
// testing a path's connections one after another loses to the wavefront's
// shadow-ray kernel (measured: the 256x256x16 C1 frame 1.72 instead of 1.30
// ms, the 1920x1080x64 one 48.4 instead of 47.1, the 256-job sweep one job
// per call 94.5 instead of 103.1 jobs/s), and so did the light subpaths'
// analogue.  On the benchmark frame: 38.40 instead of 38.67 ms (at most 2^17
// paths: the same; 2^19 or 2^20, which start the tail at bounce 4: 39.0).
constexpr int kTailMin = 3;
constexpr uint32_t kTailPaths = 1u << 18;
// counter slots of the tail kernel (beyond the per-bounce ranges)
constexpr int kCtrTailWorkCam = 510;
constexpr int kCtrTailDone = 511;

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want)
{
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, want);
    if (!m) return 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// NVTX range for profilers (a wave, a stage, a bounce); free without a tool attached
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
constexpr const char* kBounceNames[] = {"bounce 0",  "bounce 1",  "bounce 2",  "bounce 3",  "bounce 4",  "bounce 5",
                                        "bounce 6",  "bounce 7",  "bounce 8",  "bounce 9",  "bounce 10", "bounce 11",
                                        "bounce 12", "bounce 13", "bounce 14", "bounce 15", "bounce > 15"};
inline const char* bounce_name(int b) { return kBounceNames[b < 16 ? b : 16]; }

// Opportunistic warp aggregation (for appends inside divergent code): the
// threads of a warp that arrive together take consecutive slots with one atomic.
__device__ __forceinline__ uint32_t coalesced_append(uint32_t* counter)
{
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, (uint32_t)g.size());
    return g.shfl(base, 0) + (uint32_t)g.thread_rank();
}

// Direction bin of a ray: the cube face its direction points to (dominant
// axis and sign) and the quadrant on that face, 24 bins.
constexpr int kDirBins = 24;
__device__ __forceinline__ uint32_t direction_bin(V3 d)
{
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    uint32_t f;
    float u, v;
    if (ax >= ay && ax >= az) {
        f = d.x < 0.0f ? 1u : 0u;
        u = d.y;
        v = d.z;
    } else if (ay >= az) {
        f = d.y < 0.0f ? 3u : 2u;
        u = d.z;
        v = d.x;
    } else {
        f = d.z < 0.0f ? 5u : 4u;
        u = d.x;
        v = d.y;
    }
    return 4u * f + (u < 0.0f ? 2u : 0u) + (v < 0.0f ? 1u : 0u);
}

struct BinScratch {
    uint32_t count[kDirBins];
    uint32_t base;
};

// Block-wide append to a queue with the block's entries grouped by bin, so
// that the warps tracing the queue get rays of similar direction from nearby
// pixels.  One atomic per block; every thread of the block must call it.
__device__ __forceinline__ uint32_t block_append_binned(uint32_t* counter, bool want, uint32_t bin, BinScratch& sh)
{
    if (threadIdx.x < kDirBins) sh.count[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t rank = want ? atomicAdd(&sh.count[bin], 1u) : 0u;
    __syncthreads();
    if (threadIdx.x < 32) {
        // exclusive scan of the bin counts in the first warp; lane 31 reserves
        const uint32_t c = threadIdx.x < kDirBins ? sh.count[threadIdx.x] : 0u;
        uint32_t x = c;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if ((int)threadIdx.x >= o) x += y;
        }
        if (threadIdx.x < kDirBins) sh.count[threadIdx.x] = x - c;
        if (threadIdx.x == 31) sh.base = x ? atomicAdd(counter, x) : 0u;
    }
    __syncthreads();
    const uint32_t slot = sh.base + sh.count[bin] + rank;
    __syncthreads();  // the scratch is reused by the next call
    return slot;
}

// Division of 32-bit unsigned integers by a divisor fixed for a frame, by one
// multiply-high, a subtraction and two shifts (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994, 4.1):
// exact for every numerator and every divisor >= 1, where the hardware has
// no integer divide.
struct FastDiv {
    uint32_t d, m;
    int s1, s2;
};
inline FastDiv make_fastdiv(uint32_t d)
{
    int l = 0;
    while (l < 32 && (1ull << l) < d) ++l;
    FastDiv f;
    f.d = d;
    f.m = (uint32_t)(((((1ull << l) - d) << 32) / d) + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}
__device__ __forceinline__ uint32_t fast_div(const FastDiv& f, uint32_t n)
{
    const uint32_t t1 = __umulhi(f.m, n);
    return (t1 + ((n - t1) >> f.s1)) >> f.s2;
}

struct WaveArgs {
    DevScene S;
    const uint32_t* items;
    omv_camera cam;
    uint64_t seed;
    int64_t wave_base;
    int32_t wave_n;
    int32_t wave_cap;
    int32_t npix;
    int32_t spp;
    int32_t sample_offset;
    uint32_t base_q, base_r;  // wave_base / spp, wave_base % spp (batch: first global pixel, unused)
    uint32_t last_pixel;      // pixel of the wave's last path (batch: global pixel)
    const DevJob* jobs;       // batch job table (num_jobs == 0: one frame with the fields above)
    int32_t num_jobs;
    uint32_t* path_job;       // batch: job of each path of the wave
    float4* env_q;  // MIS environment rays (3 float4 each), after the vertex connections' slots
    int32_t cam_bounces, light_bounces, max_len;
    int32_t atten_mode;
    float light_scale, min_dist, cut;
    FastDiv spp_div, width_div;  // by spp and by cam.width (one frame)
    RenderScratch R;
};

// Path g of the frame is sample g % spp of pixel g / spp: the samples of one
// pixel are neighbours, so a warp's camera rays (and first shading points) are
// nearly identical.  Random numbers are keyed by (pixel, sample), so the order
// does not change the image.
__device__ __forceinline__ void path_ids(const WaveArgs& A, int k, uint32_t& pixel, uint32_t& sample)
{
    const uint32_t t = A.base_r + (uint32_t)k;  // < spp + 2^31
    const uint32_t q = fast_div(A.spp_div, t);
    pixel = A.base_q + q;
    sample = (uint32_t)A.sample_offset + (t - q * (uint32_t)A.spp);
}

// What a path needs to know about its job: pixel and sample within the job,
// the job's seed and material table (one frame: the frame's).
struct PathCtx {
    uint32_t pixel, sample;
    uint64_t seed;
    const DevMaterial* mats;
};
__device__ __forceinline__ PathCtx path_ctx(const WaveArgs& A, int k)
{
    PathCtx c;
    if (A.num_jobs == 0) {
        path_ids(A, k, c.pixel, c.sample);
        c.seed = A.seed;
        c.mats = A.S.mats;
    } else {
        const DevJob& J = A.jobs[A.path_job[k]];
        const uint32_t local = (uint32_t)(A.wave_base + k - J.path_base);
        c.pixel = local / (uint32_t)J.spp;
        c.sample = (uint32_t)J.sample_offset + local % (uint32_t)J.spp;
        c.seed = J.seed;
        c.mats = J.mats;
    }
    return c;
}

// batch: the job of every path of the wave (largest job whose first path <= g)
__global__ void __launch_bounds__(kShadeThreads) k_job_ids(WaveArgs A)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.wave_n) return;
    const int64_t g = A.wave_base + k;
    int lo = 0, hi = A.num_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.jobs[mid].path_base <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    A.path_job[k] = (uint32_t)lo;
}

// ------------------------------------------------------------ raygen ---
__global__ void __launch_bounds__(kShadeThreads) k_camera_gen(WaveArgs A)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = k < A.wave_n;
    uint32_t pixel = 0, sample = 0;
    V3 O = v3(0, 0, 0), R = v3(0, 0, 1);
    if (ok) {
        const PathCtx c = path_ctx(A, k);
        pixel = c.pixel;
        sample = c.sample;
        const omv_camera& cam = A.num_jobs ? A.jobs[A.path_job[k]].cam : A.cam;
        Rng4 r = rng4(c.seed, pixel, sample, 0u, kStreamCamera);
        const uint32_t row = A.num_jobs ? pixel / (uint32_t)cam.width : fast_div(A.width_div, pixel);
        camera_ray(cam, (int)(pixel - row * (uint32_t)cam.width), (int)row, r.u[0], r.u[1], O, R);
        // throughput starts at 1 and radiance at 0: the first camera shade uses
        // the constants and writes both, so only a frame without camera
        // bounces needs the radiance cleared here
        if (A.cam_bounces == 0) A.R.rad[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    // every path emits a camera ray: queue slot = path index, no append
    if (k == 0) A.R.ctr[kCtrCam + 1] = (uint32_t)A.wave_n;
    if (ok) {
        V3 so = shifted_origin(O, R, 1.0f);
        A.R.rq[0][2 * (size_t)k] = make_float4(so.x, so.y, so.z, 0.0f);
        A.R.rq[0][2 * (size_t)k + 1] = make_float4(R.x, R.y, R.z, __int_as_float(k));
    }
}

// tryComputeLightPath (BDPTRenderer.cpp:194-206): sampleLight + getRandomRay
__global__ void __launch_bounds__(kShadeThreads) k_light_gen(WaveArgs A)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = k < A.wave_n;
    V3 O = v3(0, 0, 0), R = v3(0, 0, 1);
    if (ok) {
        const PathCtx c = path_ctx(A, k);
        const uint32_t pixel = c.pixel, sample = c.sample;
        const DevScene& S = A.S;
        // the path's scene's lights (a batch job's; one frame: the scene's)
        int lbase = 0, N = S.num_lights;
        float lmax = S.light_max;
        if (A.num_jobs) {
            const DevJob& J = A.jobs[A.path_job[k]];
            lbase = J.light_base;
            N = J.light_count;
            lmax = J.light_max;
        }
        const float* cdf = S.light_cdf + lbase;
        // DistanceRandom::getValue (DistanceRandom.h:98-115); one light: no draw
        int li = 0;
        if (N > 1) {
            const float d = rng4(c.seed, pixel, sample, 0u, kStreamLight).u[0] * lmax;
            if (d <= cdf[0])
                li = 0;
            else if (d >= cdf[N - 2])
                li = N - 1;
            else {
                int L = 0, Rr = N - 1;
                while (L < Rr) {
                    int C = (L + Rr) / 2;
                    if (d <= cdf[C])
                        Rr = C;
                    else
                        L = C + 1;
                }
                li = (L + Rr) / 2;
            }
        }
        li += lbase;
        R = light_direction(c.seed, pixel, sample);  // RandomSampler::uniformSphere
        const float4 lp = __ldg(S.light_pos + li);
        O = v3(lp.x, lp.y, lp.z);
        // the light vertex itself is the light's position and intensity: the
        // connections and the first light vertex read them from the light, so
        // only the light index (and the subpath length 1) is stored here
        A.R.lmeta[k] = (uint32_t)li | (1u << 16);
    }
    // with light bounces every path emits a light ray: queue slot = path index
    const bool push = ok && A.light_bounces >= 1;
    if (k == 0 && A.light_bounces >= 1) A.R.ctr[kCtrLight + 1] = (uint32_t)A.wave_n;
    if (push) {
        V3 so = shifted_origin(O, R, 1.0f);
        A.R.rq[1][2 * (size_t)k] = make_float4(so.x, so.y, so.z, 0.0f);
        A.R.rq[1][2 * (size_t)k + 1] = make_float4(R.x, R.y, R.z, __int_as_float(k));
    }
}

// ------------------------------------------------------------ extend ---
// Persistent closest-hit over one ray queue (count at *count): a warp takes 32
// consecutive rays and the next 32 when all are done (camera rays: the 32
// samples of one pixel stay together).  Replacing finished rays lane by lane
// (Aila & Laine 2009) was measured slower on every bounce.
// `jobs` (batches over a group of scenes, else null): the top-level tree of
// the path's scene (the path index travels in the ray's last word)
__device__ __forceinline__ uint32_t path_root(const DevJob* jobs, const uint32_t* path_job, int k)
{
    return jobs ? jobs[path_job[k]].tlas_root : kInvalid;
}

__global__ void __launch_bounds__(kTraceThreads, kTraceMinBlocks) k_extend(DevScene S, const uint32_t* items, float4* rq, uint4* hits,
                                                          const uint32_t* count, uint32_t* work,
                                                          unsigned long long* stats, int stat_kind,
                                                          const DevJob* jobs, const uint32_t* path_job)
{
    __shared__ uint2 sstack[kStackShared * kTraceThreads];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kTraceThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    const uint32_t n = *count;
    const int lane = threadIdx.x & 31;
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            float4 a = rq[2 * (size_t)i], b = rq[2 * (size_t)i + 1];
            V3 o = v3(a.x, a.y, a.z), d = v3(b.x, b.y, b.z);
            float tnear = a.w;
            RayHit h;
            uint4 out;
            if (scene_intersect(S, items, o, d, tnear, kFltMax, h, st, tc,
                                path_root(jobs, path_job, __float_as_int(b.w))))
                out = make_uint4(h.inst, h.prim, __float_as_uint(h.u), __float_as_uint(h.v));
            else
                out = make_uint4(kInvalid, kInvalid, 0u, 0u);
            hits[i] = out;
            if (tnear != a.w) rq[2 * (size_t)i].w = tnear;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats[stat_kind], (unsigned long long)n);
    uint32_t nodes = tc.nodes, tris = tc.tris;
    for (int o = 16; o; o >>= 1) {
        nodes += __shfl_xor_sync(0xFFFFFFFFu, nodes, o);
        tris += __shfl_xor_sync(0xFFFFFFFFu, tris, o);
    }
    const bool ov = __any_sync(0xFFFFFFFFu, st.overflow);
    if (lane == 0 && nodes) {
        atomicAdd(&stats[kStatNodes], (unsigned long long)nodes);
        atomicAdd(&stats[kStatTris], (unsigned long long)tris);
    }
    if (lane == 0 && ov) atomicAdd(&stats[kStatOverflow], 1ull);
}

// ------------------------------------------------------- light shade ---
// BDPTRenderer::computePath for the light subpath (inv = false), vertex b of
// path k reached by the ray (ra, rb) with hit h: the vertex's position and
// radiance for the connections, its throughput and the next ray.  True when
// the path goes on (next ray: origin so, direction O, tnear).
__device__ __forceinline__ bool light_vertex(const WaveArgs& A, int b, int k, float4 ra, float4 rb, uint4 h, V3& so,
                                             V3& O, float& tnear)
{
    const DevScene& S = A.S;
    bool push = false;
    tnear = ra.w;
    if (h.x == kInvalid) return false;
    const PathCtx c = path_ctx(A, k);
    const uint32_t pixel = c.pixel, sample = c.sample;
    const DevMaterial& M = c.mats[__ldg(&S.insts[h.x].material)];
    const Surf sp = surface_point(S, h.x, h.y, __uint_as_float(h.z), __uint_as_float(h.w), true, &M);
    const V3 in = v3(rb.x, rb.y, rb.z);
    const Rng4 u = rng4(c.seed, pixel, sample, kDimLightBounce + (uint32_t)b, kStreamLight);
    const V3 brdf = material_sample(S, M, pbr_params(S, M, sp), sp, in, false, u, O);
    const float ct = fabsf(dot(in, sp.nrm));
    const uint32_t meta = A.R.lmeta[k];
    const uint32_t li = meta & 0xFFFFu;
    float4 tp0, lr;
    if (b == 1) {  // throughput 1; the light's radiance and the attenuation to this vertex
        tp0 = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        const float4 I = __ldg(S.light_int + li);
        const float4 lp = __ldg(S.light_pos + li);
        const V3 d = sp.pos - v3(lp.x, lp.y, lp.z);
        lr = make_float4(I.x * A.light_scale, I.y * A.light_scale, I.z * A.light_scale,
                         light_attenuation(A.atten_mode, A.min_dist, sqrtf(dot(d, d)), lp.w));
        A.R.lrad[k] = lr;
    } else {
        tp0 = A.R.ltp[k];
        lr = A.R.lrad[k];
    }
    const V3 tp = v3(tp0.x * brdf.x * ct, tp0.y * brdf.y * ct, tp0.z * brdf.z * ct);
    const V3 orad = v3(tp.x * lr.x * lr.w, tp.y * lr.y * lr.w, tp.z * lr.z * lr.w);
    if (!(intensity(orad) < A.cut)) {
        const size_t slot = (size_t)b * A.wave_cap + k;
        A.R.lv_pos[slot] = make_float4(sp.pos.x, sp.pos.y, sp.pos.z, 0.0f);
        A.R.lv_rad[slot] = make_float4(orad.x, orad.y, orad.z, 0.0f);
        A.R.lmeta[k] = li | ((uint32_t)(b + 1) << 16);
        A.R.ltp[k] = make_float4(tp.x, tp.y, tp.z, 0.0f);
        if (b < A.light_bounces && (tp.x != 0.0f || tp.y != 0.0f || tp.z != 0.0f)) {
            push = true;
            so = shifted_origin(sp.pos, O, 1.0f);
        }
    }
    return push;
}

// k_light_shade: light_vertex for every ray of the bounce-b queue
__global__ void __launch_bounds__(kShadeThreads, 4) k_light_shade(WaveArgs A, int b, const float4* rq_in,
                                                                float4* rq_out)
{
    const uint32_t n = A.R.ctr[kCtrLight + b];
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        bool push = false;
        V3 so = v3(0, 0, 0), O = v3(0, 0, 1);
        float tnear = 0.0f;
        int k = 0;
        if (i < n) {
            const uint4 h = A.R.hits[i];
            if (h.x != kInvalid) {  // most light rays leave the scene: their ray is not read
                const float4 ra = rq_in[2 * (size_t)i], rb = rq_in[2 * (size_t)i + 1];
                k = __float_as_int(rb.w);
                push = light_vertex(A, b, k, ra, rb, h, so, O, tnear);
            }
        }
        const uint32_t slot = warp_append(&A.R.ctr[kCtrLight + b + 1], push);
        if (push) {
            rq_out[2 * (size_t)slot] = make_float4(so.x, so.y, so.z, tnear);
            rq_out[2 * (size_t)slot + 1] = make_float4(O.x, O.y, O.z, __int_as_float(k));
        }
    }
}

// ------------------------------------------------ environment connection ---
constexpr uint32_t kDimEnvConnect = 2048u;

// The MIS estimator at camera vertex b of a PBR surface: a direction drawn
// from the environment's alias table, weighted by the power heuristic against
// the vertex's own reflection sampling, and queued as an environment ray; the
// escape of the sampled direction O (next bounce) gets the complementary
// weight from the density returned here.  Both strategies estimate the
// sampler's own integrand (bsdf_reflection_mix), and the environment ray is
// traced exactly as a sampled ray in that direction would be (origin shifted
// along it, the path's tnear, unbounded, escaping when nothing is hit, so
// that both see the same self-intersections), so the image's expectation is
// the reference estimator's.  Only an escape the reference would count is
// connected: b < camera bounces and b + 1 <= maxPathLength.
struct EnvRay {
    V3 so, w, c;  // shifted origin, direction, contribution
    float tnear;
    bool push;
};
static __device__ __noinline__ float env_connect(const WaveArgs& A, int b, uint64_t seed, uint32_t pixel,
                                                 uint32_t sample, BsdfIn d, V3 pos, V3 nrm, V3 tp, V3 O, int kind,
                                                 float tnear, EnvRay& er)
{
    const DevScene& S = A.S;
    float pdf_o = 0.0f;
    V3 unused;
    if (kind == 0 || kind == 1) pdf_o = bsdf_reflection_mix(d, O, 1.0f, unused);
    bool push = false;
    V3 w = v3(0.0f, 0.0f, 1.0f), c = v3(0.0f, 0.0f, 0.0f);
    if (b < A.cam_bounces && b + 1 <= A.max_len) {
        const Rng4 r = rng4(seed, pixel, sample, kDimEnvConnect + (uint32_t)b, kStreamCamera);
        const float pe = env_sample(S.env, r.u[0], r.u[1], r.u[2], r.u[3], w);
        if (pe > 0.0f) {
            V3 feff;
            const float pb = bsdf_reflection_mix(d, w, fabsf(dot(w, nrm)), feff);
            if (pb > 0.0f) {
                const V3 L = env_radiance(S.env, w);
                const float m = pe / (pe * pe + pb * pb);  // power heuristic pe^2 / (pe^2 + pb^2), over pe
                c = v3(tp.x * feff.x * L.x * m, tp.y * feff.y * L.y * m, tp.z * feff.z * L.z * m);
                push = c.x > 0.0f || c.y > 0.0f || c.z > 0.0f;
            }
        }
    }
    er.push = push;
    er.w = w;
    er.c = c;
    er.tnear = tnear;
    er.so = push ? shifted_origin(pos, w, 1.0f) : pos;
    return pdf_o;
}

// ------------------------------------------------------ camera shade ---
// Where a camera vertex's connections to the light subpath go: the wavefront
// queues each for k_shadow; the tail kernel tests it at once.
struct QueueSink {
    __device__ __forceinline__ void connect(const WaveArgs& A, int b, int k, V3 lpos, V3 pos, V3 lc)
    {
        const uint32_t sl = coalesced_append(&A.R.ctr[kCtrShadow + b]);
        float4* q = A.R.sq + 3 * (size_t)sl;
        q[0] = make_float4(lpos.x, lpos.y, lpos.z, __int_as_float(k));
        q[1] = make_float4(pos.x, pos.y, pos.z, 0.0f);
        q[2] = make_float4(lc.x, lc.y, lc.z, 0.0f);
    }
};

// Camera vertex b of path k, reached by the ray (ra, rb) with hit h: the
// escape term, the vertex's emission and connections, its throughput and the
// next ray.  True when the path goes on (next ray: origin so, direction O,
// tnear); er: the MIS estimator's environment ray (kMis).
template <bool kMis, typename Sink>
__device__ __forceinline__ bool camera_vertex(const WaveArgs& A, int b, int k, float4 ra, float4 rb, uint4 h, V3& so,
                                              V3& O, float& tnear, EnvRay& er, Sink& sink)
{
    const DevScene& S = A.S;
    bool push = false;
    tnear = ra.w;
    const V3 in = v3(rb.x, rb.y, rb.z);
    const bool first = b == 1;  // throughput 1, radiance 0 (not stored yet)
    const float4 tp4 = first ? make_float4(1.0f, 1.0f, 1.0f, 0.0f) : A.R.tp[k];
    const V3 tp = v3(tp4.x, tp4.y, tp4.z);
    if (h.x == kInvalid) {
        // escape: background x throughput when cp_len <= maxPathLength (:251-258)
        if (S.env.present && b <= A.max_len) {
            V3 bg = env_radiance(S.env, in);
            if (kMis && tp4.w > 0.0f) {  // the sampler's share (power heuristic) against env_connect
                const float pe = env_pdf(S.env, in);
                bg = bg * (tp4.w * tp4.w / (tp4.w * tp4.w + pe * pe));
            }
            float4 r = first ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : A.R.rad[k];
            r.x += bg.x * tp.x;
            r.y += bg.y * tp.y;
            r.z += bg.z * tp.z;
            A.R.rad[k] = r;
        } else if (first) {
            A.R.rad[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    } else {
        if (first) A.R.rad[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const PathCtx c = path_ctx(A, k);
        const uint32_t pixel = c.pixel, sample = c.sample;
        const DevMaterial& M = c.mats[__ldg(&S.insts[h.x].material)];
        const Surf sp = surface_point(S, h.x, h.y, __uint_as_float(h.z), __uint_as_float(h.w), true, &M);
        const PbrParams P = pbr_params(S, M, sp);
        const Rng4 u = rng4(c.seed, pixel, sample, (uint32_t)b, kStreamCamera);
        SampleInfo info;
        info.kind = -1;
        const V3 brdf = material_sample(S, M, P, sp, in, true, u, O, kMis ? &info : nullptr);
        const float ct = fabsf(dot(O, sp.nrm));
        const V3 tpn = v3(tp.x * brdf.x * ct, tp.y * brdf.y * ct, tp.z * brdf.z * ct);
        float mis_pdf = 0.0f;  // density of O for the next escape's MIS weight (0: weight 1)
        if (kMis && M.type == kMatPbr)
            mis_pdf = env_connect(A, b, c.seed, pixel, sample, pbr_bsdf_in(M, P, sp, in), sp.pos, sp.nrm,
                                  tp, O, info.kind, tnear, er);
        if (M.type == kMatPbr && M.emissive_on) {  // Rad += outFactor x emission (:171-173)
            const V3 e = pbr_emission(S, M, tex_hit(sp));
            float4 r = A.R.rad[k];
            r.x += tpn.x * e.x;
            r.y += tpn.y * e.y;
            r.z += tpn.z * e.z;
            A.R.rad[k] = r;
        }
        if (S.num_lights > 0) {
            const uint32_t meta = A.R.lmeta[k];
            const int lp_len = (int)(meta >> 16);
            const uint32_t li = meta & 0xFFFFu;
            const V3 outV = -in;
            for (int li_v = 0; li_v < lp_len && li_v + b <= A.max_len; ++li_v) {
                const size_t slot = (size_t)li_v * A.wave_cap + k;
                const float4 lp = li_v == 0 ? __ldg(S.light_pos + li) : A.R.lv_pos[slot];  // vertex 0: the light
                const V3 lPos = v3(lp.x, lp.y, lp.z);
                V3 lRad;
                const V3 LC = normalize(sp.pos - lPos);
                if (li_v == 0) {
                    const float4 I = __ldg(S.light_int + li);
                    const float4 L = __ldg(S.light_pos + li);
                    const V3 dd = sp.pos - lPos;
                    const float lsc = light_attenuation(A.atten_mode, A.min_dist, sqrtf(dot(dd, dd)), L.w);
                    const float f = A.light_scale * lsc;
                    lRad = v3(I.x * f, I.y * f, I.z * f);
                } else {
                    const float4 lr = A.R.lv_rad[slot];
                    lRad = v3(lr.x, lr.y, lr.z);
                }
                const float c = fabsf(dot(LC, sp.nrm));
                V3 lc = v3(lRad.x * c * tp.x, lRad.y * c * tp.y, lRad.z * c * tp.z);
                if (intensity(lc) < A.cut) continue;
                V3 f = material_eval(M, P, sp, LC, outV) * c;
                lc = v3(f.x * tp.x * lRad.x, f.y * tp.y * lRad.y, f.z * tp.z * lRad.z);
                if (intensity(lc) < A.cut) continue;
                sink.connect(A, b, k, lPos, sp.pos, lc);
            }
        }
        A.R.tp[k] = make_float4(tpn.x, tpn.y, tpn.z, mis_pdf);
        if (b < A.cam_bounces && (tpn.x != 0.0f || tpn.y != 0.0f || tpn.z != 0.0f)) {
            push = true;
            so = shifted_origin(sp.pos, O, 1.0f);
        }
    }
    return push;
}

// BDPTRenderer::computePath for the camera subpath (inv = true), vertex b, plus
// the escape term and the connections of computePaths (:251-298) at vertex b.
// kMis: the MIS estimator's environment connections (a separate instantiation,
// so the reference estimator's kernel carries none of their registers).  Four
// resident blocks of 256 (64 registers, 28 B of spills) hide more of the
// vertex-gather latency than three (72 registers): 37.9 vs 38.5 ms per frame.
// The MIS instantiation keeps three (it would spill 140 B at four).
template <bool kMis>
__global__ void __launch_bounds__(kShadeThreads, kMis ? 3 : 4) k_camera_shade(WaveArgs A, int b, const float4* rq_in,
                                                                 float4* rq_out)
{
    __shared__ BinScratch bins;
    const uint32_t n = A.R.ctr[kCtrCam + b];
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        bool push = false;
        V3 so = v3(0, 0, 0), O = v3(0, 0, 1);
        float tnear = 0.0f;
        int k = 0;
        EnvRay er;
        er.push = false;
        er.w = v3(0.0f, 0.0f, 1.0f);
        if (i < n) {
            const float4 ra = rq_in[2 * (size_t)i], rb = rq_in[2 * (size_t)i + 1];
            k = __float_as_int(rb.w);
            QueueSink qs;
            push = camera_vertex<kMis>(A, b, k, ra, rb, A.R.hits[i], so, O, tnear, er, qs);
        }
        const uint32_t slot = block_append_binned(&A.R.ctr[kCtrCam + b + 1], push, direction_bin(O), bins);
        if (push) {
            rq_out[2 * (size_t)slot] = make_float4(so.x, so.y, so.z, tnear);
            rq_out[2 * (size_t)slot + 1] = make_float4(O.x, O.y, O.z, __int_as_float(k));
        }
        if (kMis) {  // environment rays grouped by direction like the next-bounce rays
            const uint32_t es = block_append_binned(&A.R.ctr[kCtrEnv + b], er.push, direction_bin(er.w), bins);
            if (er.push) {
                float4* q = A.env_q + 3 * (size_t)es;
                q[0] = make_float4(er.so.x, er.so.y, er.so.z, __int_as_float(k));
                q[1] = make_float4(er.w.x, er.w.y, er.w.z, er.tnear);
                q[2] = make_float4(er.c.x, er.c.y, er.c.z, 0.0f);
            }
        }
    }
}

// ------------------------------------------------------------ shadow ---
// BDPTRenderer::isConnected (BDPTRenderer.cpp:208-235): whether vertex A sees
// vertex B.  Without alpha-masked materials the closest-hit query stops at a
// hit well short of B, which already decides "not connected".
template <bool kMasked>
__device__ __forceinline__ bool is_connected(const DevScene& S, const uint32_t* items, V3 A, V3 B, TraceStack& st,
                                             TraceCounters& tc, uint32_t root)
{
    bool connected = true;
    V3 dir = B - A;
    const float len = sqrtf(dot(dir, dir));
    float maxsz = max_abs(A, 1.0f);
    float safeD = 2.0f * kEpsAcc * kEps * maxsz;
    if (!(len <= safeD)) {
        dir = v3(dir.x / len, dir.y / len, dir.z / len);
        float tnear = safeD;
        const float tfar = len + (0.1f * len > safeD ? 0.1f * len : safeD);
        const float sb = 10.0f * kEps * max_abs(B, 1.0f);
        RayHit h;
        bool hit;
        if (kMasked) {
            hit = scene_intersect(S, items, A, dir, tnear, tfar, h, st, tc, root);
        } else {
            // any hit this far short of B is farther than sb from it (the
            // margin is ~800 ulps of the coordinates, far above the error of
            // the hit's surface position), so it decides: not connected,
            // whichever hit is the closest.  Hits near B get the exact test.
            const float margin = 1.0e-4f * fmaxf(maxsz, max_abs(B, 1.0f)) + 2.0f * sb;
            hit = trace_closest_or_below(S, items, A, dir, tnear, tfar, len - margin, h, st, tc, root);
            if (hit && h.t < len - margin) {
                hit = false;
                connected = false;
            }
        }
        if (hit) {
            const Surf sp = surface_point(S, h.inst, h.prim, h.u, h.v, false);
            const V3 dd = sp.pos - B;
            const float sd = dot(dd, dd);
            connected = sd <= sb * sb;
        }
    }
    return connected;
}

// whether the environment ray (shifted origin so, direction w, the path's
// tnear) escapes: no hit at all
template <bool kMasked>
__device__ __forceinline__ bool env_escapes(const DevScene& S, const uint32_t* items, V3 so, V3 w, float tnear,
                                            TraceStack& st, TraceCounters& tc, uint32_t root)
{
    RayHit h;
    return kMasked ? !scene_intersect(S, items, so, w, tnear, kFltMax, h, st, tc, root)
                   : !trace_any(S, items, so, w, tnear, kFltMax, st, tc, root);
}

// kEnv = false: the vertex connections (records: end points A, B and the
// contribution).  kEnv = true: the MIS estimator's environment rays (records:
// shifted origin, direction and tnear, contribution), which reach the
// environment when a sampled ray in that direction would escape: no hit at
// all.  Without alpha-masked materials that is an any-hit query; with them
// sceneIntersect's closest hit and retries decide, as in k_extend.
template <bool kEnv, bool kMasked>
__global__ void __launch_bounds__(kTraceThreads, kTraceMinBlocks) k_shadow(DevScene S, const uint32_t* items, const float4* sq,
                                                          const uint32_t* count, uint32_t* work, float4* rad,
                                                          unsigned long long* stats, const DevJob* jobs,
                                                          const uint32_t* path_job)
{
    __shared__ uint2 sstack[kStackShared * kTraceThreads];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kTraceThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    const uint32_t n = *count;
    const int lane = threadIdx.x & 31;
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
        const float4 q0 = sq[3 * (size_t)i], q1 = sq[3 * (size_t)i + 1], q2 = sq[3 * (size_t)i + 2];
        const V3 A = v3(q0.x, q0.y, q0.z), B = v3(q1.x, q1.y, q1.z);
        const int k = __float_as_int(q0.w);
        const uint32_t root = path_root(jobs, path_job, k);
        const bool connected = kEnv ? env_escapes<kMasked>(S, items, A, B, q1.w, st, tc, root)
                                    : is_connected<kMasked>(S, items, A, B, st, tc, root);
        if (connected) {
            atomicAdd(&rad[k].x, q2.x);
            atomicAdd(&rad[k].y, q2.y);
            atomicAdd(&rad[k].z, q2.z);
        }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats[kStatShadow], (unsigned long long)n);
    uint32_t nodes = tc.nodes, tris = tc.tris;
    for (int o = 16; o; o >>= 1) {
        nodes += __shfl_xor_sync(0xFFFFFFFFu, nodes, o);
        tris += __shfl_xor_sync(0xFFFFFFFFu, tris, o);
    }
    const bool ov = __any_sync(0xFFFFFFFFu, st.overflow);
    if (lane == 0 && nodes) {
        atomicAdd(&stats[kStatShadowNodes], (unsigned long long)nodes);
        atomicAdd(&stats[kStatShadowTris], (unsigned long long)tris);
    }
    if (lane == 0 && ov) atomicAdd(&stats[kStatOverflow], 1ull);
}

// ------------------------------------------------------- camera tail ---
// End of a tail kernel that ran: the last block to finish (every block has
// read the queue count by then) sets the count to zero, so that the bounce's
// wavefront kernels find nothing to do, and records the bounce.
__device__ __forceinline__ void tail_finish(const WaveArgs& A, uint32_t* count, int stat, int b0)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&A.R.ctr[kCtrTailDone], 1u) == gridDim.x - 1u) {
            *count = 0u;
            A.R.ctr[kCtrTailDone] = 0u;
            atomicMax(&A.R.stats[stat], (unsigned long long)b0);
        }
    }
}

// A camera vertex's connections tested at once (the tail kernel's sink):
// the path's radiance is this thread's alone while the tail runs.
template <bool kMasked>
struct TestSink {
    const uint32_t* items;
    TraceStack* st;
    TraceCounters* tc;
    uint32_t root;
    uint32_t* tests;
    __device__ __forceinline__ void connect(const WaveArgs& A, int b, int k, V3 lpos, V3 pos, V3 lc)
    {
        ++*tests;
        if (is_connected<kMasked>(A.S, items, lpos, pos, *st, *tc, root)) {
            float4 r = A.R.rad[k];
            r.x += lc.x;
            r.y += lc.y;
            r.z += lc.z;
            A.R.rad[k] = r;
        }
    }
};

// Camera bounces b0 .. camera bounces in one launch: each thread takes a path
// alive at bounce b0 (queue rq_in) and runs it to its end: extension ray,
// vertex (camera_vertex, as k_camera_shade), connections and MIS environment
// ray tested at once, the next ray kept in registers.  The additions to the
// path's radiance come in the wavefront's order (escape / emission, then
// connections, then the environment ray, bounce by bounce).
template <bool kMis, bool kMasked>
__global__ void __launch_bounds__(kTraceThreads, 4) k_camera_tail(WaveArgs A, int b0, const float4* rq_in, uint32_t* work,
                                                                  const DevJob* jobs)
{
    __shared__ uint2 sstack[kStackShared * kTraceThreads];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kTraceThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    uint32_t rays = 0, tests = 0;
    const DevScene& S = A.S;
    const uint32_t n = A.R.ctr[kCtrCam + b0];
    if (n == 0u || n > kTailPaths) return;  // the same decision in every block
    const int lane = threadIdx.x & 31;
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            float4 ra = rq_in[2 * (size_t)i], rb = rq_in[2 * (size_t)i + 1];
            const int k = __float_as_int(rb.w);
            const uint32_t root = path_root(jobs, A.path_job, k);
            TestSink<kMasked> sink{A.items, &st, &tc, root, &tests};
            for (int b = b0; b <= A.cam_bounces; ++b) {
                float tn = ra.w;
                RayHit hh;
                ++rays;
                uint4 h = make_uint4(kInvalid, kInvalid, 0u, 0u);
                if (scene_intersect(S, A.items, v3(ra.x, ra.y, ra.z), v3(rb.x, rb.y, rb.z), tn, kFltMax, hh, st, tc, root))
                    h = make_uint4(hh.inst, hh.prim, __float_as_uint(hh.u), __float_as_uint(hh.v));
                ra.w = tn;
                V3 so = v3(0.0f, 0.0f, 0.0f), O = v3(0.0f, 0.0f, 1.0f);
                float tnear = 0.0f;
                EnvRay er;
                er.push = false;
                const bool more = camera_vertex<kMis>(A, b, k, ra, rb, h, so, O, tnear, er, sink);
                if (kMis && er.push) {
                    ++tests;
                    if (env_escapes<kMasked>(S, A.items, er.so, er.w, er.tnear, st, tc, root)) {
                        float4 r = A.R.rad[k];
                        r.x += er.c.x;
                        r.y += er.c.y;
                        r.z += er.c.z;
                        A.R.rad[k] = r;
                    }
                }
                if (!more) break;
                ra = make_float4(so.x, so.y, so.z, tnear);
                rb = make_float4(O.x, O.y, O.z, __int_as_float(k));
            }
        }
    }
    uint32_t nodes = tc.nodes, tris = tc.tris;
    for (int o = 16; o; o >>= 1) {
        nodes += __shfl_xor_sync(0xFFFFFFFFu, nodes, o);
        tris += __shfl_xor_sync(0xFFFFFFFFu, tris, o);
        rays += __shfl_xor_sync(0xFFFFFFFFu, rays, o);
        tests += __shfl_xor_sync(0xFFFFFFFFu, tests, o);
    }
    const bool ov = __any_sync(0xFFFFFFFFu, st.overflow);
    if (lane == 0) {
        atomicAdd(&A.R.stats[kStatExt], (unsigned long long)rays);
        atomicAdd(&A.R.stats[kStatShadow], (unsigned long long)tests);
        atomicAdd(&A.R.stats[kStatTailNodes], (unsigned long long)nodes);
        atomicAdd(&A.R.stats[kStatTailTris], (unsigned long long)tris);
        if (ov) atomicAdd(&A.R.stats[kStatOverflow], 1ull);
    }
    tail_finish(A, &A.R.ctr[kCtrCam + b0], kStatTailCam, b0);
}

// -------------------------------------------------------------- film ---
// PinholeCamera::hit (PinholeCamera.cpp:97-108), FP64 accumulation
// Float-float accumulator (value = hi + lo, |lo| <= ulp(hi) / 2): sums of a
// few hundred FP32 samples kept to about 2^-44 relative, in FP32 arithmetic
// (FP64 throughput is a small fraction of FP32 on this GPU).  ff_add is
// Knuth's TwoSum of the high parts with the low parts folded in.  Squares of
// samples beyond 1.8e19 overflow to infinity (the FP32 range).
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    if (fabsf(s) > kFltMax) return FF{s, 0.0f};  // an infinite sample stays infinite (not NaN)
    return FF{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}
// x * x exactly as a float-float (the FMA gives the rounding error of the product)
__device__ __forceinline__ FF ff_sqr(float x)
{
    const float p = __fmul_rn(x, x);
    return FF{p, fmaf(x, x, -p)};
}

// PinholeCamera::hit for every path of the wave, without atomics: each pixel
// of the wave gets an aligned group of `group` lanes (a power of two), lane j
// sums samples j, j + group, ... of the pixel's paths in this wave, the group
// reduces by xor butterfly and its first lane adds the totals to the FP64 film.
// No other thread of the launch touches that pixel and the order of every
// addition is fixed, so the film is deterministic for a given wave split.
__global__ void __launch_bounds__(kShadeThreads) k_film(WaveArgs A, int group, double* sum, double* sumsq,
                                                        uint32_t* count)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = threadIdx.x & (group - 1);
    const int64_t spp = A.spp;
    const int64_t g_begin = A.wave_base, g_end = A.wave_base + A.wave_n;
    const int64_t p = (int64_t)A.base_q + (t >> (__ffs(group) - 1));  // group is a power of two
    const bool live = p <= (int64_t)A.last_pixel;
    // the pixel's paths, film and index in it (batch: p is a pixel of the
    // concatenated job films)
    int64_t first_path = p * spp, npp = spp, lp = p;
    double* fsum = sum;
    double* fsq = sumsq;
    uint32_t* fcnt = count;
    if (A.num_jobs > 0 && live) {
        int lo = 0, hi = A.num_jobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((int64_t)A.jobs[mid].pixel_base <= p)
                lo = mid;
            else
                hi = mid - 1;
        }
        const DevJob& J = A.jobs[lo];
        lp = p - (int64_t)J.pixel_base;
        npp = J.spp;
        first_path = J.path_base + lp * npp;
        fsum = J.sum;
        fsq = J.sumsq;
        fcnt = J.count;
    }
    uint32_t c = 0;
    FF v[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) v[q] = FF{0.0f, 0.0f};
    // squares only for a film with a variance channel (the same for all lanes
    // of a pixel's group)
    const bool squares = fsq != nullptr;
    if (live) {
        const int64_t g0 = max(first_path, g_begin), g1 = min(first_path + npp, g_end);
        for (int64_t g = g0 + j; g < g1; g += group) {
            const float4 r = A.R.rad[g - g_begin];
            v[0] = ff_add(v[0], FF{r.x, 0.0f});
            v[1] = ff_add(v[1], FF{r.y, 0.0f});
            v[2] = ff_add(v[2], FF{r.z, 0.0f});
            if (squares) {
                v[3] = ff_add(v[3], ff_sqr(r.x));
                v[4] = ff_add(v[4], ff_sqr(r.y));
                v[5] = ff_add(v[5], ff_sqr(r.z));
            }
            ++c;
        }
    }
    const int nq = __any_sync(0xFFFFFFFFu, squares) ? 6 : 3;
    for (int off = group >> 1; off > 0; off >>= 1) {
        c += __shfl_xor_sync(0xFFFFFFFFu, c, off);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            if (q >= nq) break;
            FF o;
            o.hi = __shfl_xor_sync(0xFFFFFFFFu, v[q].hi, off);
            o.lo = __shfl_xor_sync(0xFFFFFFFFu, v[q].lo, off);
            v[q] = (j & off) ? ff_add(o, v[q]) : ff_add(v[q], o);  // same operand order on both lanes
        }
    }
    if (!live || j != 0 || c == 0) return;
    double* ps = fsum + 3 * (size_t)lp;
#pragma unroll
    for (int q = 0; q < 3; ++q) ps[q] += (double)v[q].hi + (double)v[q].lo;
    if (fsq) {
        double* pq = fsq + 3 * (size_t)lp;
#pragma unroll
        for (int q = 0; q < 3; ++q) pq[q] += (double)v[3 + q].hi + (double)v[3 + q].lo;
    }
    fcnt[lp] += c;
}

// ------------------------------------------------------------ ID pass ---
__global__ void k_ids(DevScene S, const uint32_t* items, omv_camera cam, const float* jitter, uint64_t seed,
                      omv_hit* out, uint32_t* gprim, const uint32_t* face_prefix)
{
    __shared__ uint2 sstack[kStackShared * kTraceThreads];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kTraceThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    const int npix = cam.width * cam.height;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float ux, uy;
    if (jitter) {
        ux = jitter[2 * (size_t)p];
        uy = jitter[2 * (size_t)p + 1];
    } else {
        Rng4 r = rng4(seed, (uint32_t)p, 0u, 0u, kStreamCamera);
        ux = r.u[0];
        uy = r.u[1];
    }
    V3 O, R;
    camera_ray(cam, p % cam.width, p / cam.width, ux, uy, O, R);
    const V3 so = shifted_origin(O, R, 1.0f);
    float tnear = 0.0f;
    RayHit h;
    omv_hit o;
    if (scene_intersect(S, items, so, R, tnear, kFltMax, h, st, tc)) {
        const DevInstance* I = S.insts + h.inst;
        o.inst = h.inst;
        o.geom = I->mesh;
        o.prim = h.prim;
        o.material = I->material;
        o.t = h.t;
        o.u = h.u;
        o.v = h.v;
        if (gprim) gprim[p] = face_prefix[I->mesh] + h.prim;
    } else {
        o.inst = o.geom = o.prim = o.material = kInvalid;
        o.t = o.u = o.v = 0.0f;
        if (gprim) gprim[p] = kInvalid;
    }
    o.pad = 0;
    out[p] = o;
}

__global__ void k_trace_rays(DevScene S, const uint32_t* items, int64_t n, const float* rays, omv_hit* out)
{
    __shared__ uint2 sstack[kStackShared * kTraceThreads];
    TraceStack st;
    st.sh = sstack + threadIdx.x;
    st.stride = kTraceThreads;
    st.overflow = 0;
    TraceCounters tc{0u, 0u};
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + 8 * i;
    float tnear = r[3];
    RayHit h;
    omv_hit o;
    if (scene_intersect(S, items, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), tnear, r[7], h, st, tc)) {
        const DevInstance* I = S.insts + h.inst;
        o.inst = h.inst;
        o.geom = I->mesh;
        o.prim = h.prim;
        o.material = I->material;
        o.t = h.t;
        o.u = h.u;
        o.v = h.v;
    } else {
        o.inst = o.geom = o.prim = o.material = kInvalid;
        o.t = o.u = o.v = 0.0f;
    }
    o.pad = 0;
    out[i] = o;
}

__global__ void k_env(DevEnv env, int64_t n, const float* dirs, float* rgb)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 v = env.present ? env_radiance(env, v3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2])) : v3(0, 0, 0);
    rgb[3 * i] = v.x;
    rgb[3 * i + 1] = v.y;
    rgb[3 * i + 2] = v.z;
}

inline int grid_for(int64_t n, int t) { return (int)std::max<int64_t>(1, (n + t - 1) / t); }

}  // namespace

// -------------------------------------------------------------- host ---

namespace {

// Byte offsets of one wave's arrays inside a single scratch block (each array
// starts on a 256-byte boundary).
struct ScratchLayout {
    size_t tp, rad, ltp, lrad, lmeta, lvp, lvr, rq0, rq1, hits, pjob, sq, ctr, stats, bytes;
};

ScratchLayout scratch_layout(int64_t wave_cap, int light_slots, int shadow_slots)
{
    const size_t W = (size_t)wave_cap;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    ScratchLayout L;
    L.tp = take(W * 16);
    L.rad = take(W * 16);
    L.ltp = take(W * 16);
    L.lrad = take(W * 16);
    L.lmeta = take(W * 4);
    L.lvp = take((size_t)light_slots * W * 16);
    L.lvr = take((size_t)light_slots * W * 16);
    L.rq0 = take(W * 32);
    L.rq1 = take(W * 32);
    L.hits = take(W * 16);
    L.pjob = take(W * 4);
    L.sq = take((size_t)shadow_slots * W * 48 + 48);
    L.ctr = take(kMaxCounters * 4);
    L.stats = take(16 * 8);
    L.bytes = off;
    return L;
}

// Scratch bytes of one path: tp rad ltp lrad (16 B each), lmeta 4, light
// vertices 32 per slot, two ray-queue entries 64, hit 16, batch job 4, shadow
// entries 48 per slot (each array is further rounded up to 256 bytes).
size_t path_scratch_bytes(int light_slots, int shadow_slots)
{
    return 68 + 32 * (size_t)light_slots + 84 + 48 * (size_t)shadow_slots;
}

void carve_scratch(RenderScratch& R, void* base, int64_t wave_cap, int light_slots, int shadow_slots)
{
    const ScratchLayout L = scratch_layout(wave_cap, light_slots, shadow_slots);
    char* b = static_cast<char*>(base);
    R.base = base;
    R.bytes = L.bytes;
    R.wave_cap = wave_cap;
    R.light_slots = light_slots;
    R.shadow_slots = shadow_slots;
    R.tp = (float4*)(b + L.tp);
    R.rad = (float4*)(b + L.rad);
    R.ltp = (float4*)(b + L.ltp);
    R.lrad = (float4*)(b + L.lrad);
    R.lmeta = (uint32_t*)(b + L.lmeta);
    R.lv_pos = (float4*)(b + L.lvp);
    R.lv_rad = (float4*)(b + L.lvr);
    R.rq[0] = (float4*)(b + L.rq0);
    R.rq[1] = (float4*)(b + L.rq1);
    R.hits = (uint4*)(b + L.hits);
    R.path_job = (uint32_t*)(b + L.pjob);
    R.sq = (float4*)(b + L.sq);
    R.ctr = (uint32_t*)(b + L.ctr);
    R.stats = (unsigned long long*)(b + L.stats);
}

// Validated sizes of one frame: paths, wave capacity and vertex slots.
struct FramePlan {
    int64_t npix, total, cap;
    int light_slots, shadow_slots;
    bool lights;
};

// the MIS estimator (environment connections) runs when asked for and the
// scene has an environment
bool mis_on(const SceneHost& s, const omv_params& p)
{
    if (p.estimator != OMV_ESTIMATOR_REFERENCE && p.estimator != OMV_ESTIMATOR_MIS)
        throw ArgError("unknown estimator");
    return p.estimator == OMV_ESTIMATOR_MIS && s.dev.env.present;
}

// `cap` is the requested wave size (0: `default_cap`), clamped to the frame.
FramePlan plan_frame(const SceneHost& s, const omv_camera& cam, const omv_params& p, int64_t default_cap)
{
    if (cam.width <= 0 || cam.height <= 0) throw ArgError("camera resolution must be positive");
    if (p.samples_per_pixel < 0 || p.camera_bounces < 0 || p.light_bounces < 0)
        throw ArgError("negative sample or bounce count");
    if (p.camera_bounces > 60 || p.light_bounces > 60) throw ArgError("at most 60 bounces are supported");
    FramePlan P;
    P.npix = (int64_t)cam.width * cam.height;
    P.total = P.npix * p.samples_per_pixel;
    if (P.npix > (int64_t)0x7FFFFFFF) throw ArgError("image too large");
    P.cap = p.wave_paths > 0 ? p.wave_paths : default_cap;
    P.cap = std::min<int64_t>(P.cap, std::max<int64_t>(P.total, 1));
    P.lights = s.num_lights > 0;
    P.light_slots = P.lights ? p.light_bounces + 1 : 1;
    P.shadow_slots = std::max(1, (P.lights ? P.light_slots : 0) + (mis_on(s, p) ? 1 : 0));
    return P;
}

// A batch as the wave loop sees it: the device job table and its host copy.
struct BatchPlan {
    const DevJob* d_jobs;
    const std::vector<DevJob>* h_jobs;
    int min_spp;
};

// pixel of the concatenated job films that holds global path g
uint32_t batch_global_pixel(const std::vector<DevJob>& jobs, int64_t g)
{
    size_t lo = 0, hi = jobs.size() - 1;
    while (lo < hi) {
        const size_t mid = (lo + hi + 1) / 2;
        if (jobs[mid].path_base <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return jobs[lo].pixel_base + (uint32_t)((g - jobs[lo].path_base) / jobs[lo].spp);
}

// The wave loop of one frame (or, with `batch`, of all jobs of a batch) on
// scratch R (at least P.cap paths).  With `events` false no CUDA event is
// created: no frame or kernel timing, and `stats` must be null.
void run_waves(SceneHost& s, RenderScratch& R, const FramePlan& P, const omv_camera& cam, const omv_params& p,
               double* d_sum, double* d_sumsq, uint32_t* d_count, cudaStream_t st, omv_stats* stats, bool events,
               const BatchPlan* batch = nullptr)
{
    const int64_t total = P.total, npix = P.npix, cap = P.cap;
    const bool lights = P.lights;
    const bool mis = mis_on(s, p);
    if (mis) ensure_env_sampler(s);
    bool masked = false;  // material sets keep which materials are masked
    for (const DevMaterial& m : s.h_mats) masked = masked || m.masked != 0;
    OMV_CUDA(cudaMemsetAsync(R.stats, 0, 16 * 8, st));
    WaveArgs A;
    A.S = s.dev;
    A.items = s.tlas_items;
    A.cam = cam;
    A.seed = p.seed;
    A.wave_cap = (int32_t)cap;
    A.npix = (int32_t)npix;
    A.spp = p.samples_per_pixel;
    A.spp_div = make_fastdiv((uint32_t)std::max(1, p.samples_per_pixel));  // used by single frames only
    A.width_div = make_fastdiv((uint32_t)std::max(1, cam.width));
    A.sample_offset = p.sample_offset;
    A.cam_bounces = p.camera_bounces;
    A.light_bounces = p.light_bounces;
    A.max_len = p.max_path_length;
    A.atten_mode = p.light_distance_attenuation;
    A.light_scale = p.light_scale;
    A.min_dist = p.light_min_distance;
    A.cut = p.ray_cut_value;
    A.R = R;
    A.env_q = mis ? R.sq + 3 * (size_t)R.wave_cap * (size_t)(R.shadow_slots - 1) : nullptr;
    A.jobs = batch ? batch->d_jobs : nullptr;
    A.num_jobs = batch ? (int32_t)batch->h_jobs->size() : 0;
    A.path_job = R.path_job;
    int occ_t = 0, occ_s = 0;
    OMV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_t, k_extend, kTraceThreads, 0));
    // threads per block of the shading-side kernels: 256, or a batch's
    // autotuned choice (a multiple of 32 up to 256)
    const int sth = batch && s.batch_shade_threads > 0 ? s.batch_shade_threads : kShadeThreads;
    OMV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, mis ? k_camera_shade<true> : k_camera_shade<false>,
                                                           sth, 0));
    const int trace_grid = std::max(1, occ_t) * s.num_sms;
    int occ_tail = 0;
    OMV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_tail, k_camera_tail<false, false>, kTraceThreads, 0));
    const int tail_grid = std::max(1, occ_tail) * s.num_sms;
    // a batch over a group of scenes: every ray starts at its own scene's top-level tree
    const DevJob* gjobs = batch && s.parts.size() > 1 ? batch->d_jobs : nullptr;
    const int shade_grid = std::max(1, occ_s) * s.num_sms;
    int64_t launches = 0;
    // optional per-launch events around the closest-hit kernels
    std::vector<cudaEvent_t> ext_ev, sh_ev, tail_ev;
    const bool time_kernels = events && p.time_kernels;
    auto timed = [&](std::vector<cudaEvent_t>& pool) -> cudaEvent_t {
        cudaEvent_t e;
        OMV_CUDA(cudaEventCreate(&e));
        OMV_CUDA(cudaEventRecord(e, st));
        pool.push_back(e);
        return e;
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (events) {
        OMV_CUDA(cudaEventCreate(&e0));
        OMV_CUDA(cudaEventCreate(&e1));
        OMV_CUDA(cudaEventRecord(e0, st));
    }
    for (int64_t wb = 0; wb < total; wb += cap) {
        const NvtxRange wave_range("omv wave");
        A.wave_base = wb;
        A.wave_n = (int32_t)std::min<int64_t>(cap, total - wb);
        if (batch) {
            A.base_q = batch_global_pixel(*batch->h_jobs, wb);
            A.base_r = 0;
            A.last_pixel = batch_global_pixel(*batch->h_jobs, wb + A.wave_n - 1);
        } else {
            A.base_q = (uint32_t)(wb / p.samples_per_pixel);
            A.base_r = (uint32_t)(wb % p.samples_per_pixel);
            A.last_pixel = (uint32_t)((wb + A.wave_n - 1) / p.samples_per_pixel);
        }
        OMV_CUDA(cudaMemsetAsync(R.ctr, 0, kMaxCounters * 4, st));
        int work = 0;
        if (batch) {
            k_job_ids<<<grid_for(A.wave_n, sth), sth, 0, st>>>(A);
            ++launches;
        }
        if (lights) {
            const NvtxRange light_range("omv light subpaths");
            k_light_gen<<<grid_for(A.wave_n, sth), sth, 0, st>>>(A);
            ++launches;
            for (int b = 1; b <= p.light_bounces; ++b) {
                const NvtxRange bounce_range(bounce_name(b));
                float4* in = R.rq[1];
                float4* out = R.rq[0];
                if (b % 2 == 0) std::swap(in, out);
                if (time_kernels) timed(ext_ev);
                k_extend<<<trace_grid, kTraceThreads, 0, st>>>(s.dev, s.tlas_items, in, R.hits,
                                                               R.ctr + kCtrLight + b, R.ctr + kCtrWork + work++,
                                                               R.stats, kStatLight, gjobs, R.path_job);
                if (time_kernels) timed(ext_ev);
                k_light_shade<<<shade_grid, sth, 0, st>>>(A, b, in, out);
                launches += 2;
            }
        }
        {
            const NvtxRange camera_range("omv camera subpaths");
            k_camera_gen<<<grid_for(A.wave_n, sth), sth, 0, st>>>(A);
            ++launches;
            for (int b = 1; b <= p.camera_bounces; ++b) {
                const NvtxRange bounce_range(bounce_name(b));
                float4* in = R.rq[(b + 1) % 2];
                float4* out = R.rq[b % 2];
                if (!lights && b >= kTailMin) {  // the remaining bounces in one launch, once few paths are alive
                    uint32_t* tw = R.ctr + kCtrTailWorkCam;
                    if (time_kernels) timed(tail_ev);
                    if (mis)
                        masked ? k_camera_tail<true, true><<<tail_grid, kTraceThreads, 0, st>>>(A, b, in, tw, gjobs)
                               : k_camera_tail<true, false><<<tail_grid, kTraceThreads, 0, st>>>(A, b, in, tw, gjobs);
                    else
                        masked ? k_camera_tail<false, true><<<tail_grid, kTraceThreads, 0, st>>>(A, b, in, tw, gjobs)
                               : k_camera_tail<false, false><<<tail_grid, kTraceThreads, 0, st>>>(A, b, in, tw, gjobs);
                    if (time_kernels) timed(tail_ev);
                    ++launches;
                }
                if (time_kernels) timed(ext_ev);
                k_extend<<<trace_grid, kTraceThreads, 0, st>>>(s.dev, s.tlas_items, in, R.hits, R.ctr + kCtrCam + b,
                                                               R.ctr + kCtrWork + work++, R.stats, kStatExt, gjobs,
                                                               R.path_job);
                if (time_kernels) timed(ext_ev);
                if (mis)
                    k_camera_shade<true><<<shade_grid, sth, 0, st>>>(A, b, in, out);
                else
                    k_camera_shade<false><<<shade_grid, sth, 0, st>>>(A, b, in, out);
                launches += 2;
                if (lights) {
                    if (time_kernels) timed(sh_ev);
                    if (masked)
                        k_shadow<false, true><<<trace_grid, kTraceThreads, 0, st>>>(s.dev, s.tlas_items, R.sq, R.ctr + kCtrShadow + b,
                                                                          R.ctr + kCtrWork + work++, R.rad, R.stats, gjobs, R.path_job);
                    else
                        k_shadow<false, false><<<trace_grid, kTraceThreads, 0, st>>>(s.dev, s.tlas_items, R.sq, R.ctr + kCtrShadow + b,
                                                                          R.ctr + kCtrWork + work++, R.rad, R.stats, gjobs, R.path_job);
                    if (time_kernels) timed(sh_ev);
                    ++launches;
                }
                if (mis) {
                    if (time_kernels) timed(sh_ev);
                    if (masked)
                        k_shadow<true, true><<<trace_grid, kTraceThreads, 0, st>>>(s.dev, s.tlas_items, A.env_q, R.ctr + kCtrEnv + b,
                                                                         R.ctr + kCtrWork + work++, R.rad, R.stats, gjobs, R.path_job);
                    else
                        k_shadow<true, false><<<trace_grid, kTraceThreads, 0, st>>>(s.dev, s.tlas_items, A.env_q, R.ctr + kCtrEnv + b,
                                                                         R.ctr + kCtrWork + work++, R.rad, R.stats, gjobs, R.path_job);
                    if (time_kernels) timed(sh_ev);
                    ++launches;
                }
            }
        }
        {
            const NvtxRange film_range("omv film");
            // about 8 samples per lane: group = power of two <= spp / 8, in [1, 32]
            const int64_t spp = batch ? batch->min_spp : p.samples_per_pixel;
            int group = 1;
            while (group < 32 && group * 16 <= spp) group *= 2;
            const int64_t pixels = (int64_t)A.last_pixel - (int64_t)A.base_q + 1;
            k_film<<<grid_for(pixels * group, sth), sth, 0, st>>>(A, group, d_sum, d_sumsq,
                                                                                     d_count);
            ++launches;
        }
        OMV_CUDA(cudaGetLastError());
    }
    if (!events) {
        OMV_CUDA(cudaGetLastError());
        return;
    }
    OMV_CUDA(cudaEventRecord(e1, st));
    if (stats) {
        unsigned long long h[16];
        OMV_CUDA(cudaMemcpyAsync(h, R.stats, sizeof(h), cudaMemcpyDeviceToHost, st));
        OMV_CUDA(cudaEventSynchronize(e1));
        OMV_CUDA(cudaStreamSynchronize(st));
        float ms = 0.0f;
        OMV_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        stats->paths = total;
        stats->extension_rays = (int64_t)h[kStatExt];
        stats->shadow_rays = (int64_t)h[kStatShadow];
        stats->light_rays = (int64_t)h[kStatLight];
        stats->render_ms = ms;
        stats->kernel_launches = launches;
        stats->nodes_visited = (int64_t)h[kStatNodes];
        stats->triangles_tested = (int64_t)h[kStatTris];
        stats->stack_overflows = (int64_t)h[kStatOverflow];
        stats->shadow_nodes_visited = (int64_t)h[kStatShadowNodes];
        stats->shadow_triangles_tested = (int64_t)h[kStatShadowTris];
        stats->tail_nodes_visited = (int64_t)h[kStatTailNodes];
        stats->tail_triangles_tested = (int64_t)h[kStatTailTris];
        stats->tail_bounce = (int64_t)h[kStatTailCam];
        auto sum_pairs = [](std::vector<cudaEvent_t>& ev) {
            double t = 0.0;
            for (size_t i = 0; i + 1 < ev.size(); i += 2) {
                float x = 0.0f;
                cudaEventElapsedTime(&x, ev[i], ev[i + 1]);
                t += x;
            }
            return t;
        };
        stats->extend_ms = sum_pairs(ext_ev);
        stats->extend_launches = (int64_t)ext_ev.size() / 2;
        stats->shadow_ms = sum_pairs(sh_ev);
        stats->shadow_launches = (int64_t)sh_ev.size() / 2;
        stats->tail_ms = sum_pairs(tail_ev);
    } else if (!ext_ev.empty() || !sh_ev.empty() || !tail_ev.empty()) {
        OMV_CUDA(cudaStreamSynchronize(st));
    }
    for (auto e : ext_ev) cudaEventDestroy(e);
    for (auto e : sh_ev) cudaEventDestroy(e);
    for (auto e : tail_ev) cudaEventDestroy(e);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

}  // namespace

static void ensure_scratch(SceneHost& s, int64_t wave_cap, int light_slots, int shadow_slots)
{
    RenderScratch& R = s.scratch;
    if (R.base && R.wave_cap >= wave_cap && R.light_slots >= light_slots && R.shadow_slots >= shadow_slots) return;
    if (R.base) {
        OMV_CUDA(cudaStreamSynchronize(s.stream));
        cudaFree(R.base);
        R = RenderScratch{};
        if (s.batch_graph) {  // it refers to the old scratch
            cudaGraphExecDestroy(s.batch_graph);
            s.batch_graph = nullptr;
            s.batch_key.clear();
        }
    }
    void* base = nullptr;
    OMV_CUDA(cudaMalloc(&base, scratch_layout(wave_cap, light_slots, shadow_slots).bytes));
    carve_scratch(R, base, wave_cap, light_slots, shadow_slots);
}

// Default wave scratch: up to 32 GiB (and at most half of the free device
// memory), enough for a full-HD frame at 64 spp in one wave.  Every wave pays
// the latency of its last, nearly empty bounces once, so fewer waves are faster.
constexpr size_t kWaveScratchBudget = (size_t)32 << 30;

void render_frame(SceneHost& s, const omv_camera& cam, const omv_params& p, double* d_sum, double* d_sumsq,
                  uint32_t* d_count, cudaStream_t st, omv_stats* stats)
{
    FramePlan P = plan_frame(s, cam, p, 1);
    if (p.wave_paths <= 0) {
        size_t free_b = 0, total_b = 0;
        OMV_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const size_t budget = std::min(kWaveScratchBudget, (free_b + s.scratch.bytes) / 2);
        const int64_t fit = (int64_t)(budget / path_scratch_bytes(P.light_slots, P.shadow_slots));
        P.cap = std::max<int64_t>(1, std::min<int64_t>({fit, std::max<int64_t>(P.total, 1), (int64_t)0x7FFFFFFF}));
    }
    ensure_scratch(s, P.cap, P.light_slots, P.shadow_slots);
    run_waves(s, s.scratch, P, cam, p, d_sum, d_sumsq, d_count, st, stats, true);
}

// ------------------------------------------------------------- batches ---

namespace {

// Checked device job table of a batch (host copy) with its totals.
struct BatchJobs {
    std::vector<DevJob> jobs;
    int64_t total_paths = 0;
    int min_spp = 0;
};

BatchJobs make_batch(const SceneHost& s, int n, const omv_job* jobs, const omv_params& p)
{
    if (n <= 0 || !jobs) throw ArgError("a batch needs at least one job");
    if (p.camera_bounces < 0 || p.light_bounces < 0) throw ArgError("negative bounce count");
    if (p.camera_bounces > 60 || p.light_bounces > 60) throw ArgError("at most 60 bounces are supported");
    BatchJobs B;
    B.jobs.resize(n);
    int64_t paths = 0, pixels = 0;
    B.min_spp = 1 << 30;
    for (int i = 0; i < n; ++i) {
        const omv_job& j = jobs[i];
        if (j.camera.width <= 0 || j.camera.height <= 0) throw ArgError("batch job with a non-positive resolution");
        if (j.samples_per_pixel <= 0) throw ArgError("batch job with no samples");
        if (!j.d_sum_rgb || !j.d_count) throw ArgError("batch job without a film");
        if (p.accumulate_variance && !j.d_sumsq_rgb) throw ArgError("accumulate_variance needs every job's d_sumsq_rgb");
        if (j.material_set < -1 || j.material_set >= s.num_mat_sets) throw ArgError("batch job material set out of range");
        if (j.part < 0 || j.part >= (int)s.parts.size()) throw ArgError("batch job scene (part) out of range");
        const int64_t npix = (int64_t)j.camera.width * j.camera.height;
        if (npix * j.samples_per_pixel > (int64_t)0x7FFFFFFF) throw ArgError("batch job too large");
        DevJob& d = B.jobs[i];
        d = DevJob{};
        d.cam = j.camera;
        d.path_base = paths;
        d.pixel_base = (uint32_t)pixels;
        d.spp = j.samples_per_pixel;
        d.sample_offset = j.sample_offset;
        d.seed = j.seed;
        d.mats = j.material_set < 0 ? s.dev.mats : s.mat_sets + (size_t)j.material_set * s.num_materials;
        const ScenePart& part = s.parts[j.part];
        d.part = j.part;
        d.tlas_root = part.tlas_root;
        d.light_base = part.light_base;
        d.light_count = part.light_count;
        d.light_max = part.light_max;
        d.sum = j.d_sum_rgb;
        d.sumsq = p.accumulate_variance ? j.d_sumsq_rgb : nullptr;
        d.count = j.d_count;
        paths += npix * j.samples_per_pixel;
        pixels += npix;
        B.min_spp = std::min(B.min_spp, j.samples_per_pixel);
    }
    if (pixels > (int64_t)0xFFFFFFFFu) throw ArgError("batch has too many pixels");
    B.total_paths = paths;
    return B;
}

FramePlan batch_frame_plan(SceneHost& s, const BatchJobs& B, const omv_params& p, int64_t wave_paths)
{
    FramePlan P;
    P.npix = 0;
    P.total = B.total_paths;
    P.lights = s.num_lights > 0;
    P.light_slots = P.lights ? p.light_bounces + 1 : 1;
    P.shadow_slots = std::max(1, (P.lights ? P.light_slots : 0) + (mis_on(s, p) ? 1 : 0));
    int64_t cap = wave_paths;
    if (cap <= 0) {
        size_t free_b = 0, total_b = 0;
        OMV_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const size_t budget = std::min(kWaveScratchBudget, (free_b + s.scratch.bytes) / 2);
        cap = (int64_t)(budget / path_scratch_bytes(P.light_slots, P.shadow_slots));
    }
    P.cap = std::max<int64_t>(1, std::min<int64_t>({cap, std::max<int64_t>(P.total, 1), (int64_t)0x7FFFFFFF}));
    return P;
}

void upload_jobs(SceneHost& s, const BatchJobs& B, cudaStream_t st)
{
    if (s.jobs_cap < B.jobs.size()) {
        OMV_CUDA(cudaStreamSynchronize(s.stream));
        OMV_CUDA(cudaStreamSynchronize(st));
        if (s.d_jobs) cudaFree(s.d_jobs);
        s.d_jobs = nullptr;
        s.jobs_cap = 0;
        if (s.batch_graph) {  // it refers to the old table
            cudaGraphExecDestroy(s.batch_graph);
            s.batch_graph = nullptr;
            s.batch_key.clear();
        }
        const size_t cap = std::max<size_t>(64, B.jobs.size());
        OMV_CUDA(cudaMalloc(&s.d_jobs, sizeof(DevJob) * cap));
        s.jobs_cap = cap;
    }
    // ordered on the caller's stream: after the batches still reading the old
    // table (a replay on the scene's stream is joined back into it) and before
    // this batch's kernels or graph, which start after it; the host vector is
    // pageable, so the call returns once the runtime has staged it
    OMV_CUDA(cudaMemcpyAsync(s.d_jobs, B.jobs.data(), sizeof(DevJob) * B.jobs.size(), cudaMemcpyHostToDevice, st));
}

}  // namespace

void render_batch(SceneHost& s, int n, const omv_job* jobs, const omv_params& p, cudaStream_t st, omv_stats* stats,
                  bool use_graph)
{
    const BatchJobs B = make_batch(s, n, jobs, p);
    const FramePlan P = batch_frame_plan(s, B, p, s.batch_wave_paths);
    if (mis_on(s, p)) ensure_env_sampler(s);  // allocates: never inside a graph capture
    ensure_scratch(s, P.cap, P.light_slots, P.shadow_slots);
    upload_jobs(s, B, st);
    const BatchPlan plan{s.d_jobs, &B.jobs, B.min_spp};
    omv_camera cam0 = B.jobs[0].cam;
    if (!use_graph) {
        run_waves(s, s.scratch, P, cam0, p, nullptr, nullptr, nullptr, st, stats, stats != nullptr, &plan);
        return;
    }
    // a default stream cannot be captured: capture and replay on the scene's
    // stream, ordered after the caller's stream and the caller's stream after it
    const cudaStream_t caller = st;
    const bool fork = st == nullptr || st == cudaStreamLegacy || st == cudaStreamPerThread;
    if (fork) {
        if (!s.fork_ev) OMV_CUDA(cudaEventCreateWithFlags(&s.fork_ev, cudaEventDisableTiming));
        if (!s.join_ev) OMV_CUDA(cudaEventCreateWithFlags(&s.join_ev, cudaEventDisableTiming));
        OMV_CUDA(cudaEventRecord(s.fork_ev, caller));
        OMV_CUDA(cudaStreamWaitEvent(s.stream, s.fork_ev, 0));
        st = s.stream;
    }
    // the captured graph is valid for this job table, these parameters and this wave size
    std::vector<unsigned char> key(sizeof(DevJob) * B.jobs.size() + sizeof(omv_params) + sizeof(int64_t));
    std::memcpy(key.data(), B.jobs.data(), sizeof(DevJob) * B.jobs.size());
    omv_params pk = p;
    pk.time_kernels = 0;
    std::memcpy(key.data() + sizeof(DevJob) * B.jobs.size(), &pk, sizeof(pk));
    std::memcpy(key.data() + sizeof(DevJob) * B.jobs.size() + sizeof(pk), &P.cap, sizeof(int64_t));
    if (!s.batch_graph || s.batch_key != key) {
        if (s.batch_graph) {
            cudaGraphExecDestroy(s.batch_graph);
            s.batch_graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        OMV_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            run_waves(s, s.scratch, P, cam0, pk, nullptr, nullptr, nullptr, st, nullptr, false, &plan);
        } catch (...) {
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        OMV_CUDA(cudaStreamEndCapture(st, &g));
        cudaGraphExec_t ge = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        OMV_CUDA(e);
        s.batch_graph = ge;
        s.batch_key = key;
    }
    OMV_CUDA(cudaGraphLaunch(s.batch_graph, st));
    if (fork) {
        OMV_CUDA(cudaEventRecord(s.join_ev, st));
        OMV_CUDA(cudaStreamWaitEvent(caller, s.join_ev, 0));
    }
    if (stats) {
        OMV_CUDA(cudaStreamSynchronize(st));
        *stats = omv_stats{};
        stats->paths = B.total_paths;
    }
}

void autotune_batch(SceneHost& s, int n, const omv_job* jobs, const omv_params& p, cudaStream_t st,
                    int64_t* chosen, int32_t* chosen_threads)
{
    const BatchJobs B = make_batch(s, n, jobs, p);
    const FramePlan Pmax = batch_frame_plan(s, B, p, 0);
    // candidates: wave sizes 4M x 4^k up to the largest that fits (the queue
    // capacities follow the wave size), each with 128 and 256 threads per
    // block of the shading kernels
    std::vector<int64_t> cand;
    for (int64_t c = (int64_t)1 << 22; c < Pmax.cap; c *= 4) cand.push_back(c);
    cand.push_back(Pmax.cap);
    const int threads[] = {128, 256};
    cudaEvent_t e0, e1;
    OMV_CUDA(cudaEventCreate(&e0));
    OMV_CUDA(cudaEventCreate(&e1));
    int64_t best = Pmax.cap;
    int best_t = kShadeThreads;
    float best_ms = 3.0e38f;
    const int64_t saved = s.batch_wave_paths;
    const int saved_t = s.batch_shade_threads;
    try {
        for (int64_t c : cand)
            for (int t : threads) {
                s.batch_wave_paths = c;
                s.batch_shade_threads = t;
                render_batch(s, n, jobs, p, st, nullptr, false);  // warm-up (and scratch)
                OMV_CUDA(cudaEventRecord(e0, st));
                render_batch(s, n, jobs, p, st, nullptr, false);
                OMV_CUDA(cudaEventRecord(e1, st));
                OMV_CUDA(cudaEventSynchronize(e1));
                float ms = 0.0f;
                OMV_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                    best_t = t;
                }
            }
    } catch (...) {
        s.batch_wave_paths = saved;
        s.batch_shade_threads = saved_t;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s.batch_wave_paths = best;
    s.batch_shade_threads = best_t;
    if (chosen) *chosen = best;
    if (chosen_threads) *chosen_threads = best_t;
}

// ------------------------------------------ render without allocation ---
//
// Callers that must not allocate device memory while they render: a host
// framework that owns the device memory through its own pool and leaves no
// headroom, or a loop that cannot afford cudaMalloc/cudaFree (cudaFree
// synchronises the whole device).  The wave scratch then comes from one fixed
// array in the library's device image instead of the scene's grown buffer.
namespace {

__device__ __align__(256) unsigned char g_static_scratch[OMV_STATIC_SCRATCH_BYTES];

// Loads every kernel the wave loop of a reference-estimator frame can launch
// into the current context.  With lazy module loading (the CUDA default) a
// kernel is loaded, and its module's device memory allocated, on its first
// launch; a later frame on a scene with point lights or alpha-masked
// materials would otherwise load k_light_gen / k_light_shade / the masked
// shadow kernel then.  Querying a kernel's attributes loads it.
void load_wave_kernels()
{
    cudaFuncAttributes a;
    OMV_CUDA(cudaFuncGetAttributes(&a, k_job_ids));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_camera_gen));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_light_gen));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_extend));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_light_shade));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_camera_shade<false>));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_shadow<false, false>));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_shadow<false, true>));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_camera_tail<false, false>));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_camera_tail<false, true>));
    OMV_CUDA(cudaFuncGetAttributes(&a, k_film));
}

// Device address of g_static_scratch in the current context, resolved on
// every call (a lookup once the module is loaded), so that a context created
// after a device reset gets its own address.  The first call in a context
// loads the module and the wave kernels.
void* static_scratch_address()
{
    load_wave_kernels();
    void* addr = nullptr;
    OMV_CUDA(cudaGetSymbolAddress(&addr, g_static_scratch));
    return addr;
}

}  // namespace

int64_t static_wave_limit(int light_slots, int shadow_slots)
{
    const size_t per_path = path_scratch_bytes(light_slots, shadow_slots);
    const size_t fixed = 48 + kMaxCounters * 4 + 16 * 8 + 14 * 256;
    int64_t cap = (int64_t)((OMV_STATIC_SCRATCH_BYTES - fixed) / per_path) & ~(int64_t)31;
    while (cap > 0 && scratch_layout(cap, light_slots, shadow_slots).bytes > OMV_STATIC_SCRATCH_BYTES) cap -= 32;
    return cap;
}

void render_frame_static(SceneHost& s, const omv_camera& cam, const omv_params& p, double* d_sum, double* d_sumsq,
                         uint32_t* d_count, cudaStream_t st)
{
    if (p.time_kernels) throw ArgError("time_kernels needs CUDA events, which the no-allocation render does not create");
    if (mis_on(s, p))
        throw ArgError("the MIS estimator builds an environment table on first use; the no-allocation render "
                       "supports the reference estimator only (MIS has no effect on a scene without an HDRI)");
    FramePlan P = plan_frame(s, cam, p, 1);
    const int64_t limit = static_wave_limit(P.light_slots, P.shadow_slots);
    if (p.wave_paths > 0) {
        const size_t need = scratch_layout(P.cap, P.light_slots, P.shadow_slots).bytes;
        if (need > OMV_STATIC_SCRATCH_BYTES)
            throw ArgError("wave_paths " + std::to_string(p.wave_paths) + " needs " + std::to_string(need) +
                           " bytes of scratch; the static scratch holds " +
                           std::to_string((size_t)OMV_STATIC_SCRATCH_BYTES) + " bytes (at most " +
                           std::to_string(limit) + " paths per wave with these bounce counts)");
    } else {
        P.cap = std::min<int64_t>(limit, std::max<int64_t>(P.total, 1));
    }
    RenderScratch R;
    carve_scratch(R, static_scratch_address(), P.cap, P.light_slots, P.shadow_slots);
    run_waves(s, R, P, cam, p, d_sum, d_sumsq, d_count, st, nullptr, false);
}

void render_ids(SceneHost& s, const omv_camera& cam, const float* d_jitter, uint64_t seed, omv_hit* d_hits,
                uint32_t* d_gprim, cudaStream_t st)
{
    const int64_t npix = (int64_t)cam.width * cam.height;
    k_ids<<<grid_for(npix, kTraceThreads), kTraceThreads, 0, st>>>(s.dev, s.tlas_items, cam, d_jitter, seed, d_hits,
                                                                    d_gprim, s.d_face_prefix);
    OMV_CUDA(cudaGetLastError());
}

void trace_rays(SceneHost& s, int64_t n, const float* d_rays, omv_hit* d_hits, cudaStream_t st)
{
    if (n <= 0) return;
    k_trace_rays<<<grid_for(n, kTraceThreads), kTraceThreads, 0, st>>>(s.dev, s.tlas_items, n, d_rays, d_hits);
    OMV_CUDA(cudaGetLastError());
}

void env_radiance(SceneHost& s, int64_t n, const float* d_dirs, float* d_rgb, cudaStream_t st)
{
    if (n <= 0) return;
    k_env<<<grid_for(n, 256), 256, 0, st>>>(s.dev.env, n, d_dirs, d_rgb);
    OMV_CUDA(cudaGetLastError());
}

}  // namespace omv
