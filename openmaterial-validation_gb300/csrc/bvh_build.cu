// GPU acceleration-structure build, replacing Embree's BVH build of
// RenderScene::buildEmbreeScene (RenderScene.cpp:225-272): one bottom-level
// tree per mesh (Embree: one scene per mesh) and one top-level tree over the
// instances (Embree: instance geometries in the top scene).
//
// Pipeline per tree (all on the device):
//   1. item boxes + centroid bounds (block reduction, atomics on ordered ints)
//   2. 30-bit Morton codes of the centroids
//   3. LSD radix sort of (code, item) pairs, 8-bit digits, stable block ranks
//      from warp match_any + per-warp digit counts
//   4. Karras LBVH ("Maximizing parallelism in the construction of BVHs,
//      octrees, and k-d trees", HPG 2012): one thread per internal node
//   5. bottom-up boxes with arrival counters
//   6. top-down collapse into 8-wide nodes (greedy: expand the child of largest
//      surface area; children placed in octant slots), leaves of at most
//      kLeafMax triangles, child boxes
//      quantised to 16 bits per bound against the node box, rounded outward and
//      verified in float so the decoded box always contains the true box.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "bvh_build.h"
#include "omv_types.h"

namespace omv {

// throws with the runtime's message ("out of memory" for a failed allocation,
// which the C ABI reports as OMV_ERR_OUT_OF_MEMORY) and clears the runtime's
// non-sticky error state
#define OMV_CK(x)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) {                                                                  \
            (void)cudaGetLastError();                                                             \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " \
                                     + __FILE__ + ":" + std::to_string(__LINE__));                \
        }                                                                                         \
    } while (0)

namespace {

constexpr int kSortTile = 4096;
constexpr int kSortThreads = 256;

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ uint32_t f2ord(float f)
{
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// ---------------------------------------------------------- item boxes ---
__global__ void k_tri_boxes(int n, const float* __restrict__ pos, const uint32_t* __restrict__ faces, Box* boxes,
                            uint32_t* cbounds /* 6 ordered: lo xyz, hi xyz */)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float c[3] = {0.f, 0.f, 0.f};
    bool ok = i < n;
    if (ok) {
        Box b;
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = 3.0e38f;
            b.hi[a] = -3.0e38f;
        }
        bool finite = true;
        for (int k = 0; k < 3; ++k) {
            const float* p = pos + 3 * (size_t)faces[3 * (size_t)i + k];
            for (int a = 0; a < 3; ++a) {
                finite = finite && isfinite(p[a]);
                b.lo[a] = fminf(b.lo[a], p[a]);
                b.hi[a] = fmaxf(b.hi[a], p[a]);
            }
        }
        // a triangle with a NaN or infinite coordinate can never be hit; it gets
        // an empty box (never entered, no effect on any bound), as an Embree
        // robust build leaves invalid primitives out
        if (!finite)
            for (int a = 0; a < 3; ++a) {
                b.lo[a] = 3.0e38f;
                b.hi[a] = -3.0e38f;
            }
        boxes[i] = b;
        for (int a = 0; a < 3; ++a) c[a] = finite ? 0.5f * (b.lo[a] + b.hi[a]) : 0.0f;
    }
    for (int a = 0; a < 3; ++a) {
        uint32_t lo = ok ? f2ord(c[a]) : 0xFFFFFFFFu, hi = ok ? f2ord(c[a]) : 0u;
        for (int o = 16; o; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&cbounds[a], lo);
            atomicMax(&cbounds[3 + a], hi);
        }
    }
}

// World bounds of one instance: every vertex its finite faces reference, through the
// instance transform (double arithmetic, rounded to float), reduced into six
// ordered ints (lo xyz, hi xyz).  Tighter than the box of the transformed
// object box, which a rotation inflates.
struct Xf34 {
    float m[12];
};
__global__ void k_instance_bounds(int nfaces, const float* __restrict__ pos, const uint32_t* __restrict__ faces,
                                  Xf34 xf, uint32_t* out6)
{
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nfaces; f += gridDim.x * blockDim.x) {
        const float* v[3];
        bool finite = true;
        for (int k = 0; k < 3; ++k) {
            v[k] = pos + 3 * (size_t)faces[3 * (size_t)f + k];
            finite = finite && isfinite(v[k][0]) && isfinite(v[k][1]) && isfinite(v[k][2]);
        }
        if (!finite) continue;  // left out of the tree (k_tri_boxes)
        for (int k = 0; k < 3; ++k) {
            const float* p = v[k];
            for (int a = 0; a < 3; ++a) {
                const double w = (double)xf.m[4 * a] * p[0] + (double)xf.m[4 * a + 1] * p[1] +
                                 (double)xf.m[4 * a + 2] * p[2] + (double)xf.m[4 * a + 3];
                lo[a] = fminf(lo[a], (float)w);
                hi[a] = fmaxf(hi[a], (float)w);
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        uint32_t l = f2ord(lo[a]), h = f2ord(hi[a]);
        for (int o = 16; o; o >>= 1) {
            l = min(l, __shfl_xor_sync(0xFFFFFFFFu, l, o));
            h = max(h, __shfl_xor_sync(0xFFFFFFFFu, h, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&out6[a], l);
            atomicMax(&out6[3 + a], h);
        }
    }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(int n, const Box* boxes, const uint32_t* cbounds, uint32_t* keys, uint32_t* vals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        float lo = ord2f(cbounds[a]), hi = ord2f(cbounds[3 + a]);
        float c = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
        float ext = hi - lo;
        float t = ext > 0.f ? (c - lo) / ext : 0.5f;
        q[a] = (uint32_t)fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
    }
    keys[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    vals[i] = (uint32_t)i;
}

// ------------------------------------------------------------- sort ---
__global__ void k_sort_hist(int n, int shift, const uint32_t* __restrict__ keys, uint32_t* hist, int nblocks)
{
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int base = blockIdx.x * kSortTile;
    for (int i = base + threadIdx.x; i < min(n, base + kSortTile); i += blockDim.x)
        atomicAdd(&h[(keys[i] >> shift) & 0xFF], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * nblocks + blockIdx.x] = h[d];
}

// exclusive scan of m entries, one block
__global__ void k_scan(int m, uint32_t* data)
{
    __shared__ uint32_t part[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < m; base += 1024) {
        int i = base + threadIdx.x;
        uint32_t v = i < m ? data[i] : 0u;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            uint32_t t = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < m) data[i] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(int n, int shift, const uint32_t* __restrict__ kin,
                                                               const uint32_t* __restrict__ vin, uint32_t* kout,
                                                               uint32_t* vout, const uint32_t* offs, int nblocks)
{
    constexpr int W = kSortThreads / 32;
    __shared__ uint32_t run[256];
    __shared__ uint32_t cnt[W][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) run[d] = offs[d * nblocks + blockIdx.x];
    const int base = blockIdx.x * kSortTile;
    const int end = min(n, base + kSortTile);
    for (int c0 = base; c0 < end; c0 += kSortThreads) {
        for (int i = threadIdx.x; i < W * 256; i += blockDim.x) (&cnt[0][0])[i] = 0;
        __syncthreads();
        int i = c0 + threadIdx.x;
        bool ok = i < end;
        uint32_t key = ok ? kin[i] : 0u;
        uint32_t val = ok ? vin[i] : 0u;
        uint32_t dig = ok ? (key >> shift) & 0xFF : 256u + lane;  // invalid lanes never match
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, dig);
        uint32_t lt = peers & ((1u << lane) - 1u);
        if (ok && lt == 0) cnt[warp][dig] = __popc(peers);
        __syncthreads();
        if (ok) {
            uint32_t pre = 0;
            for (int w = 0; w < warp; ++w) pre += cnt[w][dig];
            uint32_t dst = run[dig] + pre + __popc(lt);
            kout[dst] = key;
            vout[dst] = val;
        }
        __syncthreads();
        for (int d = threadIdx.x; d < 256; d += blockDim.x) {
            uint32_t t = 0;
            for (int w = 0; w < W; ++w) t += cnt[w][d];
            run[d] += t;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ LBVH ---
struct Node2 {
    int left, right;  // >= 0: internal id; < 0: ~leaf position (sorted index)
    int first, last;  // covered sorted range
    int parent;
    Box box;
};

__device__ __forceinline__ int delta(const uint32_t* k, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    uint32_t a = k[i], b = k[j];
    return a == b ? 32 + __clz((uint32_t)i ^ (uint32_t)j) : __clz(a ^ b);
}

__global__ void k_karras(int n, const uint32_t* __restrict__ keys, Node2* nodes, int* leaf_parent)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) > 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int g = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    Node2& nd = nodes[i];
    nd.first = lo;
    nd.last = hi;
    if (lo == g) {
        nd.left = ~g;
        leaf_parent[g] = i;
    } else {
        nd.left = g;
        nodes[g].parent = i;
    }
    if (hi == g + 1) {
        nd.right = ~(g + 1);
        leaf_parent[g + 1] = i;
    } else {
        nd.right = g + 1;
        nodes[g + 1].parent = i;
    }
    if (i == 0) nd.parent = -1;
}

__device__ __forceinline__ Box box_union(const Box& a, const Box& b)
{
    Box r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = fminf(a.lo[k], b.lo[k]);
        r.hi[k] = fmaxf(a.hi[k], b.hi[k]);
    }
    return r;
}

__global__ void k_bottom_up(int n, const uint32_t* __restrict__ vals, const Box* __restrict__ item_boxes,
                            Node2* nodes, const int* leaf_parent, int* arrivals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = leaf_parent[i];
    for (int guard = 0; p >= 0 && guard < 96; ++guard) {
        __threadfence();
        if (atomicAdd(&arrivals[p], 1) == 0) return;
        __threadfence();
        Node2& nd = nodes[p];
        Box bl = nd.left >= 0 ? nodes[nd.left].box : item_boxes[vals[~nd.left]];
        Box br = nd.right >= 0 ? nodes[nd.right].box : item_boxes[vals[~nd.right]];
        Box u = box_union(bl, br);
        volatile float* dst = (volatile float*)&nd.box;
        for (int k = 0; k < 3; ++k) {
            dst[k] = u.lo[k];
            dst[3 + k] = u.hi[k];
        }
        p = nd.parent;
    }
}

// ---------------------------------------------------------- collapse ---
struct Work {
    int node2;  // internal Node2 id, or ~sorted position for a single-item tree
    uint32_t node8;
};

__device__ __forceinline__ float half_area(const Box& b)
{
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void child_info(const Node2* nodes, const uint32_t* vals, const Box* item_boxes, int c,
                                           Box& b, int& first, int& last)
{
    if (c >= 0) {
        const Node2& nd = nodes[c];
        volatile const float* src = (volatile const float*)&nd.box;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = src[k];
            b.hi[k] = src[3 + k];
        }
        first = nd.first;
        last = nd.last;
    } else {
        b = item_boxes[vals[~c]];
        first = last = ~c;
    }
}

// exponent byte e such that 2^(e-127) * 65532 >= extent
__device__ __forceinline__ uint32_t quant_exponent(float ext)
{
    if (!(ext > 0.0f)) return 1u;
    float s = ext / 65532.0f;
    uint32_t bits = __float_as_uint(s);
    uint32_t e = (bits >> 23) & 0xFF;
    if (bits & 0x7FFFFFu) e += 1;  // round up to a power of two
    if (e < 1) e = 1;
    if (e > 254) e = 254;
    return e;
}

template <bool kTlas>
__global__ void k_collapse(int nwork, const Work* __restrict__ work, const Node2* nodes, const uint32_t* vals,
                           const Box* item_boxes, Bvh8Node* out_nodes, uint32_t* node_counter, Work* next_work,
                           uint32_t* next_count, float4* out_tris, uint32_t* out_items, uint32_t* prim_counter,
                           const float* pos, const uint32_t* faces, uint32_t node_cap, uint32_t* overflow)
{
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwork) return;
    Work it = work[w];
    int slot[8];
    Box sb[8];
    int sf[8], sl[8];
    int ns = 0;
    if (it.node2 < 0) {
        slot[0] = it.node2;
        child_info(nodes, vals, item_boxes, slot[0], sb[0], sf[0], sl[0]);
        ns = 1;
    } else {
        const Node2& nd = nodes[it.node2];
        slot[0] = nd.left;
        slot[1] = nd.right;
        child_info(nodes, vals, item_boxes, slot[0], sb[0], sf[0], sl[0]);
        child_info(nodes, vals, item_boxes, slot[1], sb[1], sf[1], sl[1]);
        ns = 2;
        const int leaf_max = kTlas ? 1 : kLeafMax;
        while (ns < 8) {
            int best = -1;
            float ba = -1.0f;
            bool must = false;
            for (int s = 0; s < ns; ++s) {
                if (slot[s] < 0) continue;
                int cnt = sl[s] - sf[s] + 1;
                bool m = cnt > leaf_max;
                float a = half_area(sb[s]);
                if ((m && !must) || (m == must && a > ba)) {
                    best = s;
                    ba = a;
                    must = m;
                }
            }
            if (best < 0) break;
            const Node2& e = nodes[slot[best]];
            int l = e.left, r = e.right;
            slot[best] = l;
            child_info(nodes, vals, item_boxes, l, sb[best], sf[best], sl[best]);
            slot[ns] = r;
            child_info(nodes, vals, item_boxes, r, sb[ns], sf[ns], sl[ns]);
            ++ns;
        }
    }
    const int leaf_max = kTlas ? 1 : kLeafMax;
    Box nb = sb[0];
    for (int s = 1; s < ns; ++s) nb = box_union(nb, sb[s]);
    int n_int = 0, n_prim = 0;
    for (int s = 0; s < ns; ++s) {
        int cnt = sl[s] - sf[s] + 1;
        if (cnt > leaf_max)
            ++n_int;
        else
            n_prim += cnt;
    }
    uint32_t cbase = n_int ? atomicAdd(node_counter, (uint32_t)n_int) : 0u;
    uint32_t pbase = n_prim ? atomicAdd(prim_counter, (uint32_t)n_prim) : 0u;
    if (cbase + n_int > node_cap) {
        atomicAdd(overflow, 1u);
        return;
    }
    Bvh8Node o;
    uint32_t e[3];
    float sc[3];
    for (int a = 0; a < 3; ++a) {
        e[a] = quant_exponent(nb.hi[a] - nb.lo[a]);
        sc[a] = __uint_as_float(e[a] << 23);
    }
    o.px = __fsub_rn(nb.lo[0], sc[0]);
    o.py = __fsub_rn(nb.lo[1], sc[1]);
    o.pz = __fsub_rn(nb.lo[2], sc[2]);
    const float p[3] = {o.px, o.py, o.pz};
    // octant slot assignment (Ylitie, Karras, Laine, "Efficient incoherent ray
    // traversal on GPUs through compressed wide BVHs", HPG 2017): slot s stands
    // for the corner direction (+-1,+-1,+-1) given by its bits; children go to the
    // slot their centroid offset points to (greedy on the largest projection), so
    // visiting slots in the order s ^ octant(ray) is approximately front to back.
    int at[8];
    {
        float score[8][8];
        const float cx = 0.5f * (nb.lo[0] + nb.hi[0]), cy = 0.5f * (nb.lo[1] + nb.hi[1]),
                    cz = 0.5f * (nb.lo[2] + nb.hi[2]);
        for (int i = 0; i < ns; ++i) {
            const float dx = 0.5f * (sb[i].lo[0] + sb[i].hi[0]) - cx;
            const float dy = 0.5f * (sb[i].lo[1] + sb[i].hi[1]) - cy;
            const float dz = 0.5f * (sb[i].lo[2] + sb[i].hi[2]) - cz;
            for (int q = 0; q < 8; ++q)
                score[i][q] = ((q & 1) ? dx : -dx) + ((q & 2) ? dy : -dy) + ((q & 4) ? dz : -dz);
        }
        for (int q = 0; q < 8; ++q) at[q] = -1;
        uint32_t used_child = 0, used_slot = 0;
        for (int k = 0; k < ns; ++k) {
            float best = -3.0e38f;
            int bi = -1, bq = -1;
            for (int i = 0; i < ns; ++i) {
                if (used_child & (1u << i)) continue;
                for (int q = 0; q < 8; ++q) {
                    if (used_slot & (1u << q)) continue;
                    if (score[i][q] > best) {
                        best = score[i][q];
                        bi = i;
                        bq = q;
                    }
                }
            }
            at[bq] = bi;
            used_child |= 1u << bi;
            used_slot |= 1u << bq;
        }
    }
    uint32_t imask = 0, meta[8];
    int rank = 0, off = 0;
    for (int s = 0; s < 8; ++s) {
        meta[s] = 0;
        for (int a = 0; a < 3; ++a) {
            o.qlo[a][s] = 0xFFFF;
            o.qhi[a][s] = 0;
        }
    }
    // internal children are stored in slot order: child(s) = child_base + popc(imask & ((1<<s)-1));
    // leaf primitives in slot order from prim_base
    for (int s = 0; s < 8; ++s) {
        const int c = at[s];
        if (c < 0) continue;
        int cnt = sl[c] - sf[c] + 1;
        for (int a = 0; a < 3; ++a) {
            float lo = sb[c].lo[a], hi = sb[c].hi[a];
            int ql = (int)floorf(__fdiv_rn(__fsub_rn(lo, p[a]), sc[a]));
            int qh = (int)ceilf(__fdiv_rn(__fsub_rn(hi, p[a]), sc[a]));
            ql = max(0, min(65535, ql));
            qh = max(0, min(65535, qh));
            while (ql > 0 && __fadd_rn(p[a], __fmul_rn((float)ql, sc[a])) > lo) --ql;
            while (qh < 65535 && __fadd_rn(p[a], __fmul_rn((float)qh, sc[a])) < hi) ++qh;
            ql = ql > 0 ? ql - 1 : 0;          // one quantum of slack each side
            qh = qh < 65535 ? qh + 1 : 65535;
            o.qlo[a][s] = (uint16_t)ql;
            o.qhi[a][s] = (uint16_t)qh;
        }
        if (cnt > leaf_max) {
            imask |= 1u << s;
            meta[s] = (uint32_t)rank;
            uint32_t idx = atomicAdd(next_count, 1u);
            next_work[idx] = Work{slot[c], cbase + (uint32_t)rank};
            ++rank;
        } else {
            meta[s] = ((uint32_t)cnt << 5) | (uint32_t)off;
            for (int k = 0; k < cnt; ++k) {
                uint32_t item = vals[sf[c] + k];
                uint32_t dst = pbase + (uint32_t)(off + k);
                if (kTlas) {
                    out_items[dst] = item;
                } else {
                    const uint32_t* f = faces + 3 * (size_t)item;
                    const float* a0 = pos + 3 * (size_t)f[0];
                    const float* a1 = pos + 3 * (size_t)f[1];
                    const float* a2 = pos + 3 * (size_t)f[2];
                    out_tris[3 * (size_t)dst + 0] = make_float4(a0[0], a0[1], a0[2], __uint_as_float(item));
                    out_tris[3 * (size_t)dst + 1] = make_float4(a1[0], a1[1], a1[2], 0.0f);
                    out_tris[3 * (size_t)dst + 2] = make_float4(a2[0], a2[1], a2[2], 0.0f);
                }
            }
            off += cnt;
        }
    }
    o.exps = e[0] | (e[1] << 8) | (e[2] << 16) | (imask << 24);
    o.child_base = cbase;
    o.prim_base = pbase;
    o.meta_lo = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (meta[3] << 24);
    o.meta_hi = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (meta[7] << 24);
    out_nodes[it.node8] = o;
}

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    explicit DBuf(size_t count) : n(count)
    {
        if (count) OMV_CK(cudaMalloc(&p, sizeof(T) * count));
    }
    ~DBuf() { cudaFree(p); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
};

inline int blocks(size_t n, int t) { return (int)((n + t - 1) / t); }

// sorts (keys, vals) in place; tmp buffers provided
void radix_sort(int n, uint32_t* keys, uint32_t* vals, uint32_t* k2, uint32_t* v2, cudaStream_t st)
{
    int nb = blocks(n, kSortTile);
    DBuf<uint32_t> hist((size_t)nb * 256);
    uint32_t *ki = keys, *vi = vals, *ko = k2, *vo = v2;
    for (int shift = 0; shift < 32; shift += 8) {
        k_sort_hist<<<nb, 256, 0, st>>>(n, shift, ki, hist.p, nb);
        k_scan<<<1, 1024, 0, st>>>(nb * 256, hist.p);
        k_sort_scatter<<<nb, kSortThreads, 0, st>>>(n, shift, ki, vi, ko, vo, hist.p, nb);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    OMV_CK(cudaGetLastError());
    // four passes: the result is back in (keys, vals)
}

}  // namespace

// Builds one tree over n items whose boxes are in `item_boxes` (device).
// Appends nodes at node_base... of `out_nodes`, primitives at prim_base... .
static uint32_t collapse_tree(bool tlas, int n, const Node2* nodes, const uint32_t* vals, const Box* item_boxes,
                              const float* pos, const uint32_t* faces, Bvh8Node* out_nodes, uint32_t* node_counter,
                              uint32_t node_cap, float4* out_tris, uint32_t* out_items, uint32_t* prim_counter,
                              uint32_t* overflow, cudaStream_t st);

// Binary tree by the surface area heuristic, leaves of one item: binned
// (kSahBins bins per axis over the centroid bounds) on ranges of more than
// kSweepMax items, a full sweep over every split position below.  nodes[0] is
// the root; `order` receives the item order the node ranges refer to.  Runs on
// the host: for the top-level tree and for bottom-level trees of up to
// kHostSahMaxTris triangles (one thread per mesh).
constexpr int kSahBins = 32;
constexpr int kSweepMax = 32;
constexpr int kHostSahMaxTris = 1 << 21;

static void host_sah_tree(const std::vector<Box>& boxes, std::vector<Node2>& nodes, std::vector<uint32_t>& order)
{
    const int n = (int)boxes.size();
    order.resize(n);
    for (int i = 0; i < n; ++i) order[i] = (uint32_t)i;
    nodes.clear();
    if (n < 2) return;
    nodes.reserve(n - 1);
    auto area = [](const Box& b) {
        const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
        return dx * dy + dy * dz + dz * dx;
    };
    auto unite = [](const Box& a, const Box& b) {
        Box u;
        for (int k = 0; k < 3; ++k) {
            u.lo[k] = std::min(a.lo[k], b.lo[k]);
            u.hi[k] = std::max(a.hi[k], b.hi[k]);
        }
        return u;
    };
    Box empty;
    for (int k = 0; k < 3; ++k) {
        empty.lo[k] = 3.0e38f;
        empty.hi[k] = -3.0e38f;
    }
    std::vector<float> c2(3 * (size_t)n);  // twice the centroid
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) c2[3 * (size_t)i + k] = boxes[i].lo[k] + boxes[i].hi[k];
    struct Task {
        int first, last, parent, side;
    };
    std::vector<Task> todo{{0, n - 1, -1, 0}};
    std::vector<float> right_area(n);
    while (!todo.empty()) {
        const Task t = todo.back();
        todo.pop_back();
        const int cnt = t.last - t.first + 1;
        int ref;
        if (cnt == 1) {
            ref = ~t.first;
        } else {
            ref = (int)nodes.size();
            nodes.push_back(Node2{});
            Box b = empty;
            for (int k = t.first; k <= t.last; ++k) b = unite(b, boxes[order[k]]);
            int split = t.first + cnt / 2 - 1;  // fallback: halves in the current order
            if (cnt <= kSweepMax) {
                float best = 3.0e38f;
                int best_axis = -1;
                for (int a = 0; a < 3; ++a) {
                    std::stable_sort(order.begin() + t.first, order.begin() + t.last + 1,
                                     [&](uint32_t x, uint32_t y) { return c2[3 * (size_t)x + a] < c2[3 * (size_t)y + a]; });
                    Box acc = boxes[order[t.last]];
                    for (int k = t.last; k > t.first; --k) {
                        acc = unite(acc, boxes[order[k]]);
                        right_area[k] = area(acc);
                    }
                    acc = boxes[order[t.first]];
                    for (int k = t.first; k < t.last; ++k) {
                        acc = unite(acc, boxes[order[k]]);
                        const float c = area(acc) * (float)(k - t.first + 1) + right_area[k + 1] * (float)(t.last - k);
                        if (c < best) {
                            best = c;
                            best_axis = a;
                            split = k;
                        }
                    }
                }
                if (best_axis >= 0)
                    std::stable_sort(order.begin() + t.first, order.begin() + t.last + 1, [&](uint32_t x, uint32_t y) {
                        return c2[3 * (size_t)x + best_axis] < c2[3 * (size_t)y + best_axis];
                    });
            } else {
                float cmin[3], cmax[3];
                for (int k = 0; k < 3; ++k) {
                    cmin[k] = 3.0e38f;
                    cmax[k] = -3.0e38f;
                }
                for (int k = t.first; k <= t.last; ++k)
                    for (int a = 0; a < 3; ++a) {
                        cmin[a] = std::min(cmin[a], c2[3 * (size_t)order[k] + a]);
                        cmax[a] = std::max(cmax[a], c2[3 * (size_t)order[k] + a]);
                    }
                float best = 3.0e38f;
                int best_axis = -1, best_bin = 0;
                for (int a = 0; a < 3; ++a) {
                    const float ext = cmax[a] - cmin[a];
                    if (!(ext > 0.0f)) continue;
                    const float scale = (float)kSahBins / ext;
                    auto bin = [&](uint32_t it) {  // clamped before the conversion (scale may overflow)
                        return (int)std::min((float)(kSahBins - 1), (c2[3 * (size_t)it + a] - cmin[a]) * scale);
                    };
                    int bc[kSahBins] = {};
                    Box bb[kSahBins];
                    for (int q = 0; q < kSahBins; ++q) bb[q] = empty;
                    for (int k = t.first; k <= t.last; ++k) {
                        const uint32_t it = order[k];
                        const int q = bin(it);
                        ++bc[q];
                        bb[q] = unite(bb[q], boxes[it]);
                    }
                    float ra[kSahBins];
                    int rc[kSahBins];
                    Box acc = empty;
                    int accn = 0;
                    for (int q = kSahBins - 1; q > 0; --q) {
                        acc = unite(acc, bb[q]);
                        accn += bc[q];
                        ra[q] = accn ? area(acc) : 0.0f;
                        rc[q] = accn;
                    }
                    acc = empty;
                    accn = 0;
                    for (int q = 0; q < kSahBins - 1; ++q) {
                        acc = unite(acc, bb[q]);
                        accn += bc[q];
                        if (accn == 0 || rc[q + 1] == 0) continue;
                        const float c = area(acc) * (float)accn + ra[q + 1] * (float)rc[q + 1];
                        if (c < best) {
                            best = c;
                            best_axis = a;
                            best_bin = q;
                        }
                    }
                }
                if (best_axis >= 0) {
                    const int a = best_axis;
                    const float scale = (float)kSahBins / (cmax[a] - cmin[a]);
                    auto mid = std::stable_partition(order.begin() + t.first, order.begin() + t.last + 1, [&](uint32_t it) {
                        return (int)std::min((float)(kSahBins - 1), (c2[3 * (size_t)it + a] - cmin[a]) * scale) <=
                               best_bin;
                    });
                    split = (int)(mid - order.begin()) - 1;
                }
            }
            Node2& nd = nodes[ref];
            nd.first = t.first;
            nd.last = t.last;
            nd.parent = t.parent;
            nd.box = b;
            nd.left = nd.right = 0;
            todo.push_back({split + 1, t.last, ref, 1});
            todo.push_back({t.first, split, ref, 0});
        }
        if (t.parent >= 0) (t.side ? nodes[t.parent].right : nodes[t.parent].left) = ref;
    }
}

static uint32_t build_tree(bool tlas, int n, Box* item_boxes, uint32_t* cbounds, const float* pos,
                           const uint32_t* faces, Bvh8Node* out_nodes, uint32_t* node_counter, uint32_t node_cap,
                           float4* out_tris, uint32_t* out_items, uint32_t* prim_counter, uint32_t* overflow,
                           cudaStream_t st)
{
    DBuf<uint32_t> keys(n), vals(n), k2(n), v2(n);
    k_morton<<<blocks(n, 256), 256, 0, st>>>(n, item_boxes, cbounds, keys.p, vals.p);
    radix_sort(n, keys.p, vals.p, k2.p, v2.p, st);
    int ni = n > 1 ? n - 1 : 1;
    DBuf<Node2> nodes(ni);
    DBuf<int> leaf_parent(n), arrivals(ni);
    OMV_CK(cudaMemsetAsync(arrivals.p, 0, sizeof(int) * ni, st));
    if (n > 1) {
        k_karras<<<blocks(n - 1, 256), 256, 0, st>>>(n, keys.p, nodes.p, leaf_parent.p);
        k_bottom_up<<<blocks(n, 256), 256, 0, st>>>(n, vals.p, item_boxes, nodes.p, leaf_parent.p, arrivals.p);
    }
    return collapse_tree(tlas, n, nodes.p, vals.p, item_boxes, pos, faces, out_nodes, node_counter, node_cap, out_tris,
                         out_items, prim_counter, overflow, st);
}

// Top-down collapse of a binary tree (nodes[0] the root when n > 1) into 8-wide
// nodes appended to out_nodes; returns the root's index.
static uint32_t collapse_tree(bool tlas, int n, const Node2* nodes, const uint32_t* vals, const Box* item_boxes,
                              const float* pos, const uint32_t* faces, Bvh8Node* out_nodes, uint32_t* node_counter,
                              uint32_t node_cap, float4* out_tris, uint32_t* out_items, uint32_t* prim_counter,
                              uint32_t* overflow, cudaStream_t st)
{
    Work root{};
    root.node2 = n > 1 ? 0 : ~0;
    uint32_t root_index = 0;
    OMV_CK(cudaMemcpyAsync(&root_index, node_counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    OMV_CK(cudaStreamSynchronize(st));
    root.node8 = root_index;
    uint32_t one = root_index + 1;
    OMV_CK(cudaMemcpyAsync(node_counter, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    DBuf<Work> wa(n + 1), wb(n + 1);
    DBuf<uint32_t> cnt(1);
    OMV_CK(cudaMemcpyAsync(wa.p, &root, sizeof(Work), cudaMemcpyHostToDevice, st));
    int nwork = 1;
    Work *cur = wa.p, *nxt = wb.p;
    for (int level = 0; nwork > 0; ++level) {
        if (level > 200) throw std::runtime_error("BVH collapse did not terminate");
        OMV_CK(cudaMemsetAsync(cnt.p, 0, sizeof(uint32_t), st));
        if (tlas)
            k_collapse<true><<<blocks(nwork, 128), 128, 0, st>>>(nwork, cur, nodes, vals, item_boxes, out_nodes,
                                                                 node_counter, nxt, cnt.p, out_tris, out_items,
                                                                 prim_counter, pos, faces, node_cap, overflow);
        else
            k_collapse<false><<<blocks(nwork, 128), 128, 0, st>>>(nwork, cur, nodes, vals, item_boxes, out_nodes,
                                                                  node_counter, nxt, cnt.p, out_tris, out_items,
                                                                  prim_counter, pos, faces, node_cap, overflow);
        OMV_CK(cudaGetLastError());
        uint32_t h = 0;
        OMV_CK(cudaMemcpyAsync(&h, cnt.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        OMV_CK(cudaStreamSynchronize(st));
        nwork = (int)h;
        std::swap(cur, nxt);
    }
    return root_index;
}

void validate_accel(const AccelResult& a, const std::vector<MeshGeom>& meshes, cudaStream_t st);

void build_accel(const std::vector<MeshGeom>& meshes, const std::vector<InstanceGeom>& insts, AccelResult& out,
                 cudaStream_t st)
{
    size_t total_tri = 0;
    for (const auto& m : meshes) total_tri += m.num_faces;
    const uint32_t node_cap = (uint32_t)(total_tri + 2 * meshes.size() + 2 * insts.size() + 16);
    OMV_CK(cudaMalloc(&out.nodes, sizeof(Bvh8Node) * node_cap));
    OMV_CK(cudaMalloc(&out.tris, sizeof(float4) * 3 * (total_tri ? total_tri : 1)));
    OMV_CK(cudaMalloc(&out.tlas_items, sizeof(uint32_t) * (insts.size() ? insts.size() : 1)));
    DBuf<uint32_t> counters(3);  // nodes, prims, overflow
    OMV_CK(cudaMemsetAsync(counters.p, 0, sizeof(uint32_t) * 3, st));
    DBuf<uint32_t> cb(6);
    out.blas_root.assign(meshes.size(), 0xFFFFFFFFu);
    // host SAH trees for the meshes that are small enough, one thread per mesh
    struct HostTree {
        std::vector<Box> boxes;
        std::vector<Node2> nodes;
        std::vector<uint32_t> order;
    };
    std::vector<HostTree> ht(meshes.size());
    {
        std::vector<size_t> todo;
        for (size_t mi = 0; mi < meshes.size(); ++mi)
            if (meshes[mi].valid && meshes[mi].num_faces > 0 && meshes[mi].num_faces <= kHostSahMaxTris &&
                meshes[mi].h_pos && meshes[mi].h_faces)
                todo.push_back(mi);
        std::atomic<size_t> next{0};
        auto worker = [&]() {
            for (size_t j; (j = next.fetch_add(1)) < todo.size();) {
                const MeshGeom& m = meshes[todo[j]];
                HostTree& t = ht[todo[j]];
                t.boxes.resize(m.num_faces);
                for (int f = 0; f < m.num_faces; ++f) {
                    Box& b = t.boxes[f];
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = 3.0e38f;
                        b.hi[a] = -3.0e38f;
                    }
                    bool finite = true;
                    for (int k = 0; k < 3; ++k) {
                        const float* p = m.h_pos + 3 * (size_t)m.h_faces[3 * (size_t)f + k];
                        for (int a = 0; a < 3; ++a) finite = finite && std::isfinite(p[a]);
                    }
                    if (!finite) continue;  // empty box: left out of the tree, as in k_tri_boxes
                    for (int k = 0; k < 3; ++k) {
                        const float* p = m.h_pos + 3 * (size_t)m.h_faces[3 * (size_t)f + k];
                        for (int a = 0; a < 3; ++a) {
                            b.lo[a] = std::min(b.lo[a], p[a]);
                            b.hi[a] = std::max(b.hi[a], p[a]);
                        }
                    }
                }
                host_sah_tree(t.boxes, t.nodes, t.order);
            }
        };
        const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)todo.size()));
        std::vector<std::thread> pool;
        for (unsigned k = 1; k < nt; ++k) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
    }
    for (size_t mi = 0; mi < meshes.size(); ++mi) {
        const MeshGeom& m = meshes[mi];
        if (!m.valid || m.num_faces <= 0) continue;
        const HostTree& t = ht[mi];
        if (!t.boxes.empty()) {
            const int n = m.num_faces;
            DBuf<Box> boxes(n);
            DBuf<uint32_t> vals(n);
            DBuf<Node2> d_nodes(std::max<size_t>(1, t.nodes.size()));
            OMV_CK(cudaMemcpyAsync(boxes.p, t.boxes.data(), sizeof(Box) * n, cudaMemcpyHostToDevice, st));
            OMV_CK(cudaMemcpyAsync(vals.p, t.order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
            if (!t.nodes.empty())
                OMV_CK(cudaMemcpyAsync(d_nodes.p, t.nodes.data(), sizeof(Node2) * t.nodes.size(),
                                       cudaMemcpyHostToDevice, st));
            out.blas_root[mi] = collapse_tree(false, n, d_nodes.p, vals.p, boxes.p, m.d_pos, m.d_faces, out.nodes,
                                              counters.p, node_cap, out.tris, nullptr, counters.p + 1, counters.p + 2,
                                              st);
            continue;
        }
        // very large meshes: device LBVH
        DBuf<Box> boxes(m.num_faces);
        uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
        OMV_CK(cudaMemcpyAsync(cb.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
        k_tri_boxes<<<blocks(m.num_faces, 256), 256, 0, st>>>(m.num_faces, m.d_pos, m.d_faces, boxes.p, cb.p);
        OMV_CK(cudaGetLastError());
        out.blas_root[mi] = build_tree(false, m.num_faces, boxes.p, cb.p, m.d_pos, m.d_faces, out.nodes, counters.p,
                                       node_cap, out.tris, nullptr, counters.p + 1, counters.p + 2, st);
    }
    // top level: world boxes of the valid instances (their referenced vertices
    // through the instance transform), widened so that no object-space hit is
    // ever culled by world-space rounding
    std::vector<uint32_t> ids;
    for (size_t i = 0; i < insts.size(); ++i)
        if (insts[i].valid) ids.push_back((uint32_t)i);
    std::vector<Box> ib(ids.size());
    if (!ids.empty()) {
        DBuf<uint32_t> ob(6 * ids.size());
        std::vector<uint32_t> init(6 * ids.size());
        for (size_t j = 0; j < ids.size(); ++j)
            for (int a = 0; a < 3; ++a) {
                init[6 * j + a] = 0xFFFFFFFFu;
                init[6 * j + 3 + a] = 0u;
            }
        OMV_CK(cudaMemcpyAsync(ob.p, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice, st));
        for (size_t j = 0; j < ids.size(); ++j) {
            const InstanceGeom& g = insts[ids[j]];
            const MeshGeom& m = meshes[g.mesh];
            Xf34 xf;
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 4; ++c) xf.m[4 * a + c] = g.xf[a][c];
            const int nb = std::max(1, std::min(64, blocks((size_t)3 * m.num_faces, 256)));
            k_instance_bounds<<<nb, 256, 0, st>>>(m.num_faces, m.d_pos, m.d_faces, xf, ob.p + 6 * j);
        }
        OMV_CK(cudaGetLastError());
        OMV_CK(cudaMemcpyAsync(init.data(), ob.p, sizeof(uint32_t) * init.size(), cudaMemcpyDeviceToHost, st));
        OMV_CK(cudaStreamSynchronize(st));
        auto dec = [](uint32_t u) {
            const uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
            float f;
            std::memcpy(&f, &b, 4);
            return f;
        };
        for (size_t j = 0; j < ids.size(); ++j) {
            Box& b = ib[j];
            for (int a = 0; a < 3; ++a) {
                b.lo[a] = dec(init[6 * j + a]);
                b.hi[a] = dec(init[6 * j + 3 + a]);
                const float pad = (b.hi[a] - b.lo[a]) * 1e-5f + (std::fabs(b.lo[a]) + std::fabs(b.hi[a])) * 1e-5f + 1e-20f;
                b.lo[a] -= pad;
                b.hi[a] += pad;
            }
        }
    }
    out.num_valid_instances = (uint32_t)ib.size();
    if (!ib.empty()) {
        const int n = (int)ib.size();
        std::vector<Node2> h_nodes;
        std::vector<uint32_t> h_order;
        host_sah_tree(ib, h_nodes, h_order);
        DBuf<Box> boxes(n);
        DBuf<uint32_t> vals(n);
        DBuf<Node2> d_nodes(std::max<size_t>(1, h_nodes.size()));
        OMV_CK(cudaMemcpyAsync(boxes.p, ib.data(), sizeof(Box) * n, cudaMemcpyHostToDevice, st));
        OMV_CK(cudaMemcpyAsync(vals.p, h_order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
        if (!h_nodes.empty())
            OMV_CK(cudaMemcpyAsync(d_nodes.p, h_nodes.data(), sizeof(Node2) * h_nodes.size(), cudaMemcpyHostToDevice,
                                   st));
        OMV_CK(cudaMemsetAsync(counters.p + 1, 0, sizeof(uint32_t), st));
        out.tlas_root = collapse_tree(true, n, d_nodes.p, vals.p, boxes.p, nullptr, nullptr, out.nodes, counters.p,
                                      node_cap, nullptr, out.tlas_items, counters.p + 1, counters.p + 2, st);
        // TLAS items are positions in `ids`; translate to instance indices
        std::vector<uint32_t> items(n);
        OMV_CK(cudaMemcpyAsync(items.data(), out.tlas_items, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st));
        OMV_CK(cudaStreamSynchronize(st));
        for (auto& x : items) x = ids[x];
        OMV_CK(cudaMemcpyAsync(out.tlas_items, items.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
    }
    uint32_t hc[3];
    OMV_CK(cudaMemcpyAsync(hc, counters.p, sizeof(hc), cudaMemcpyDeviceToHost, st));
    OMV_CK(cudaStreamSynchronize(st));
    if (hc[2]) throw std::runtime_error("BVH node capacity exceeded");
    out.num_nodes = hc[0];
    out.num_tris = total_tri;
    validate_accel(out, meshes, st);
}

// Host walk of the finished trees before any traversal runs: every child index,
// primitive range and instance id in bounds, every node reached exactly once.
void validate_accel(const AccelResult& a, const std::vector<MeshGeom>& meshes, cudaStream_t st)
{
    std::vector<Bvh8Node> nodes(a.num_nodes);
    std::vector<float4> tris(3 * a.num_tris);
    std::vector<uint32_t> items(a.num_valid_instances);
    OMV_CK(cudaMemcpyAsync(nodes.data(), a.nodes, sizeof(Bvh8Node) * nodes.size(), cudaMemcpyDeviceToHost, st));
    if (!tris.empty())
        OMV_CK(cudaMemcpyAsync(tris.data(), a.tris, sizeof(float4) * tris.size(), cudaMemcpyDeviceToHost, st));
    if (!items.empty())
        OMV_CK(cudaMemcpyAsync(items.data(), a.tlas_items, sizeof(uint32_t) * items.size(), cudaMemcpyDeviceToHost, st));
    OMV_CK(cudaStreamSynchronize(st));
    std::vector<uint8_t> seen(nodes.size(), 0);
    auto walk = [&](uint32_t root, bool tlas, uint32_t prim_limit, uint32_t face_limit) {
        std::vector<std::pair<uint32_t, int>> stack{{root, 0}};
        while (!stack.empty()) {
            auto [n, depth] = stack.back();
            stack.pop_back();
            if (n >= nodes.size() || seen[n] || depth > 64) throw std::runtime_error("BVH validation: bad node index");
            seen[n] = 1;
            const Bvh8Node& nd = nodes[n];
            const uint32_t imask = nd.exps >> 24;
            for (int s = 0; s < 8; ++s) {
                const uint32_t meta = ((s < 4 ? nd.meta_lo : nd.meta_hi) >> (8 * (s & 3))) & 0xFFu;
                if ((imask >> s) & 1u) {
                    if (meta != (uint32_t)__builtin_popcount(imask & ((1u << s) - 1u)))
                        throw std::runtime_error("BVH validation: internal children not in slot order");
                    stack.push_back({nd.child_base + meta, depth + 1});
                } else if (meta) {
                    const uint32_t cnt = meta >> 5, off = meta & 31u;
                    if (cnt == 0 || cnt > (uint32_t)(tlas ? 1 : kLeafMax) ||
                        (uint64_t)nd.prim_base + off + cnt > prim_limit)
                        throw std::runtime_error("BVH validation: bad leaf range");
                    for (uint32_t k = 0; k < cnt; ++k) {
                        const uint32_t id = nd.prim_base + off + k;
                        if (tlas) {
                            if (items[id] >= face_limit) throw std::runtime_error("BVH validation: bad instance id");
                        } else {
                            uint32_t prim;
                            std::memcpy(&prim, &tris[3 * (size_t)id].w, 4);
                            if (prim >= face_limit) throw std::runtime_error("BVH validation: bad primitive id");
                        }
                    }
                }
            }
        }
    };
    for (size_t i = 0; i < meshes.size(); ++i)
        if (a.blas_root[i] != 0xFFFFFFFFu) walk(a.blas_root[i], false, (uint32_t)a.num_tris, (uint32_t)meshes[i].num_faces);
    if (a.num_valid_instances) walk(a.tlas_root, true, a.num_valid_instances, 0xFFFFFFFFu);
}

}  // namespace omv
