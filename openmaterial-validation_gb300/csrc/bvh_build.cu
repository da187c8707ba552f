// GPU acceleration-structure build, replacing Embree's BVH build of
// RenderScene::buildEmbreeScene (RenderScene.cpp:225-272): one bottom-level
// tree per mesh (Embree: one scene per mesh) and one top-level tree over the
// instances (Embree: instance geometries in the top scene).
//
// Four builders of the binary tree, one collapse:
//   OMV_BVH_SAH (default, on the device): top-down surface area heuristic
//     over all meshes at once, level by level: binned (32 bins per axis) on
//     ranges of more than 32 items, a full sweep below (Wald 2007); the
//     algorithm of the host build, so the same trace speed.
//   OMV_BVH_PLOC (on the device): item boxes and per-mesh centroid
//     bounds; 30-bit Morton codes; LSD radix sort by (mesh, code); parallel
//     locally-ordered clustering over all meshes at once (Meister and
//     Bittner 2018), one tree per mesh; leaf counts bottom-up, leaf order and
//     node ranges by a walk to the root.
//   OMV_BVH_LBVH (on the device): Morton codes, radix sort, Karras LBVH
//     ("Maximizing parallelism in the construction of BVHs, octrees, and k-d
//     trees", HPG 2012), one thread per internal node, boxes bottom-up with
//     arrival counters; one mesh after another.
//   OMV_BVH_HOST_SAH: binned surface-area-heuristic trees on host threads.
// Collapse (device, level by level): top-down into 8-wide nodes (greedy:
// expand the child of largest surface area; children placed in octant
// slots), leaves of at most kLeafMax triangles, child boxes quantised to 16
// bits per bound against the node box, rounded outward and verified in float
// so the decoded box always contains the true box.  Every box test of the
// traversal is conservative, so hits do not depend on the builder.
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

// exponent byte e such that 2^(e-127) * 32764 >= extent (at most 239, so
// that the traversal's 2^(e-127+15) stays a finite float)
__device__ __forceinline__ uint32_t quant_exponent(float ext)
{
    if (!(ext > 0.0f)) return 1u;
    float s = ext / 32764.0f;
    uint32_t bits = __float_as_uint(s);
    uint32_t e = (bits >> 23) & 0xFF;
    if (bits & 0x7FFFFFu) e += 1;  // round up to a power of two
    if (e < 1) e = 1;
    if (e > 239) e = 239;
    return e;
}

// The meshes of a bottom-level forest: mesh s owns the items (triangles)
// [base, base + its face count) of the forest's item numbering.
struct SegPtr {
    const float* pos;
    const uint32_t* faces;
    uint32_t base;
};

// segment of item g: the last s with segs[s].base <= g
__device__ __forceinline__ int segment_of(const SegPtr* segs, int nseg, uint32_t g)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (segs[mid].base <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <bool kTlas>
__global__ void k_collapse(int nwork, const Work* __restrict__ work, const Node2* nodes, const uint32_t* vals,
                           const Box* item_boxes, Bvh8Node* out_nodes, uint32_t* node_counter, Work* next_work,
                           uint32_t* next_count, float4* out_tris, uint32_t* out_items, uint32_t* prim_counter,
                           const SegPtr* segs, int nseg, uint32_t node_cap, uint32_t* overflow)
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
    for (int s = 0; s < 8; ++s) {  // empty slots: inverted boxes
        meta[s] = 0;
        for (int a = 0; a < 3; ++a) {
            o.qlo[a][s] = kQuantFlag | kQuantMax;
            o.qhi[a][s] = kQuantFlag;
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
            ql = max(0, min((int)kQuantMax, ql));
            qh = max(0, min((int)kQuantMax, qh));
            while (ql > 0 && __fadd_rn(p[a], __fmul_rn((float)ql, sc[a])) > lo) --ql;
            while (qh < (int)kQuantMax && __fadd_rn(p[a], __fmul_rn((float)qh, sc[a])) < hi) ++qh;
            ql = ql > 0 ? ql - 1 : 0;          // one quantum of slack each side
            qh = qh < (int)kQuantMax ? qh + 1 : (int)kQuantMax;
            o.qlo[a][s] = (uint16_t)(kQuantFlag | ql);
            o.qhi[a][s] = (uint16_t)(kQuantFlag | qh);
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
                    const SegPtr& sg = segs[segment_of(segs, nseg, item)];
                    const uint32_t prim = item - sg.base;  // face index within its mesh
                    const uint32_t* f = sg.faces + 3 * (size_t)prim;
                    const float* a0 = sg.pos + 3 * (size_t)f[0];
                    const float* a1 = sg.pos + 3 * (size_t)f[1];
                    const float* a2 = sg.pos + 3 * (size_t)f[2];
                    out_tris[3 * (size_t)dst + 0] = make_float4(a0[0], a0[1], a0[2], __uint_as_float(prim));
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

// sorts (keys, vals) in place by the low 8 * passes key bits (stable, LSD);
// tmp buffers provided; passes even, so the result ends in (keys, vals)
void radix_sort(int n, uint32_t* keys, uint32_t* vals, uint32_t* k2, uint32_t* v2, cudaStream_t st, int passes = 4)
{
    int nb = blocks(n, kSortTile);
    DBuf<uint32_t> hist((size_t)nb * 256);
    uint32_t *ki = keys, *vi = vals, *ko = k2, *vo = v2;
    for (int shift = 0; shift < 8 * passes; shift += 8) {
        k_sort_hist<<<nb, 256, 0, st>>>(n, shift, ki, hist.p, nb);
        k_scan<<<1, 1024, 0, st>>>(nb * 256, hist.p);
        k_sort_scatter<<<nb, kSortThreads, 0, st>>>(n, shift, ki, vi, ko, vo, hist.p, nb);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    OMV_CK(cudaGetLastError());
}

// ------------------------------------------------------------- PLOC ---
// Parallel locally-ordered clustering (D. Meister and J. Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction",
// IEEE TVCG 24(3), 2018): the items of every segment (one mesh, or the
// instances) start as clusters in Morton order; each round, every cluster
// finds the cluster within kPlocRadius positions (same segment) whose union
// box has the smallest surface area, mutual nearest neighbours merge into a
// new node at the lower position, and the survivors are compacted in order.
// The globally cheapest pair (ties to the lowest indices) is always mutual,
// so every round merges at least one pair per segment with two clusters.
constexpr int kPlocRadius = 16;
constexpr int kPlocThreads = 256;
constexpr int kScanBlock = 1024;

__global__ void k_morton_seg(int n, const Box* boxes, const uint32_t* seg_base, int nseg, const uint32_t* cbounds,
                             uint32_t* keys, uint32_t* vals, uint32_t* segs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (seg_base[mid] <= (uint32_t)i)
            lo = mid;
        else
            hi = mid - 1;
    }
    const uint32_t* cb = cbounds + 6 * lo;
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        const float l = ord2f(cb[a]), h = ord2f(cb[3 + a]);
        const float c = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
        const float ext = h - l;
        const float t = ext > 0.f ? (c - l) / ext : 0.5f;
        q[a] = (uint32_t)fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
    }
    keys[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    vals[i] = (uint32_t)i;
    segs[i] = (uint32_t)lo;
}

// segment of every sorted item (the key of the second, segment-major sort)
__global__ void k_gather_u32(int n, const uint32_t* idx, const uint32_t* src, uint32_t* dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

// centroid bounds of n boxes into one segment's six ordered ints
__global__ void k_box_cbounds(int n, const Box* boxes, uint32_t* cbounds)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = i < n;
    for (int a = 0; a < 3; ++a) {
        const float c = ok ? 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]) : 0.0f;
        uint32_t lo = ok ? f2ord(c) : 0xFFFFFFFFu, hi = ok ? f2ord(c) : 0u;
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

// clusters from the sorted items: leaf i (sorted position) is the reference ~i
__global__ void k_ploc_init(int n, const uint32_t* vals, const uint32_t* segs, const Box* item_boxes, int* ref,
                            Box* box, uint32_t* seg, int* leaf_parent)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ref[i] = ~i;
    box[i] = item_boxes[vals[i]];
    seg[i] = segs[i];
    leaf_parent[i] = -1;
}

__global__ void __launch_bounds__(kPlocThreads) k_ploc_nn(int c, const Box* __restrict__ box,
                                                          const uint32_t* __restrict__ seg, int* nn)
{
    constexpr int W = kPlocThreads + 2 * kPlocRadius;
    __shared__ Box sb[W];
    __shared__ uint32_t ss[W];
    const int base = blockIdx.x * kPlocThreads - kPlocRadius;
    for (int t = threadIdx.x; t < W; t += blockDim.x) {
        const int g = base + t;
        const bool in = g >= 0 && g < c;
        ss[t] = in ? seg[g] : 0xFFFFFFFFu;
        if (in) sb[t] = box[g];
    }
    __syncthreads();
    const int i = blockIdx.x * kPlocThreads + threadIdx.x;
    if (i >= c) return;
    const int li = threadIdx.x + kPlocRadius;
    const Box bi = sb[li];
    const uint32_t si = ss[li];
    float best = 3.4e38f;
    int bj = -1;
    for (int d = -kPlocRadius; d <= kPlocRadius; ++d) {  // ascending positions: ties keep the lower one
        if (d == 0 || ss[li + d] != si) continue;
        const float a = half_area(box_union(bi, sb[li + d]));
        if (a < best || bj < 0) {
            best = a;
            bj = i + d;
        }
    }
    nn[i] = bj;
}

__device__ __forceinline__ void set_parent(int ref, int p, int* node_parent, int* leaf_parent)
{
    if (ref >= 0)
        node_parent[ref] = p;
    else
        leaf_parent[~ref] = p;
}

__global__ void k_ploc_merge(int c, const int* __restrict__ nn, int* ref, Box* box, uint32_t* keep, uint32_t* counter,
                             int2* child, Box* node_box, int* node_parent, int* leaf_parent, uint32_t cap,
                             uint32_t* overflow)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c) return;
    const int j = nn[i];
    uint32_t k_ = 1u;
    if (j >= 0 && nn[j] == i) {
        if (i < j) {  // this position takes the new node; position j is dropped
            const uint32_t k = atomicAdd(counter, 1u);
            if (k >= cap) {
                atomicAdd(overflow, 1u);
            } else {
                const int a = ref[i], b = ref[j];
                const Box u = box_union(box[i], box[j]);
                child[k] = make_int2(a, b);
                node_box[k] = u;
                node_parent[k] = -1;
                set_parent(a, (int)k, node_parent, leaf_parent);
                set_parent(b, (int)k, node_parent, leaf_parent);
                ref[i] = (int)k;
                box[i] = u;
            }
        } else {
            k_ = 0u;
        }
    }
    keep[i] = k_;
}

// kept clusters per block of kScanBlock positions (and in total)
__global__ void __launch_bounds__(kScanBlock) k_count_kept(int c, const uint32_t* keep, uint32_t* bsum, uint32_t* total)
{
    __shared__ uint32_t w[kScanBlock / 32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, i < c && keep[i]);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = __popc(m);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = w[threadIdx.x];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if (threadIdx.x == 0) {
            bsum[blockIdx.x] = v;
            atomicAdd(total, v);
        }
    }
}

// order-preserving compaction of the kept clusters (block offsets: the
// exclusive scan of k_count_kept's sums)
__global__ void __launch_bounds__(kScanBlock) k_compact(int c, const uint32_t* keep, const uint32_t* boff,
                                                        const int* ref, const Box* box, const uint32_t* seg,
                                                        int* ref_out, Box* box_out, uint32_t* seg_out)
{
    __shared__ uint32_t w[kScanBlock / 32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const bool k = i < c && keep[i];
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, k);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) w[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x < 32) {
        const uint32_t v = w[threadIdx.x];
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        w[threadIdx.x] = x - v;
    }
    __syncthreads();
    if (!k) return;
    const uint32_t dst = boff[blockIdx.x] + w[warp] + __popc(m & ((1u << lane) - 1u));
    ref_out[dst] = ref[i];
    box_out[dst] = box[i];
    seg_out[dst] = seg[i];
}

// roots get the parent code -2 - segment
__global__ void k_mark_roots(int nseg, const int* ref, int* node_parent, int* leaf_parent)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nseg) set_parent(ref[s], -2 - s, node_parent, leaf_parent);
}

// leaf counts of the internal nodes, bottom-up with arrival counters
__global__ void k_ploc_counts(int n, const int* __restrict__ leaf_parent, const int* node_parent, const int2* child,
                              uint32_t* cnt, uint32_t* arrivals, uint32_t* overflow)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = leaf_parent[i];
    for (int guard = 0; p >= 0; ++guard) {
        if (guard > 4096) {
            atomicAdd(overflow, 1u);
            return;
        }
        __threadfence();
        if (atomicAdd(&arrivals[p], 1u) == 0) return;
        __threadfence();
        const int2 ch = child[p];
        const volatile uint32_t* vc = cnt;
        const uint32_t a = ch.x >= 0 ? vc[ch.x] : 1u, b = ch.y >= 0 ? vc[ch.y] : 1u;
        ((volatile uint32_t*)cnt)[p] = a + b;
        p = node_parent[p];
    }
}

// First position of every node's leaves in the final item order (each tree
// in left-to-right leaf order, segment by segment): the walk to the root adds
// the leaf count of every left sibling on the way.  Threads [0, n) are the
// leaves (sorted positions), [n, n + ni) the internal nodes.
__global__ void k_ploc_place(int n, int ni, const int* leaf_parent, const int* node_parent, const int2* child,
                             const uint32_t* cnt, const uint32_t* seg_start, const uint32_t* vals, uint32_t* vals_out,
                             uint32_t* leaf_pos, uint32_t* node_first, uint32_t* overflow)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n + ni) return;
    int x = t < n ? ~t : t - n;
    int p = t < n ? leaf_parent[t] : node_parent[t - n];
    uint32_t off = 0;
    for (int guard = 0; p >= 0; ++guard) {
        if (guard > 4096) {
            atomicAdd(overflow, 1u);
            return;
        }
        const int2 ch = child[p];
        if (ch.y == x) off += ch.x >= 0 ? cnt[ch.x] : 1u;
        x = p;
        p = node_parent[p];
    }
    const uint32_t first = seg_start[-2 - p] + off;
    if (first >= (uint32_t)n) {  // inconsistent counts: reported, never written
        atomicAdd(overflow, 1u);
        return;
    }
    if (t < n) {
        leaf_pos[t] = first;
        vals_out[first] = vals[t];
    } else {
        node_first[t - n] = first;
    }
}

__global__ void k_ploc_nodes(int ni, const int2* child, const Box* node_box, const int* node_parent,
                             const uint32_t* cnt, const uint32_t* node_first, const uint32_t* leaf_pos, Node2* out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ni) return;
    const int2 ch = child[k];
    Node2 nd;
    nd.left = ch.x >= 0 ? ch.x : ~(int)leaf_pos[~ch.x];
    nd.right = ch.y >= 0 ? ch.y : ~(int)leaf_pos[~ch.y];
    nd.first = (int)node_first[k];
    nd.last = (int)(node_first[k] + cnt[k]) - 1;
    nd.parent = node_parent[k];
    nd.box = node_box[k];
    out[k] = nd;
}

// ------------------------------------------------------- device SAH ---
// Top-down binary trees by the surface area heuristic, leaves of one item,
// the host SAH build's algorithm on the device (I. Wald, "On fast
// Construction of SAH-based Bounding Volume Hierarchies", IEEE RT 2007):
// ranges of more than kSweepMax items are split at the best of kSahBins
// centroid bins per axis (one block per range: bounds, binning in shared
// memory, one warp scans the bins, a stable block-wide partition), smaller
// ranges at the best position of a full sweep over the items sorted along
// each axis (one warp per range: bitonic sort, prefix and suffix box
// unions).  Every range of a level is processed in the same launch, across
// all meshes; a range's items stay contiguous, so node ranges need no
// placement pass.
constexpr int kSahBinsDev = 32;
constexpr int kSweepMaxDev = 32;
constexpr int kSahLargeThreads = 256;

struct SahTask {
    int first, last, node, parent;
};

__device__ __forceinline__ Box empty_box()
{
    Box b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = 3.0e38f;
        b.hi[a] = -3.0e38f;
    }
    return b;
}

// a child range: a leaf reference (~position), or a new internal node and its task
__device__ __forceinline__ int sah_child(int first, int last, int parent, uint32_t* node_counter, SahTask* next_large,
                                         uint32_t* n_large, SahTask* next_small, uint32_t* n_small)
{
    if (first == last) return ~first;
    const int id = (int)atomicAdd(node_counter, 1u);
    const SahTask t{first, last, id, parent};
    if (last - first + 1 > kSweepMaxDev)
        next_large[atomicAdd(n_large, 1u)] = t;
    else
        next_small[atomicAdd(n_small, 1u)] = t;
    return id;
}

__device__ __forceinline__ int sah_bin(float c2, float cmin, float scale)
{
    return (int)fminf((float)(kSahBinsDev - 1), (c2 - cmin) * scale);
}

__global__ void __launch_bounds__(kSahLargeThreads) k_sah_large(const SahTask* __restrict__ tasks,
                                                                const Box* __restrict__ item_boxes, uint32_t* order,
                                                                uint32_t* tmp, Node2* nodes, uint32_t* node_counter,
                                                                SahTask* next_large, uint32_t* n_large,
                                                                SahTask* next_small, uint32_t* n_small)
{
    constexpr int NW = kSahLargeThreads / 32;
    __shared__ uint32_t sbox[6], scen[6];
    __shared__ uint32_t bcnt[3][kSahBinsDev];
    __shared__ uint32_t bbox[3][kSahBinsDev][6];
    __shared__ int s_axis, s_bin, s_nl;
    __shared__ uint32_t wl[NW], wr[NW];
    const SahTask t = tasks[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < 3 * kSahBinsDev; k += blockDim.x) {
        (&bcnt[0][0])[k] = 0u;
        for (int c = 0; c < 3; ++c) {
            bbox[k / kSahBinsDev][k % kSahBinsDev][c] = 0xFFFFFFFFu;
            bbox[k / kSahBinsDev][k % kSahBinsDev][3 + c] = 0u;
        }
    }
    if (tid < 3) {
        sbox[tid] = scen[tid] = 0xFFFFFFFFu;
        sbox[3 + tid] = scen[3 + tid] = 0u;
    }
    __syncthreads();
    // bounds of the boxes and of the doubled centroids
    uint32_t lo[3], hi[3], clo[3], chi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = clo[a] = 0xFFFFFFFFu;
        hi[a] = chi[a] = 0u;
    }
    for (int i = t.first + tid; i <= t.last; i += blockDim.x) {
        const Box b = item_boxes[order[i]];
        for (int a = 0; a < 3; ++a) {
            lo[a] = min(lo[a], f2ord(b.lo[a]));
            hi[a] = max(hi[a], f2ord(b.hi[a]));
            const uint32_t c = f2ord(b.lo[a] + b.hi[a]);
            clo[a] = min(clo[a], c);
            chi[a] = max(chi[a], c);
        }
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o; o >>= 1) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xFFFFFFFFu, lo[a], o));
            hi[a] = max(hi[a], __shfl_xor_sync(0xFFFFFFFFu, hi[a], o));
            clo[a] = min(clo[a], __shfl_xor_sync(0xFFFFFFFFu, clo[a], o));
            chi[a] = max(chi[a], __shfl_xor_sync(0xFFFFFFFFu, chi[a], o));
        }
        if (lane == 0) {
            atomicMin(&sbox[a], lo[a]);
            atomicMax(&sbox[3 + a], hi[a]);
            atomicMin(&scen[a], clo[a]);
            atomicMax(&scen[3 + a], chi[a]);
        }
    }
    __syncthreads();
    float cmin[3], scale[3];
    bool on[3];
    for (int a = 0; a < 3; ++a) {
        cmin[a] = ord2f(scen[a]);
        const float ext = ord2f(scen[3 + a]) - cmin[a];
        on[a] = ext > 0.0f;
        scale[a] = on[a] ? (float)kSahBinsDev / ext : 0.0f;
    }
    // binning
    for (int i = t.first + tid; i <= t.last; i += blockDim.x) {
        const Box b = item_boxes[order[i]];
        for (int a = 0; a < 3; ++a) {
            if (!on[a]) continue;
            const int q = sah_bin(b.lo[a] + b.hi[a], cmin[a], scale[a]);
            atomicAdd(&bcnt[a][q], 1u);
            for (int c = 0; c < 3; ++c) {
                atomicMin(&bbox[a][q][c], f2ord(b.lo[c]));
                atomicMax(&bbox[a][q][3 + c], f2ord(b.hi[c]));
            }
        }
    }
    __syncthreads();
    // one warp: the best boundary between bins q and q + 1 (lane q)
    if (warp == 0) {
        float best = 3.0e38f;
        int best_axis = -1, best_bin = 0;
        for (int a = 0; a < 3; ++a) {
            if (!on[a]) continue;
            const uint32_t c = bcnt[a][lane];
            Box b = empty_box();
            if (c)
                for (int k = 0; k < 3; ++k) {
                    b.lo[k] = ord2f(bbox[a][lane][k]);
                    b.hi[k] = ord2f(bbox[a][lane][3 + k]);
                }
            // prefix (bins 0..lane) and suffix (bins lane..31) unions and counts
            Box pre = b, suf = b;
            uint32_t pc = c, sc = c;
            for (int o = 1; o < 32; o <<= 1) {
                Box x, y;
                for (int k = 0; k < 3; ++k) {
                    x.lo[k] = __shfl_up_sync(0xFFFFFFFFu, pre.lo[k], o);
                    x.hi[k] = __shfl_up_sync(0xFFFFFFFFu, pre.hi[k], o);
                    y.lo[k] = __shfl_down_sync(0xFFFFFFFFu, suf.lo[k], o);
                    y.hi[k] = __shfl_down_sync(0xFFFFFFFFu, suf.hi[k], o);
                }
                const uint32_t xc = __shfl_up_sync(0xFFFFFFFFu, pc, o), yc = __shfl_down_sync(0xFFFFFFFFu, sc, o);
                if (lane >= o) {
                    pre = box_union(x, pre);
                    pc += xc;
                }
                if (lane + o < 32) {
                    suf = box_union(suf, y);
                    sc += yc;
                }
            }
            // right side of boundary `lane`: the suffix from lane + 1
            Box r;
            for (int k = 0; k < 3; ++k) {
                r.lo[k] = __shfl_down_sync(0xFFFFFFFFu, suf.lo[k], 1);
                r.hi[k] = __shfl_down_sync(0xFFFFFFFFu, suf.hi[k], 1);
            }
            const uint32_t rc = __shfl_down_sync(0xFFFFFFFFu, sc, 1);
            float cost = 3.4e38f;
            if (lane < kSahBinsDev - 1 && pc > 0 && rc > 0)
                cost = half_area(pre) * (float)pc + half_area(r) * (float)rc;
            // the first minimum in bin order (ties: the lowest boundary)
            float mc = cost;
            int mq = lane;
            for (int o = 16; o; o >>= 1) {
                const float oc = __shfl_xor_sync(0xFFFFFFFFu, mc, o);
                const int oq = __shfl_xor_sync(0xFFFFFFFFu, mq, o);
                if (oc < mc || (oc == mc && oq < mq)) {
                    mc = oc;
                    mq = oq;
                }
            }
            if (mc < best) {
                best = mc;
                best_axis = a;
                best_bin = mq;
            }
        }
        if (lane == 0) {
            s_axis = best_axis;
            s_bin = best_bin;
            int nl = 0;
            if (best_axis >= 0)
                for (int q = 0; q <= best_bin; ++q) nl += (int)bcnt[best_axis][q];
            s_nl = nl;
        }
    }
    __syncthreads();
    const int cnt = t.last - t.first + 1;
    int split;
    if (s_axis < 0) {
        split = t.first + cnt / 2 - 1;  // no split: halves in the current order
    } else {
        // stable partition into tmp, then back into order
        const int a = s_axis, qb = s_bin, nl = s_nl;
        int lbase = 0, rbase = 0;
        for (int c0 = t.first; c0 <= t.last; c0 += blockDim.x) {
            const int i = c0 + tid;
            const bool ok = i <= t.last;
            const uint32_t item = ok ? order[i] : 0u;
            bool left = false;
            if (ok) {
                const Box b = item_boxes[item];
                left = sah_bin(b.lo[a] + b.hi[a], cmin[a], scale[a]) <= qb;
            }
            const uint32_t ml = __ballot_sync(0xFFFFFFFFu, ok && left), mr = __ballot_sync(0xFFFFFFFFu, ok && !left);
            if (lane == 0) {
                wl[warp] = __popc(ml);
                wr[warp] = __popc(mr);
            }
            __syncthreads();
            int pl = 0, pr = 0, tl = 0, tr = 0;
            for (int w = 0; w < NW; ++w) {
                if (w < warp) {
                    pl += (int)wl[w];
                    pr += (int)wr[w];
                }
                tl += (int)wl[w];
                tr += (int)wr[w];
            }
            const uint32_t below = (1u << lane) - 1u;
            if (ok) {  // positions stay inside the range even if the counts disagreed
                const int dst = left ? t.first + lbase + pl + __popc(ml & below)
                                     : t.first + nl + rbase + pr + __popc(mr & below);
                if (dst >= t.first && dst <= t.last) tmp[dst] = item;
            }
            lbase += tl;
            rbase += tr;
            __syncthreads();
        }
        for (int i = t.first + tid; i <= t.last; i += blockDim.x) order[i] = tmp[i];
        split = t.first + nl - 1;
    }
    if (tid == 0) {
        Node2 nd;
        nd.first = t.first;
        nd.last = t.last;
        nd.parent = t.parent;
        for (int k = 0; k < 3; ++k) {
            nd.box.lo[k] = ord2f(sbox[k]);
            nd.box.hi[k] = ord2f(sbox[3 + k]);
        }
        nd.left = sah_child(t.first, split, t.node, node_counter, next_large, n_large, next_small, n_small);
        nd.right = sah_child(split + 1, t.last, t.node, node_counter, next_large, n_large, next_small, n_small);
        nodes[t.node] = nd;
    }
}

// warp-wide bitonic sort of one 64-bit key per lane, ascending
__device__ __forceinline__ uint64_t warp_sort64(uint64_t key)
{
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= 32; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t lo = __shfl_xor_sync(0xFFFFFFFFu, (uint32_t)key, j);
            const uint32_t hi = __shfl_xor_sync(0xFFFFFFFFu, (uint32_t)(key >> 32), j);
            const uint64_t other = ((uint64_t)hi << 32) | lo;
            const bool up = (lane & k) == 0;
            const bool lower = (lane & j) == 0;
            const uint64_t mn = key < other ? key : other, mx = key < other ? other : key;
            key = (lower == up) ? mn : mx;
        }
    return key;
}

// ranges of 2..kSweepMaxDev items: one warp each, full sweep on every axis
__global__ void k_sah_small(int ntasks, const SahTask* __restrict__ tasks, const Box* __restrict__ item_boxes,
                            uint32_t* order, Node2* nodes, uint32_t* node_counter, SahTask* next_large,
                            uint32_t* n_large, SahTask* next_small, uint32_t* n_small)
{
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (w >= ntasks) return;  // whole warps leave together
    const int lane = threadIdx.x & 31;
    const SahTask t = tasks[w];
    const int cnt = t.last - t.first + 1;
    const bool valid = lane < cnt;
    const uint32_t item = valid ? order[t.first + lane] : 0u;
    const Box b = valid ? item_boxes[item] : empty_box();
    // node box
    Box nb = b;
    for (int o = 16; o; o >>= 1)
        for (int k = 0; k < 3; ++k) {
            nb.lo[k] = fminf(nb.lo[k], __shfl_xor_sync(0xFFFFFFFFu, nb.lo[k], o));
            nb.hi[k] = fmaxf(nb.hi[k], __shfl_xor_sync(0xFFFFFFFFu, nb.hi[k], o));
        }
    float best = 3.0e38f;
    int best_axis = -1, best_k = 0;
    for (int a = 0; a < 3; ++a) {
        // stable order along the axis: key = (doubled centroid, position)
        const uint64_t key = valid ? (((uint64_t)f2ord(b.lo[a] + b.hi[a]) << 32) | (uint32_t)lane) : ~0ull;
        const uint64_t sk = warp_sort64(key);
        const int src = (int)(sk & 31u);
        Box sb;
        for (int k = 0; k < 3; ++k) {
            sb.lo[k] = __shfl_sync(0xFFFFFFFFu, b.lo[k], src);
            sb.hi[k] = __shfl_sync(0xFFFFFFFFu, b.hi[k], src);
        }
        if (lane >= cnt) sb = empty_box();
        Box pre = sb, suf = sb;
        for (int o = 1; o < 32; o <<= 1) {
            Box x, y;
            for (int k = 0; k < 3; ++k) {
                x.lo[k] = __shfl_up_sync(0xFFFFFFFFu, pre.lo[k], o);
                x.hi[k] = __shfl_up_sync(0xFFFFFFFFu, pre.hi[k], o);
                y.lo[k] = __shfl_down_sync(0xFFFFFFFFu, suf.lo[k], o);
                y.hi[k] = __shfl_down_sync(0xFFFFFFFFu, suf.hi[k], o);
            }
            if (lane >= o) pre = box_union(x, pre);
            if (lane + o < 32) suf = box_union(suf, y);
        }
        Box r;
        for (int k = 0; k < 3; ++k) {
            r.lo[k] = __shfl_down_sync(0xFFFFFFFFu, suf.lo[k], 1);
            r.hi[k] = __shfl_down_sync(0xFFFFFFFFu, suf.hi[k], 1);
        }
        float cost = 3.4e38f;
        if (lane < cnt - 1)
            cost = half_area(pre) * (float)(lane + 1) + half_area(r) * (float)(cnt - 1 - lane);
        float mc = cost;
        int mk = lane;
        for (int o = 16; o; o >>= 1) {
            const float oc = __shfl_xor_sync(0xFFFFFFFFu, mc, o);
            const int ok_ = __shfl_xor_sync(0xFFFFFFFFu, mk, o);
            if (oc < mc || (oc == mc && ok_ < mk)) {
                mc = oc;
                mk = ok_;
            }
        }
        if (mc < best) {
            best = mc;
            best_axis = a;
            best_k = mk;
        }
    }
    int split;
    if (best_axis >= 0) {
        const uint64_t key = valid ? (((uint64_t)f2ord(b.lo[best_axis] + b.hi[best_axis]) << 32) | (uint32_t)lane)
                                   : ~0ull;
        const uint64_t sk = warp_sort64(key);
        const uint32_t it = __shfl_sync(0xFFFFFFFFu, item, (int)(sk & 31u));
        if (valid) order[t.first + lane] = it;
        split = t.first + best_k;
    } else {
        split = t.first + cnt / 2 - 1;
    }
    if (lane == 0) {
        Node2 nd;
        nd.first = t.first;
        nd.last = t.last;
        nd.parent = t.parent;
        nd.box = nb;
        nd.left = sah_child(t.first, split, t.node, node_counter, next_large, n_large, next_small, n_small);
        nd.right = sah_child(split + 1, t.last, t.node, node_counter, next_large, n_large, next_small, n_small);
        nodes[t.node] = nd;
    }
}

__global__ void k_iota(int n, uint32_t* v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

__global__ void k_add_u32(int n, uint32_t* v, uint32_t add)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] += add;
}

}  // namespace

// Binary tree by the surface area heuristic, leaves of one item: binned
// (kSahBins bins per axis over the centroid bounds) on ranges of more than
// kSweepMax items, a full sweep over every split position below.  nodes[0] is
// the root; `order` receives the item order the node ranges refer to.  Runs on
// the host (the OMV_BVH_HOST_SAH builder, one thread per mesh); k_sah_large /
// k_sah_small run the same algorithm on the device.
constexpr int kSahBins = 32;
constexpr int kSweepMax = 32;

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


// A binary forest ready for the 8-wide collapse: internal nodes, the item
// order their ranges refer to, and one root reference per tree (an internal
// node, or ~position for a tree of one item).
struct Forest {
    Node2* nodes = nullptr;    // device
    uint32_t* vals = nullptr;  // device, items in tree order
    std::vector<int> roots;
    Forest() = default;
    Forest(const Forest&) = delete;
    Forest& operator=(const Forest&) = delete;
    ~Forest()
    {
        cudaFree(nodes);
        cudaFree(vals);
    }
    void alloc(int n)
    {
        OMV_CK(cudaMalloc(&nodes, sizeof(Node2) * (size_t)std::max(1, n - 1)));
        OMV_CK(cudaMalloc(&vals, sizeof(uint32_t) * (size_t)std::max(1, n)));
    }
};

// Karras LBVH over n items (one tree): 30-bit Morton codes of the centroids
// against `cbounds`, radix sort, one thread per internal node, boxes bottom-up.
static void lbvh_tree(int n, const Box* item_boxes, const uint32_t* cbounds, Forest& f, cudaStream_t st)
{
    f.alloc(n);
    DBuf<uint32_t> keys(n), k2(n), v2(n);
    k_morton<<<blocks(n, 256), 256, 0, st>>>(n, item_boxes, cbounds, keys.p, f.vals);
    radix_sort(n, keys.p, f.vals, k2.p, v2.p, st);
    if (n > 1) {
        DBuf<int> leaf_parent(n), arrivals(n - 1);
        OMV_CK(cudaMemsetAsync(arrivals.p, 0, sizeof(int) * (n - 1), st));
        k_karras<<<blocks(n - 1, 256), 256, 0, st>>>(n, keys.p, f.nodes, leaf_parent.p);
        k_bottom_up<<<blocks(n, 256), 256, 0, st>>>(n, f.vals, item_boxes, f.nodes, leaf_parent.p, arrivals.p);
        OMV_CK(cudaGetLastError());
        OMV_CK(cudaStreamSynchronize(st));  // before the temporaries are freed
    }
    f.roots = {n > 1 ? 0 : ~0};
}

// PLOC forest: one tree per segment (items [seg_base[s], seg_base[s + 1]),
// all non-empty), Morton codes against each segment's centroid bounds
// (cbounds + 6 s), items sorted by (segment, code).
static void ploc_forest(int n, const std::vector<uint32_t>& seg_base, const Box* item_boxes, const uint32_t* cbounds,
                        Forest& f, cudaStream_t st)
{
    const int nseg = (int)seg_base.size();
    const int ni = n - nseg;  // internal nodes of the forest
    f.alloc(n);
    DBuf<uint32_t> d_seg_base(nseg), keys(n), segs(n), k2(n), v2(n);
    OMV_CK(cudaMemcpyAsync(d_seg_base.p, seg_base.data(), sizeof(uint32_t) * nseg, cudaMemcpyHostToDevice, st));
    k_morton_seg<<<blocks(n, 256), 256, 0, st>>>(n, item_boxes, d_seg_base.p, nseg, cbounds, keys.p, f.vals, segs.p);
    radix_sort(n, keys.p, f.vals, k2.p, v2.p, st);
    if (nseg > 1) {  // stable second pass by segment: (segment, code) order
        k_gather_u32<<<blocks(n, 256), 256, 0, st>>>(n, f.vals, segs.p, keys.p);
        radix_sort(n, keys.p, f.vals, k2.p, v2.p, st, nseg <= 256 ? 2 : 4);
    } else {
        OMV_CK(cudaMemsetAsync(keys.p, 0, sizeof(uint32_t) * n, st));
    }
    // clusters (ping-pong), nodes, parents
    DBuf<int> ref0(n), ref1(n), nn(n), leaf_parent(n), node_parent(std::max(1, ni));
    DBuf<Box> box0(n), box1(n), node_box(std::max(1, ni));
    DBuf<uint32_t> seg0(n), seg1(n), keep(n), bsum(blocks(n, kScanBlock)), ctr(3);  // nodes, kept, overflow
    DBuf<int2> child(std::max(1, ni));
    OMV_CK(cudaMemsetAsync(ctr.p, 0, sizeof(uint32_t) * 3, st));
    k_ploc_init<<<blocks(n, 256), 256, 0, st>>>(n, f.vals, keys.p, item_boxes, ref0.p, box0.p, seg0.p, leaf_parent.p);
    int c = n;
    int* ref = ref0.p;
    Box* box = box0.p;
    uint32_t* seg = seg0.p;
    int* ref_o = ref1.p;
    Box* box_o = box1.p;
    uint32_t* seg_o = seg1.p;
    for (int round = 0; c > nseg; ++round) {
        if (round > 10000) throw std::runtime_error("PLOC build did not converge");
        k_ploc_nn<<<blocks(c, kPlocThreads), kPlocThreads, 0, st>>>(c, box, seg, nn.p);
        k_ploc_merge<<<blocks(c, 256), 256, 0, st>>>(c, nn.p, ref, box, keep.p, ctr.p, child.p, node_box.p,
                                                     node_parent.p, leaf_parent.p, (uint32_t)std::max(0, ni), ctr.p + 2);
        const int nb = blocks(c, kScanBlock);
        OMV_CK(cudaMemsetAsync(ctr.p + 1, 0, sizeof(uint32_t), st));
        k_count_kept<<<nb, kScanBlock, 0, st>>>(c, keep.p, bsum.p, ctr.p + 1);
        k_scan<<<1, 1024, 0, st>>>(nb, bsum.p);
        k_compact<<<nb, kScanBlock, 0, st>>>(c, keep.p, bsum.p, ref, box, seg, ref_o, box_o, seg_o);
        OMV_CK(cudaGetLastError());
        uint32_t h[3];
        OMV_CK(cudaMemcpyAsync(h, ctr.p, sizeof(h), cudaMemcpyDeviceToHost, st));
        OMV_CK(cudaStreamSynchronize(st));
        if (h[2]) throw std::runtime_error("PLOC build: node capacity exceeded");
        if ((int)h[1] >= c) throw std::runtime_error("PLOC build made no progress");
        c = (int)h[1];
        std::swap(ref, ref_o);
        std::swap(box, box_o);
        std::swap(seg, seg_o);
    }
    // final item order and Node2 records (ranges of consecutive positions)
    DBuf<uint32_t> cnt(std::max(1, ni)), arrivals(std::max(1, ni)), node_first(std::max(1, ni)), leaf_pos(n),
        d_seg_start(nseg), vals_out(n);
    OMV_CK(cudaMemcpyAsync(d_seg_start.p, seg_base.data(), sizeof(uint32_t) * nseg, cudaMemcpyHostToDevice, st));
    OMV_CK(cudaMemsetAsync(arrivals.p, 0, sizeof(uint32_t) * std::max(1, ni), st));
    k_mark_roots<<<blocks(nseg, 256), 256, 0, st>>>(nseg, ref, node_parent.p, leaf_parent.p);
    k_ploc_counts<<<blocks(n, 256), 256, 0, st>>>(n, leaf_parent.p, node_parent.p, child.p, cnt.p, arrivals.p,
                                                  ctr.p + 2);
    k_ploc_place<<<blocks(n + ni, 256), 256, 0, st>>>(n, ni, leaf_parent.p, node_parent.p, child.p, cnt.p,
                                                      d_seg_start.p, f.vals, vals_out.p, leaf_pos.p, node_first.p,
                                                      ctr.p + 2);
    if (ni > 0)
        k_ploc_nodes<<<blocks(ni, 256), 256, 0, st>>>(ni, child.p, node_box.p, node_parent.p, cnt.p, node_first.p,
                                                      leaf_pos.p, f.nodes);
    OMV_CK(cudaMemcpyAsync(f.vals, vals_out.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
    OMV_CK(cudaGetLastError());
    std::vector<int> roots(nseg);
    uint32_t ov = 0;
    OMV_CK(cudaMemcpyAsync(roots.data(), ref, sizeof(int) * nseg, cudaMemcpyDeviceToHost, st));
    OMV_CK(cudaMemcpyAsync(&ov, ctr.p + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    OMV_CK(cudaStreamSynchronize(st));
    if (ov) throw std::runtime_error("PLOC build: inconsistent tree (deeper than 4096 levels or bad leaf counts)");
    for (int s = 0; s < nseg; ++s) {
        if (roots[s] < 0) {  // a one-item tree: its item's final position
            uint32_t pos = 0;
            OMV_CK(cudaMemcpy(&pos, leaf_pos.p + ~roots[s], sizeof(uint32_t), cudaMemcpyDeviceToHost));
            roots[s] = ~(int)pos;
        }
    }
    f.roots = roots;
}

// Device SAH forest: one tree per segment (items [seg_base[s], seg_base[s + 1])).
static void sah_forest(int n, const std::vector<uint32_t>& seg_base, const Box* item_boxes, Forest& f,
                       cudaStream_t st)
{
    const int nseg = (int)seg_base.size();
    f.alloc(n);
    k_iota<<<blocks(n, 256), 256, 0, st>>>(n, f.vals);
    DBuf<uint32_t> tmp(n), ctr(3);  // nodes, large tasks, small tasks
    DBuf<SahTask> la(n), lb(n), sa(n), sb(n);
    std::vector<SahTask> large, small;
    std::vector<int> roots(nseg);
    int next_id = 0;
    for (int s = 0; s < nseg; ++s) {
        const int first = (int)seg_base[s], last = (s + 1 < nseg ? (int)seg_base[s + 1] : n) - 1;
        if (first == last) {
            roots[s] = ~first;
            continue;
        }
        const SahTask t{first, last, next_id, -2 - s};
        roots[s] = next_id++;
        (last - first + 1 > kSweepMaxDev ? large : small).push_back(t);
    }
    uint32_t h[3] = {(uint32_t)next_id, (uint32_t)large.size(), (uint32_t)small.size()};
    if (!large.empty())
        OMV_CK(cudaMemcpyAsync(la.p, large.data(), sizeof(SahTask) * large.size(), cudaMemcpyHostToDevice, st));
    if (!small.empty())
        OMV_CK(cudaMemcpyAsync(sa.p, small.data(), sizeof(SahTask) * small.size(), cudaMemcpyHostToDevice, st));
    OMV_CK(cudaMemcpyAsync(ctr.p, h, sizeof(h), cudaMemcpyHostToDevice, st));
    SahTask *cl = la.p, *nl = lb.p, *cs = sa.p, *ns = sb.p;
    for (int level = 0; h[1] + h[2] > 0; ++level) {
        if (level > 4096) throw std::runtime_error("device SAH build did not terminate");
        const int nlarge = (int)h[1], nsmall = (int)h[2];
        OMV_CK(cudaMemsetAsync(ctr.p + 1, 0, 2 * sizeof(uint32_t), st));
        if (nlarge)
            k_sah_large<<<nlarge, kSahLargeThreads, 0, st>>>(cl, item_boxes, f.vals, tmp.p, f.nodes, ctr.p, nl,
                                                             ctr.p + 1, ns, ctr.p + 2);
        if (nsmall)
            k_sah_small<<<blocks((size_t)nsmall * 32, 128), 128, 0, st>>>(nsmall, cs, item_boxes, f.vals, f.nodes,
                                                                          ctr.p, nl, ctr.p + 1, ns, ctr.p + 2);
        OMV_CK(cudaGetLastError());
        OMV_CK(cudaMemcpyAsync(h, ctr.p, sizeof(h), cudaMemcpyDeviceToHost, st));
        OMV_CK(cudaStreamSynchronize(st));
        if ((int)h[0] > std::max(1, n - nseg)) throw std::runtime_error("device SAH build: node capacity exceeded");
        std::swap(cl, nl);
        std::swap(cs, ns);
    }
    f.roots = roots;
}

// host SAH tree over n boxes (one tree)
static void host_sah_forest(const std::vector<Box>& boxes, Forest& f, cudaStream_t st)
{
    const int n = (int)boxes.size();
    std::vector<Node2> nodes;
    std::vector<uint32_t> order;
    host_sah_tree(boxes, nodes, order);
    f.alloc(n);
    if (!nodes.empty())
        OMV_CK(cudaMemcpyAsync(f.nodes, nodes.data(), sizeof(Node2) * nodes.size(), cudaMemcpyHostToDevice, st));
    OMV_CK(cudaMemcpyAsync(f.vals, order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
    OMV_CK(cudaStreamSynchronize(st));  // the host vectors go out of scope
    f.roots = {n > 1 ? 0 : ~0};
}

// Top-down collapse of a binary forest into 8-wide nodes appended to
// out_nodes (counters: nodes, primitives, overflow); returns each tree's root.
static std::vector<uint32_t> collapse_forest(bool tlas, const Forest& f, int nitems, const Box* item_boxes,
                                             const SegPtr* segs, int nseg, Bvh8Node* out_nodes, uint32_t* counters,
                                             uint32_t node_cap, float4* out_tris, uint32_t* out_items,
                                             cudaStream_t st)
{
    const int nroots = (int)f.roots.size();
    uint32_t root_index = 0;
    OMV_CK(cudaMemcpyAsync(&root_index, counters, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    OMV_CK(cudaStreamSynchronize(st));
    std::vector<Work> roots(nroots);
    std::vector<uint32_t> out(nroots);
    for (int r = 0; r < nroots; ++r) {
        roots[r] = Work{f.roots[r], root_index + (uint32_t)r};
        out[r] = root_index + (uint32_t)r;
    }
    const uint32_t next = root_index + (uint32_t)nroots;
    OMV_CK(cudaMemcpyAsync(counters, &next, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    DBuf<Work> wa(nitems + nroots), wb(nitems + nroots);
    DBuf<uint32_t> cnt(1);
    OMV_CK(cudaMemcpyAsync(wa.p, roots.data(), sizeof(Work) * nroots, cudaMemcpyHostToDevice, st));
    int nwork = nroots;
    Work *cur = wa.p, *nxt = wb.p;
    for (int level = 0; nwork > 0; ++level) {
        if (level > 200) throw std::runtime_error("BVH collapse did not terminate");
        OMV_CK(cudaMemsetAsync(cnt.p, 0, sizeof(uint32_t), st));
        if (tlas)
            k_collapse<true><<<blocks(nwork, 128), 128, 0, st>>>(nwork, cur, f.nodes, f.vals, item_boxes, out_nodes,
                                                                 counters, nxt, cnt.p, out_tris, out_items,
                                                                 counters + 1, segs, nseg, node_cap, counters + 2);
        else
            k_collapse<false><<<blocks(nwork, 128), 128, 0, st>>>(nwork, cur, f.nodes, f.vals, item_boxes, out_nodes,
                                                                  counters, nxt, cnt.p, out_tris, out_items,
                                                                  counters + 1, segs, nseg, node_cap, counters + 2);
        OMV_CK(cudaGetLastError());
        uint32_t h = 0;
        OMV_CK(cudaMemcpyAsync(&h, cnt.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        OMV_CK(cudaStreamSynchronize(st));
        nwork = (int)h;
        std::swap(cur, nxt);
    }
    return out;
}

void validate_accel(const AccelResult& a, const std::vector<MeshGeom>& meshes, cudaStream_t st);

void build_accel(const std::vector<MeshGeom>& meshes, const std::vector<InstanceGeom>& insts, BvhBuilder builder,
                 AccelResult& out, cudaStream_t st, int nparts)
{
    size_t total_tri = 0;
    for (const auto& m : meshes) total_tri += m.valid ? m.num_faces : 0;
    const uint32_t node_cap = (uint32_t)(total_tri + 2 * meshes.size() + 2 * insts.size() + 16);
    OMV_CK(cudaMalloc(&out.nodes, sizeof(Bvh8Node) * node_cap));
    OMV_CK(cudaMalloc(&out.tris, sizeof(float4) * 3 * (total_tri ? total_tri : 1)));
    OMV_CK(cudaMalloc(&out.tlas_items, sizeof(uint32_t) * (insts.size() ? insts.size() : 1)));
    DBuf<uint32_t> counters(3);  // nodes, prims, overflow
    OMV_CK(cudaMemsetAsync(counters.p, 0, sizeof(uint32_t) * 3, st));
    out.blas_root.assign(meshes.size(), 0xFFFFFFFFu);
    std::vector<size_t> todo;  // meshes with triangles
    for (size_t mi = 0; mi < meshes.size(); ++mi)
        if (meshes[mi].valid && meshes[mi].num_faces > 0) todo.push_back(mi);

    // ---- bottom level: one tree per mesh
    if ((builder == BvhBuilder::Sah || builder == BvhBuilder::Ploc) && !todo.empty()) {
        // every mesh in one forest: one launch sequence for all of them
        std::vector<uint32_t> seg_base(todo.size());
        std::vector<SegPtr> segs(todo.size());
        uint32_t n = 0;
        for (size_t s = 0; s < todo.size(); ++s) {
            const MeshGeom& m = meshes[todo[s]];
            seg_base[s] = n;
            segs[s] = SegPtr{m.d_pos, m.d_faces, n};
            n += (uint32_t)m.num_faces;
        }
        DBuf<Box> boxes(n);
        DBuf<uint32_t> cb(6 * todo.size());
        DBuf<SegPtr> d_segs(todo.size());
        std::vector<uint32_t> init(6 * todo.size());
        for (size_t s = 0; s < todo.size(); ++s)
            for (int a = 0; a < 3; ++a) {
                init[6 * s + a] = 0xFFFFFFFFu;
                init[6 * s + 3 + a] = 0u;
            }
        OMV_CK(cudaMemcpyAsync(cb.p, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice, st));
        OMV_CK(cudaMemcpyAsync(d_segs.p, segs.data(), sizeof(SegPtr) * segs.size(), cudaMemcpyHostToDevice, st));
        for (size_t s = 0; s < todo.size(); ++s) {
            const MeshGeom& m = meshes[todo[s]];
            k_tri_boxes<<<blocks(m.num_faces, 256), 256, 0, st>>>(m.num_faces, m.d_pos, m.d_faces,
                                                                  boxes.p + seg_base[s], cb.p + 6 * s);
        }
        OMV_CK(cudaGetLastError());
        Forest f;
        if (builder == BvhBuilder::Sah)
            sah_forest((int)n, seg_base, boxes.p, f, st);
        else
            ploc_forest((int)n, seg_base, boxes.p, cb.p, f, st);
        const std::vector<uint32_t> roots = collapse_forest(false, f, (int)n, boxes.p, d_segs.p, (int)todo.size(),
                                                            out.nodes, counters.p, node_cap, out.tris, nullptr, st);
        for (size_t s = 0; s < todo.size(); ++s) out.blas_root[todo[s]] = roots[s];
    } else if (builder == BvhBuilder::Lbvh) {
        DBuf<uint32_t> cb(6);
        DBuf<SegPtr> d_seg(1);
        for (size_t mi : todo) {
            const MeshGeom& m = meshes[mi];
            DBuf<Box> boxes(m.num_faces);
            const uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
            const SegPtr sp{m.d_pos, m.d_faces, 0u};
            OMV_CK(cudaMemcpyAsync(cb.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
            OMV_CK(cudaMemcpyAsync(d_seg.p, &sp, sizeof(sp), cudaMemcpyHostToDevice, st));
            k_tri_boxes<<<blocks(m.num_faces, 256), 256, 0, st>>>(m.num_faces, m.d_pos, m.d_faces, boxes.p, cb.p);
            OMV_CK(cudaGetLastError());
            Forest f;
            lbvh_tree(m.num_faces, boxes.p, cb.p, f, st);
            out.blas_root[mi] = collapse_forest(false, f, m.num_faces, boxes.p, d_seg.p, 1, out.nodes, counters.p,
                                                node_cap, out.tris, nullptr, st)[0];
        }
    } else if (builder == BvhBuilder::HostSah) {
        // binned-SAH trees on the host, one thread per mesh
        std::vector<std::vector<Box>> hb(meshes.size());
        std::atomic<size_t> next{0};
        auto worker = [&]() {
            for (size_t j; (j = next.fetch_add(1)) < todo.size();) {
                const MeshGeom& m = meshes[todo[j]];
                std::vector<Box>& bx = hb[todo[j]];
                bx.resize(m.num_faces);
                for (int f = 0; f < m.num_faces; ++f) {
                    Box& b = bx[f];
                    for (int a = 0; a < 3; ++a) {
                        b.lo[a] = 3.0e38f;
                        b.hi[a] = -3.0e38f;
                    }
                    bool finite = true;
                    for (int k = 0; k < 3; ++k) {
                        const float* p = m.h_pos + 3 * (size_t)m.h_faces[3 * (size_t)f + k];
                        for (int a = 0; a < 3; ++a) finite = finite && std::isfinite(p[a]);
                    }
                    if (!finite) continue;  // empty box: no effect on any bound, as in k_tri_boxes
                    for (int k = 0; k < 3; ++k) {
                        const float* p = m.h_pos + 3 * (size_t)m.h_faces[3 * (size_t)f + k];
                        for (int a = 0; a < 3; ++a) {
                            b.lo[a] = std::min(b.lo[a], p[a]);
                            b.hi[a] = std::max(b.hi[a], p[a]);
                        }
                    }
                }
            }
        };
        const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)todo.size()));
        std::vector<std::thread> pool;
        for (unsigned k = 1; k < nt; ++k) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
        DBuf<SegPtr> d_seg(1);
        for (size_t mi : todo) {
            const MeshGeom& m = meshes[mi];
            DBuf<Box> boxes(m.num_faces);
            const SegPtr sp{m.d_pos, m.d_faces, 0u};
            OMV_CK(cudaMemcpyAsync(boxes.p, hb[mi].data(), sizeof(Box) * m.num_faces, cudaMemcpyHostToDevice, st));
            OMV_CK(cudaMemcpyAsync(d_seg.p, &sp, sizeof(sp), cudaMemcpyHostToDevice, st));
            Forest f;
            host_sah_forest(hb[mi], f, st);
            out.blas_root[mi] = collapse_forest(false, f, m.num_faces, boxes.p, d_seg.p, 1, out.nodes, counters.p,
                                                node_cap, out.tris, nullptr, st)[0];
        }
    }
    // ---- top level: world boxes of the valid instances (their referenced
    // vertices through the instance transform), widened so that no
    // object-space hit is ever culled by world-space rounding
    // valid instances grouped by scene (one top-level tree each), in order
    std::vector<uint32_t> ids, part_base(nparts, 0);
    for (int p = 0; p < nparts; ++p) {
        part_base[p] = (uint32_t)ids.size();
        for (size_t i = 0; i < insts.size(); ++i)
            if (insts[i].valid && insts[i].part == p) ids.push_back((uint32_t)i);
        if (ids.size() == part_base[p] && nparts > 1)
            throw std::runtime_error("scene " + std::to_string(p) + " of the group has no valid instance");
    }
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
    out.tlas_roots.assign(nparts, 0xFFFFFFFFu);
    if (!ib.empty()) {
        const int n = (int)ib.size();
        DBuf<Box> boxes(n);
        OMV_CK(cudaMemcpyAsync(boxes.p, ib.data(), sizeof(Box) * n, cudaMemcpyHostToDevice, st));
        OMV_CK(cudaMemsetAsync(counters.p + 1, 0, sizeof(uint32_t), st));
        auto count_of = [&](int p) { return (int)((p + 1 < nparts ? part_base[p + 1] : (uint32_t)n) - part_base[p]); };
        if (builder == BvhBuilder::Sah || builder == BvhBuilder::Ploc) {
            // all scenes' top-level trees in one forest
            Forest f;
            if (builder == BvhBuilder::Sah) {
                sah_forest(n, part_base, boxes.p, f, st);
            } else {
                DBuf<uint32_t> cb(6 * (size_t)nparts);
                std::vector<uint32_t> init(6 * (size_t)nparts);
                for (int p = 0; p < nparts; ++p)
                    for (int a = 0; a < 3; ++a) {
                        init[6 * p + a] = 0xFFFFFFFFu;
                        init[6 * p + 3 + a] = 0u;
                    }
                OMV_CK(cudaMemcpyAsync(cb.p, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice, st));
                for (int p = 0; p < nparts; ++p)
                    k_box_cbounds<<<blocks(count_of(p), 256), 256, 0, st>>>(count_of(p), boxes.p + part_base[p],
                                                                            cb.p + 6 * p);
                OMV_CK(cudaGetLastError());
                ploc_forest(n, part_base, boxes.p, cb.p, f, st);
            }
            out.tlas_roots = collapse_forest(true, f, n, boxes.p, nullptr, 0, out.nodes, counters.p, node_cap, nullptr,
                                             out.tlas_items, st);
        } else {
            // one tree per scene; item numbers made global before the collapse
            for (int p = 0; p < nparts; ++p) {
                const int cnt = count_of(p);
                Forest f;
                if (builder == BvhBuilder::HostSah) {
                    host_sah_forest(std::vector<Box>(ib.begin() + part_base[p], ib.begin() + part_base[p] + cnt), f,
                                    st);
                } else {
                    DBuf<uint32_t> cb(6);
                    const uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
                    OMV_CK(cudaMemcpyAsync(cb.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
                    k_box_cbounds<<<blocks(cnt, 256), 256, 0, st>>>(cnt, boxes.p + part_base[p], cb.p);
                    OMV_CK(cudaGetLastError());
                    lbvh_tree(cnt, boxes.p + part_base[p], cb.p, f, st);
                }
                k_add_u32<<<blocks(cnt, 256), 256, 0, st>>>(cnt, f.vals, part_base[p]);
                OMV_CK(cudaGetLastError());
                out.tlas_roots[p] = collapse_forest(true, f, cnt, boxes.p, nullptr, 0, out.nodes, counters.p, node_cap,
                                                    nullptr, out.tlas_items, st)[0];
            }
        }
        out.tlas_root = out.tlas_roots[0];
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
    if (a.num_valid_instances)
        for (uint32_t r : a.tlas_roots) walk(r, true, a.num_valid_instances, 0xFFFFFFFFu);
}

}  // namespace omv
