// Device data layout of a committed scene, shared by host and device code.
//
// HBM layout (all arrays 16-byte aligned, read through the read-only path):
//   nodes   : 8-wide BVH nodes, 128 B each (one L2 line); all per-mesh BLAS
//             trees and the instance TLAS live in one array
//   tris    : 48 B per triangle in BLAS-leaf order: 3 x float4 (v0.xyz + primID,
//             v1.xyz, v2.xyz), object space of its mesh
//   verts   : 48 B per vertex: (p.xyz, n.x) (n.yz, t.xy) (t.zw, uv0)
//   faces   : 3 x u32 per face, vertex indices local to the mesh
//   insts   : per instance object<->world transforms, normal matrix and ids
//   env     : equirectangular RGB as float4 texels
#pragma once

#include <cstdint>

#include "../../include/omv.h"

namespace omv {

// 8-wide BVH node, 128 bytes = 8 x uint4:
//   w0 = (px, py, pz, ex | ey<<8 | ez<<16 | imask<<24)
//   w1 = (child_base, prim_base, meta[0..3], meta[4..7])
//   w2..w4 = qlo x/y/z as 8 x u16;  w5..w7 = qhi x/y/z as 8 x u16
// each u16 plane is 0x8000 | q with a 15-bit q (the flag is the exponent bit
// that makes the plane's bytes, shifted up by one byte under 0x3F, the float
// 1 + q * 2^-15); child slot i box: lo = p + q(qlo[i]) * 2^(e-127),
// hi = p + q(qhi[i]) * 2^(e-127).
// imask bit i: slot i is an internal node, at child_base + meta[i].
// leaf slot: meta = (count << 5) | offset, primitives prim_base + offset ...
// empty slot: imask bit clear and meta = 0.
constexpr uint32_t kQuantFlag = 0x8000u;  // set in every stored plane
constexpr uint32_t kQuantMax = 0x7FFFu;   // largest quantised plane q
struct alignas(16) Bvh8Node {
    float px, py, pz;
    uint32_t exps;
    uint32_t child_base;
    uint32_t prim_base;
    uint32_t meta_lo, meta_hi;
    uint16_t qlo[3][8];
    uint16_t qhi[3][8];
};
static_assert(sizeof(Bvh8Node) == 128, "BVH8 node must be 128 bytes");

// triangles per leaf slot: 2 measured fastest on the 1M-triangle benchmark
// frame (37.71 ms; 1: 38.12, 3: 37.91, 4: 38.53)
constexpr int kLeafMax = 2;

struct alignas(16) DevInstance {
    float inv[12];  // world -> object, 3x4 row-major
    float xf[12];   // object -> world
    float nrm[9];   // normal matrix (inverse transpose of the 3x3 part)
    uint32_t mesh;
    uint32_t blas_root;
    uint32_t material;
    uint32_t face_base;
    uint32_t vert_base;
    uint32_t valid;
    uint32_t uv_mask;  // the mesh's coordinate sets: bit 0 TEXCOORD_0, bit 1 TEXCOORD_1
    float4 olo, ohi;   // object-space bounds of the mesh's vertices (w unused)
};

enum : int32_t { kMatPbr = 0, kMatOm = 1, kMatMissing = 2 };

// PBR texture slots
enum : int32_t { kTexBase = 0, kTexMetRough = 1, kTexNormal = 2, kTexOcclusion = 3, kTexEmissive = 4, kTexSlots = 5 };

// one texture slot: image (-1: none), TEXCOORD set, rows 0-1 of the transform
struct DevTexRef {
    int32_t tex;
    int32_t ch;
    float m[6];
};

// one RGBA8 image in the texel pool
struct alignas(16) DevTexture {
    uint32_t offset;  // first texel
    int32_t width, height;
    int32_t present;  // 0: BitmapTexture without an image (samples 0.5 0.5 0.5 1)
};

// material constants precomputed at commit (PhysicallyBasedMaterial with no
// textures, OpenMaterial with IOR evaluated at the RGB wavelengths)
struct alignas(16) DevMaterial {
    int32_t type;
    int32_t transmissive;
    int32_t masked;
    int32_t om_valid;
    float color[4];
    float metal;
    float alpha;  // roughness^2
    float eta;    // 1 / ior, or 1 when double sided
    float rough;  // roughness factor as given (the rmp validation subject)
    float om_n[4];
    float om_k[4];
    // textured PBR (textured != 0): the per-vertex values are resolved from
    // these at shading time; the constants above then hold the factors
    int32_t textured;       // some slot has a valid image
    int32_t alpha_mode;
    int32_t double_sided;
    float cutoff;
    float factor[4];        // base colour factors as given
    float normal_scale, occl_strength;
    float emissive[3];
    int32_t emissive_on;    // |emissive factor| > FLT_EPSILON and an emissive image
    DevTexRef tex[kTexSlots];
};

// environment importance sampling (the MIS estimator): one cell per texel
// square [i, i+1) x [j, j+1) of the lookup's (u, v) grid, weighted by the
// largest luminance its bilinear lookup can reach times its solid angle;
// Vose's alias table over the cells, and each cell's density per steradian
struct DevEnvSampler {
    const float* prob;       // alias threshold of cell i
    const uint32_t* alias;   // alias of cell i
    const float* pdf;        // density per steradian of directions in cell i (0: never sampled)
    int32_t cells;           // width * height, 0 when not built
};

struct DevEnv {
    const float4* rgb;
    int32_t width, height;
    float fwidth, fheight;     // (float)width, (float)height
    float half_u, half_v;      // 0.5f / (float)width, 0.5f / (float)height
    float rot[9];
    float scale;
    int32_t present;
    DevEnvSampler smp;
};

struct DevScene {
    const uint4* nodes;
    uint32_t tlas_root;
    uint32_t num_instances;
    const float4* tris;
    const DevInstance* insts;
    const float4* verts;
    const uint32_t* faces;
    const DevMaterial* mats;
    int32_t num_materials;  // including the missing material (last)
    int32_t num_lights;
    const float4* light_pos;  // xyz, attenuation distance
    const float4* light_int;  // xyz intensity, w unused
    const float* light_cdf;
    float light_max;
    DevEnv env;
    const uchar4* texels;        // all images, RGBA8
    const DevTexture* textures;
    int32_t num_textures;
    const float2* uv1;           // TEXCOORD_1 per vertex (TEXCOORD_0 is in verts), or null
};

// hit record of a closest-hit query
struct alignas(16) HitRec {
    uint32_t inst;  // kInvalid on a miss
    uint32_t prim;
    float u, v;
};

}  // namespace omv
