// Scene commit and device upload: the work of RenderScene::allocate/set*/
// commitScene (RenderScene.cpp:51-223) and RenderMesh::commitMesh
// (RenderMesh.cpp:246-264), followed by the GPU acceleration build.  The host
// arithmetic below (normal/tangent derivation, normal matrices, IOR lookup) is
// compiled without FMA contraction and follows the reference's operation
// order, so the committed vertex data equal the reference's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "bvh_build.h"
#include "omv_device.cuh"
#include "scene.h"

namespace omv {

namespace {

constexpr float kHEps = 1.1920928955078125e-07f;

struct HV3 {
    float v[3];
};

inline void hcross(const float* a, const float* b, float* r)
{
    float r0 = a[1] * b[2] - a[2] * b[1];
    float r1 = a[2] * b[0] - a[0] * b[2];
    float r2 = a[0] * b[1] - a[1] * b[0];
    r[0] = r0;
    r[1] = r1;
    r[2] = r2;
}
inline float hdot(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void hnormalize(float* a)
{
    float L = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (L != 0.0f) {
        L = 1.0f / L;
        a[0] = a[0] * L;
        a[1] = a[1] * L;
        a[2] = a[2] * L;
    } else {
        a[0] = 1.0f;
        a[1] = 0.0f;
        a[2] = 0.0f;
    }
}

// RenderMesh::computeNormals (RenderMesh.cpp:300-330); v = 10 floats per vertex
void compute_normals(std::vector<float>& v, const uint32_t* f, int vn, int fn)
{
    for (int i = 0; i < vn; ++i) {
        float* cn = &v[(size_t)i * 10 + 3];
        cn[0] = 0.0f;
        cn[1] = 0.0f;
        cn[2] = kHEps;
    }
    for (int i = 0; i < fn; ++i) {
        const float* p0 = &v[(size_t)f[3 * (size_t)i] * 10];
        const float* p1 = &v[(size_t)f[3 * (size_t)i + 1] * 10];
        const float* p2 = &v[(size_t)f[3 * (size_t)i + 2] * 10];
        float v0[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        float v1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        float N[3];
        hcross(v0, v1, N);
        if (N[0] * N[0] + N[1] * N[1] + N[2] * N[2] > kHEps) hnormalize(N);
        for (int j = 0; j < 3; ++j) {
            float* cn = &v[(size_t)f[3 * (size_t)i + j] * 10 + 3];
            cn[0] += N[0];
            cn[1] += N[1];
            cn[2] += N[2];
        }
    }
    for (int i = 0; i < vn; ++i) hnormalize(&v[(size_t)i * 10 + 3]);
}

// RenderMesh::randomTangent (RenderMesh.cpp:418-432)
void random_tangent(const float* nv, float* tv)
{
    const float Zv[3] = {0.0f, 0.0f, 1.0f}, Yv[3] = {0.0f, 1.0f, 0.0f}, Xv[3] = {1.0f, 0.0f, 0.0f};
    if (nv[2] < 0.95f && nv[2] > -0.95f)
        hcross(Zv, nv, tv);
    else if (nv[1] < 0.95f && nv[1] > -0.95f)
        hcross(Yv, nv, tv);
    else
        hcross(Xv, nv, tv);
    hnormalize(tv);
    tv[3] = 1.0f;
    tv[0] *= 1.0f;
    tv[1] *= 1.0f;
    tv[2] *= 1.0f;
}

// RenderMesh::computeTangents(int) (RenderMesh.cpp:332-409)
void compute_tangents_uv(std::vector<float>& v, const uint32_t* f, int vn, int fn, const float* uv, int uvs)
{
    std::vector<float> tv((size_t)vn * 3, 0.0f), bv((size_t)vn * 3, 0.0f);
    for (int i = 0; i < fn; ++i) {
        const uint32_t* fi = f + 3 * (size_t)i;
        const float* X0 = &v[(size_t)fi[0] * 10];
        const float* X1 = &v[(size_t)fi[1] * 10];
        const float* X2 = &v[(size_t)fi[2] * 10];
        const float* U0 = uv + (size_t)fi[0] * uvs;
        const float* U1 = uv + (size_t)fi[1] * uvs;
        const float* U2 = uv + (size_t)fi[2] * uvs;
        float v0[3] = {X1[0] - X0[0], X1[1] - X0[1], X1[2] - X0[2]};
        float v1[3] = {X2[0] - X0[0], X2[1] - X0[1], X2[2] - X0[2]};
        float t0[2] = {U1[0] - U0[0], U1[1] - U0[1]};
        float t1[2] = {U2[0] - U0[0], U2[1] - U0[1]};
        float det = t0[0] * t1[1] - t1[0] * t0[1];
        if (det < kHEps) continue;
        float r = 1.0f / det;
        float S00 = r * t1[1], S01 = -r * t1[0], S10 = -r * t0[1], S11 = r * t0[0];
        float ud[3] = {v0[0] * S00 + v1[0] * S10, v0[1] * S00 + v1[1] * S10, v0[2] * S00 + v1[2] * S10};
        float vd[3] = {v0[0] * S01 + v1[0] * S11, v0[1] * S01 + v1[1] * S11, v0[2] * S01 + v1[2] * S11};
        for (int j = 0; j < 3; ++j) {
            for (int k = 0; k < 3; ++k) {
                tv[3 * (size_t)fi[k] + j] += ud[j];
                bv[3 * (size_t)fi[k] + j] += vd[j];
            }
        }
    }
    for (int i = 0; i < vn; ++i) {
        float* tan = &v[(size_t)i * 10 + 6];
        const float* nv = &v[(size_t)i * 10 + 3];
        const float* t = &tv[3 * (size_t)i];
        float nt = hdot(nv, t);
        tan[0] = t[0] - nv[0] * nt;
        tan[1] = t[1] - nv[1] * nt;
        tan[2] = t[2] - nv[2] * nt;
        float len = std::sqrt(tan[0] * tan[0] + tan[1] * tan[1] + tan[2] * tan[2]);
        if (len <= kHEps) {
            random_tangent(nv, tan);
        } else {
            tan[0] /= len;
            tan[1] /= len;
            tan[2] /= len;
        }
        float c[3];
        hcross(nv, tan, c);
        tan[3] = hdot(c, &bv[3 * (size_t)i]) < 0.0f ? -1.0f : 1.0f;
    }
}

// Interpolation::_get, linear (Interpolation.h:44-78)
float ior_lookup(const float* t, int count, float x)
{
    int l = 0, r = count - 1;
    while ((r - l) > 1) {
        const int m = (l + r) / 2;
        if (x < t[2 * m])
            r = m;
        else
            l = m;
    }
    float dx = t[2 * r] - t[2 * l];
    float dy = t[2 * r + 1] - t[2 * l + 1];
    return t[2 * l + 1] + (x - t[2 * l]) * dy / dx;
}

// inverseMatrix3 / detMatrix3 (UtilityFunctions.h:334-349)
void inverse3(const float M[3][3], float R[3][3])
{
    float det = M[0][0] * M[1][1] * M[2][2] + M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                M[0][2] * M[1][1] * M[2][0] - M[0][1] * M[1][0] * M[2][2] - M[0][0] * M[1][2] * M[2][1];
    float k = (float)(1.0 / (double)det);
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

// world-to-object inverse of a 3x4 affine map, double precision, rounded to float
// (the same function as the oracle's, so both sides see identical object rays)
void affine_inverse(const float xf[3][4], float inv[12])
{
    double a[3][3], r[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = (double)xf[i][j];
    double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    double det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
    double id = 1.0 / det;
    r[0][0] = c00 * id;
    r[1][0] = c01 * id;
    r[2][0] = c02 * id;
    r[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
    r[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * id;
    r[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
    r[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * id;
    r[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
    r[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * id;
    for (int i = 0; i < 3; ++i) {
        double t = -(r[i][0] * (double)xf[0][3] + r[i][1] * (double)xf[1][3] + r[i][2] * (double)xf[2][3]);
        for (int j = 0; j < 3; ++j) inv[4 * i + j] = (float)r[i][j];
        inv[4 * i + 3] = (float)t;
    }
}

const float kRgbWl[3] = {6.50000004e-07f, 5.10000007e-07f, 4.40000008e-07f};

}  // namespace

SceneHost::~SceneHost()
{
    if (device >= 0) cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs) cudaFree(p);
    if (scratch.base) cudaFree(scratch.base);
    if (mat_sets) cudaFree(mat_sets);
    if (d_jobs) cudaFree(d_jobs);
    if (batch_graph) cudaGraphExecDestroy(batch_graph);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (stream) cudaStreamDestroy(stream);
}

void* SceneHost::alloc(size_t bytes)
{
    void* p = nullptr;
    OMV_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
    allocs.push_back(p);
    device_bytes += (int64_t)bytes;
    return p;
}

DevMaterial material_from_desc(const omv_material_desc& md, int num_textures)
{
    DevMaterial m{};
    if (md.type == OMV_MATERIAL_OPENMATERIAL) {
        m.type = kMatOm;
        m.om_valid = md.ior_n_count >= 2 && md.ior_k_count >= 2 && md.ior_n && md.ior_k;
        for (int c = 0; c < 3 && m.om_valid; ++c) {
            const float wl = kRgbWl[c];
            if (wl < std::max(md.ior_n[0], md.ior_k[0]) ||
                wl > std::min(md.ior_n[2 * (md.ior_n_count - 1)], md.ior_k[2 * (md.ior_k_count - 1)]))
                throw ArgError("OpenMATERIAL IOR table does not cover the RGB wavelengths");
            m.om_n[c] = ior_lookup(md.ior_n, md.ior_n_count, wl);
            m.om_k[c] = ior_lookup(md.ior_k, md.ior_k_count, wl);
        }
    } else if (md.type == OMV_MATERIAL_PBR) {
        m.type = kMatPbr;
        for (int c = 0; c < 4; ++c) m.color[c] = 1.0f * md.base_color[c];
        if (md.alpha_mode != OMV_ALPHA_BLEND) m.color[3] = 1.0f;
        m.transmissive = (md.double_sided || m.color[3] < 1.0f) ? 1 : 0;
        m.metal = md.metallic;
        m.rough = md.roughness;
        float rough = md.roughness;
        rough = std::max(0.00001f, std::min(rough, 0.99999f));
        m.alpha = std::pow(rough, 2.0f);
        m.eta = 1.0f / (md.double_sided ? 1.0f : md.ior);
        m.masked = (md.alpha_mode == OMV_ALPHA_MASK && md.base_color[3] < md.alpha_cutoff) ? 1 : 0;
        // textures (PhysicallyBasedMaterial.cpp:27-124): a slot counts when its
        // image index is in range (rangeCheck, :21-22)
        const omv_texture_ref* refs[kTexSlots] = {&md.base_color_texture, &md.metallic_roughness_texture,
                                                  &md.normal_texture, &md.occlusion_texture, &md.emissive_texture};
        for (int k = 0; k < kTexSlots; ++k) {
            DevTexRef& t = m.tex[k];
            t.tex = refs[k]->texture - 1;
            if (t.tex < 0 || t.tex >= num_textures) t.tex = -1;
            t.ch = refs[k]->texcoord;
            for (int r = 0; r < 2; ++r)
                for (int c = 0; c < 3; ++c)
                    t.m[3 * r + c] = refs[k]->has_transform ? refs[k]->transform[r][c] : (r == c ? 1.0f : 0.0f);
            if (t.tex >= 0) m.textured = 1;
        }
        m.alpha_mode = md.alpha_mode;
        m.double_sided = md.double_sided;
        m.cutoff = md.alpha_cutoff;
        for (int c = 0; c < 4; ++c) m.factor[c] = md.base_color[c];
        m.normal_scale = md.normal_scale;
        m.occl_strength = md.occlusion_strength;
        for (int c = 0; c < 3; ++c) m.emissive[c] = md.emissive_factor[c];
        const float el = std::sqrt(md.emissive_factor[0] * md.emissive_factor[0] +
                                   md.emissive_factor[1] * md.emissive_factor[1] +
                                   md.emissive_factor[2] * md.emissive_factor[2]);
        m.emissive_on = (el > kEps && m.tex[kTexEmissive].tex >= 0) ? 1 : 0;
        // isMasked (:301-316): the factor alone, else the base colour texture's alpha per hit
        if (!m.masked && md.alpha_mode == OMV_ALPHA_MASK && m.tex[kTexBase].tex >= 0) m.masked = 2;
    } else {
        throw ArgError("unknown material type");
    }
    return m;
}

// DiffuseColorMaterial (DiffuseColorMaterial.cpp:41-108): the pink stand-in
DevMaterial missing_material()
{
    DevMaterial m{};
    m.type = kMatMissing;
    const float pdf = 1.0f / kPi;
    const float bp = 1.0f / (pdf * kPi);
    m.color[0] = bp * 1000.0f;
    m.color[1] = bp * 0.0f;
    m.color[2] = bp * 1000.0f;
    m.color[3] = 1.0f;
    return m;
}

void set_material_sets(SceneHost& s, int num_sets, const omv_material_desc* descs)
{
    if (num_sets < 0 || (num_sets > 0 && !descs)) throw ArgError("material sets: NULL descriptors");
    const int per = s.num_materials;  // including the missing material
    std::vector<DevMaterial> all((size_t)num_sets * per);
    for (int k = 0; k < num_sets; ++k) {
        for (int i = 0; i + 1 < per; ++i) {
            const DevMaterial m = material_from_desc(descs[(size_t)k * (per - 1) + i], s.num_textures);
            if (m.masked != s.h_mats[i].masked ||
                (m.masked == 2 && (m.tex[kTexBase].tex != s.h_mats[i].tex[kTexBase].tex ||
                                   m.tex[kTexBase].ch != s.h_mats[i].tex[kTexBase].ch ||
                                   m.factor[3] != s.h_mats[i].factor[3] || m.cutoff != s.h_mats[i].cutoff)))
                throw ArgError("material sets cannot change which materials are alpha-masked, or how");
            all[(size_t)k * per + i] = m;
        }
        all[(size_t)k * per + per - 1] = missing_material();
    }
    if (s.mat_sets) {
        // batches still queued on any stream read the old sets
        OMV_CUDA(cudaDeviceSynchronize());
        cudaFree(s.mat_sets);
        s.mat_sets = nullptr;
        s.num_mat_sets = 0;
    }
    if (num_sets > 0) {
        OMV_CUDA(cudaMalloc(&s.mat_sets, sizeof(DevMaterial) * all.size()));
        OMV_CUDA(cudaMemcpy(s.mat_sets, all.data(), sizeof(DevMaterial) * all.size(), cudaMemcpyHostToDevice));
    }
    s.num_mat_sets = num_sets;
}

// Environment sampler for the MIS estimator: cell (i, j) of the lookup grid
// (u in [i, i+1) / W, v in [j, j+1) / H) draws its radiance from texels i, i+1 of
// rows j, j+1 (wrapping, as HDRBackground::getRadiance's bilinear lookup does),
// so its weight is the largest of their luminances times the cell's solid
// angle (2 pi / W)(cos(pi j / H) - cos(pi (j+1) / H)).  Alias table by Vose's
// method (M. D. Vose, "A linear algorithm for generating random numbers with
// a given distribution", IEEE TSE 1991).  Built once per scene on first use.
void ensure_env_sampler(SceneHost& s)
{
    DevEnv& e = s.dev.env;
    if (!e.present || e.smp.cells != 0) return;
    const int W = e.width, H = e.height;
    const size_t n = (size_t)W * H;
    std::vector<float4> tex(n);
    OMV_CUDA(cudaMemcpyAsync(tex.data(), e.rgb, sizeof(float4) * n, cudaMemcpyDeviceToHost, s.stream));
    OMV_CUDA(cudaStreamSynchronize(s.stream));
    std::vector<float> lum(n);
    for (size_t k = 0; k < n; ++k) {
        const float4 t = tex[k];
        lum[k] = std::max(0.0f, 0.2126f * t.x + 0.7152f * t.y + 0.0722f * t.z);
    }
    std::vector<double> w(n), omega(H);
    const double pi = 3.14159265358979323846;
    for (int j = 0; j < H; ++j)
        omega[j] = (2.0 * pi / W) * (std::cos(pi * j / H) - std::cos(pi * (j + 1) / H));
    double total = 0.0;
    for (int j = 0; j < H; ++j)
        for (int i = 0; i < W; ++i) {
            const int i1 = (i + 1) % W, j1 = (j + 1) % H;
            const float m = std::max(std::max(lum[(size_t)j * W + i], lum[(size_t)j * W + i1]),
                                     std::max(lum[(size_t)j1 * W + i], lum[(size_t)j1 * W + i1]));
            const double v = (double)m * omega[j];
            w[(size_t)j * W + i] = v;
            total += v;
        }
    std::vector<float> prob(n, 1.0f), pdf(n, 0.0f);
    std::vector<uint32_t> alias(n);
    for (size_t k = 0; k < n; ++k) alias[k] = (uint32_t)k;
    if (total > 0.0) {
        std::vector<double> q(n);
        std::vector<uint32_t> small, large;
        for (size_t k = 0; k < n; ++k) {
            q[k] = w[k] / total * (double)n;
            (q[k] < 1.0 ? small : large).push_back((uint32_t)k);
            pdf[k] = (float)(w[k] / total / omega[k / W]);
        }
        while (!small.empty() && !large.empty()) {
            const uint32_t a = small.back(), b = large.back();
            small.pop_back();
            prob[a] = (float)q[a];
            alias[a] = b;
            q[b] = (q[b] + q[a]) - 1.0;
            if (q[b] < 1.0) {
                large.pop_back();
                small.push_back(b);
            }
        }
        for (uint32_t k : large) prob[k] = 1.0f;
        for (uint32_t k : small) prob[k] = 1.0f;  // rounding leftovers
    }
    e.smp.prob = s.upload(prob);
    e.smp.alias = s.upload(alias);
    e.smp.pdf = s.upload(pdf);
    e.smp.cells = total > 0.0 ? (int32_t)n : 0;
    if (e.smp.cells == 0) e.smp.cells = -1;  // nothing to sample: built, but empty
    OMV_CUDA(cudaStreamSynchronize(s.stream));
}

void set_scene_materials(SceneHost& s, int num, const omv_material_desc* descs)
{
    if (num != s.num_materials - 1 || (num > 0 && !descs))
        throw ArgError("omv_scene_set_materials needs the scene's number of materials");
    std::vector<DevMaterial> mats(s.num_materials);
    for (int i = 0; i < num; ++i) {
        mats[i] = material_from_desc(descs[i], s.num_textures);
        if (mats[i].masked != s.h_mats[i].masked)
            throw ArgError("omv_scene_set_materials cannot change which materials are alpha-masked");
    }
    mats[num] = missing_material();
    // renders still queued on any stream (the caller's may be non-blocking)
    // read the table: wait for all of the device's work before replacing it
    OMV_CUDA(cudaDeviceSynchronize());
    OMV_CUDA(cudaMemcpy(const_cast<DevMaterial*>(s.dev.mats), mats.data(), sizeof(DevMaterial) * mats.size(),
                        cudaMemcpyHostToDevice));
    s.h_mats = mats;
}

SceneHost* scene_create(const omv_scene_desc& d, int device, const std::vector<int>* inst_part,
                        const std::vector<ScenePart>* parts_in)
{
    std::vector<ScenePart> parts = parts_in ? *parts_in : std::vector<ScenePart>(1);
    if (!parts_in) {
        parts[0].light_count = std::max(0, d.num_lights);
        parts[0].mat_count = std::max(0, d.num_materials);
    }
    const int nparts = (int)parts.size();
    if (d.num_meshes < 0 || d.num_instances < 0 || d.num_materials < 0 || d.num_lights < 0)
        throw ArgError("negative element count in omv_scene_desc");
    if ((d.num_meshes && !d.meshes) || (d.num_instances && !d.instances) || (d.num_materials && !d.materials) ||
        (d.num_lights && !d.lights))
        throw ArgError("NULL array for a non-zero count in omv_scene_desc");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw CudaError("no CUDA device available");
    if (device < 0 || device >= ndev) throw ArgError("device index out of range");
    auto t0 = std::chrono::steady_clock::now();
    OMV_CUDA(cudaSetDevice(device));
    std::unique_ptr<SceneHost> s(new SceneHost);
    s->device = device;
    OMV_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    OMV_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device));

    // ---- materials (+ the missing material, RenderScene.cpp:62-68)
    const int nmat = d.num_materials + 1;
    s->num_textures = std::max(0, d.num_textures);
    std::vector<DevMaterial> mats(nmat);
    std::vector<int> mat_type(nmat);
    for (int i = 0; i < d.num_materials; ++i) {
        mats[i] = material_from_desc(d.materials[i], std::max(0, d.num_textures));
        mat_type[i] = mats[i].type;
    }
    mats[nmat - 1] = missing_material();
    mat_type[nmat - 1] = kMatMissing;

    // ---- meshes
    s->num_meshes = d.num_meshes;
    std::vector<float4> verts;
    std::vector<uint32_t> faces;
    std::vector<uint32_t> face_base(d.num_meshes, 0), vert_base(d.num_meshes, 0), mesh_mat(d.num_meshes, 0);
    std::vector<uint32_t> mesh_uv_mask(d.num_meshes, 0);
    std::vector<float2> uv1;  // TEXCOORD_1 per vertex (only when some mesh has it)
    std::vector<MeshGeom> geo(d.num_meshes);
    std::vector<std::vector<float>> pos3(d.num_meshes);
    s->mesh_face_prefix.assign(d.num_meshes + 1, 0);
    s->mesh_vert_count.assign(d.num_meshes, 0);
    for (int i = 0; i < d.num_meshes; ++i) {
        const omv_mesh_desc& md = d.meshes[i];
        const bool valid = md.num_vertices > 0 && md.num_faces > 0 && md.positions && md.faces;
        int mat = md.material;
        int norm_ch = -1;  // PhysicallyBasedMaterial::getNormalTextureChannel = normalTexture.texCoord
        if (mat >= 0 && mat < nmat - 1)
            norm_ch = mat_type[mat] == kMatPbr ? d.materials[mat].normal_texture.texcoord : -1;
        else
            mat = nmat - 1;
        mesh_mat[i] = (uint32_t)mat;
        s->mesh_face_prefix[i + 1] = s->mesh_face_prefix[i] + (valid ? (uint32_t)md.num_faces : 0u);
        if (!valid) continue;
        s->mesh_vert_count[i] = (uint32_t)md.num_vertices;
        if (md.position_stride < 3 || (md.normals && md.normal_stride < 3) || (md.tangents && md.tangent_stride < 4) ||
            (md.texcoord0 && md.texcoord_stride < 2))
            throw ArgError("mesh stride smaller than its element size");
        const int vn = md.num_vertices, fn = md.num_faces;
        for (int64_t k = 0; k < 3LL * fn; ++k)
            if (md.faces[k] >= (uint32_t)vn) throw ArgError("face index out of range in mesh " + std::to_string(i));
        std::vector<float> v((size_t)vn * 10, 0.0f);
        for (int k = 0; k < vn; ++k) {
            std::memcpy(&v[(size_t)k * 10], md.positions + (size_t)k * md.position_stride, 3 * sizeof(float));
            if (md.normals)
                std::memcpy(&v[(size_t)k * 10 + 3], md.normals + (size_t)k * md.normal_stride, 3 * sizeof(float));
            if (md.tangents)
                std::memcpy(&v[(size_t)k * 10 + 6], md.tangents + (size_t)k * md.tangent_stride, 4 * sizeof(float));
        }
        if (!md.normals) compute_normals(v, md.faces, vn, fn);
        if (!md.tangents) {
            const float* tuv = norm_ch == 0 ? md.texcoord0 : (norm_ch == 1 && md.texcoord0 ? md.texcoord1 : nullptr);
            if (tuv)
                compute_tangents_uv(v, md.faces, vn, fn, tuv, md.texcoord_stride);
            else
                for (int k = 0; k < vn; ++k) random_tangent(&v[(size_t)k * 10 + 3], &v[(size_t)k * 10 + 6]);
        }
        vert_base[i] = (uint32_t)(verts.size() / 3);
        face_base[i] = (uint32_t)(faces.size() / 3);
        for (int k = 0; k < vn; ++k) {
            const float* x = &v[(size_t)k * 10];
            verts.push_back(make_float4(x[0], x[1], x[2], x[3]));
            verts.push_back(make_float4(x[4], x[5], x[6], x[7]));
            const float* t0 = md.texcoord0 ? md.texcoord0 + (size_t)k * md.texcoord_stride : nullptr;
            verts.push_back(make_float4(x[8], x[9], t0 ? t0[0] : 0.0f, t0 ? t0[1] : 0.0f));
        }
        mesh_uv_mask[i] = (md.texcoord0 ? 1u : 0u) | (md.texcoord0 && md.texcoord1 ? 2u : 0u);
        if (md.texcoord0 && md.texcoord1) {
            uv1.resize(verts.size() / 3, make_float2(0.0f, 0.0f));
            for (int k = 0; k < vn; ++k) {
                const float* t1 = md.texcoord1 + (size_t)k * md.texcoord_stride;
                uv1[vert_base[i] + k] = make_float2(t1[0], t1[1]);
            }
        }
        faces.insert(faces.end(), md.faces, md.faces + 3 * (size_t)fn);
        MeshGeom& g = geo[i];
        g.valid = true;
        g.num_faces = fn;
        pos3[i].resize((size_t)vn * 3);
        for (int k = 0; k < vn; ++k)
            for (int a = 0; a < 3; ++a) pos3[i][3 * (size_t)k + a] = v[(size_t)k * 10 + a];
        for (int a = 0; a < 3; ++a) {
            g.lo[a] = 3.0e38f;
            g.hi[a] = -3.0e38f;
        }
        for (int64_t k = 0; k < 3LL * fn; ++k) {
            const float* p = &v[(size_t)md.faces[k] * 10];
            for (int a = 0; a < 3; ++a) {
                g.lo[a] = std::min(g.lo[a], p[a]);
                g.hi[a] = std::max(g.hi[a], p[a]);
            }
        }
        s->num_triangles += 0;  // counted per instance below
    }

    // ---- instances
    s->num_instances = d.num_instances;
    std::vector<DevInstance> insts(d.num_instances);
    std::vector<InstanceGeom> igeo(d.num_instances);
    int nvalid = 0;
    for (int i = 0; i < d.num_instances; ++i) {
        const omv_instance_desc& id = d.instances[i];
        DevInstance& I = insts[i];
        std::memset(&I, 0, sizeof(I));
        float xf[3][4];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) {
                xf[r][c] = id.transform[r][c];
                I.xf[4 * r + c] = id.transform[r][c];
            }
        affine_inverse(xf, I.inv);
        float TM[3][3], NM[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) TM[a][b] = id.transform[b][a];
        inverse3(TM, NM);  // RenderInstance::computeNormalMatrix
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) I.nrm[3 * a + b] = NM[a][b];
        const bool valid = id.mesh >= 0 && id.mesh < d.num_meshes && geo[id.mesh].valid;
        I.valid = valid ? 1u : 0u;
        I.mesh = valid ? (uint32_t)id.mesh : 0u;
        I.material = valid ? mesh_mat[id.mesh] : (uint32_t)(nmat - 1);
        I.face_base = valid ? face_base[id.mesh] : 0u;
        I.vert_base = valid ? vert_base[id.mesh] : 0u;
        I.uv_mask = valid ? mesh_uv_mask[id.mesh] : 0u;
        if (valid) {
            const MeshGeom& g = geo[id.mesh];
            I.olo = make_float4(g.lo[0], g.lo[1], g.lo[2], 0.0f);
            I.ohi = make_float4(g.hi[0], g.hi[1], g.hi[2], 0.0f);
        } else {  // never entered: invalid instances are not in the top-level tree
            I.olo = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            I.ohi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        igeo[i].valid = valid;
        igeo[i].mesh = valid ? id.mesh : -1;
        igeo[i].part = inst_part ? (*inst_part)[i] : 0;
        std::memcpy(igeo[i].xf, xf, sizeof(xf));
        if (valid) {
            ++nvalid;
            s->num_triangles += d.meshes[id.mesh].num_faces;
        }
    }
    if (nvalid == 0) throw std::runtime_error("incomplete scene cannot be rendered: no valid instance");

    // ---- upload geometry, build the acceleration structure
    for (int i = 0; i < d.num_meshes; ++i) {
        if (!geo[i].valid) continue;
        float* dp = static_cast<float*>(s->alloc(pos3[i].size() * sizeof(float)));
        OMV_CUDA(cudaMemcpyAsync(dp, pos3[i].data(), pos3[i].size() * sizeof(float), cudaMemcpyHostToDevice,
                                 s->stream));
        uint32_t* df = static_cast<uint32_t*>(s->alloc(sizeof(uint32_t) * 3 * (size_t)d.meshes[i].num_faces));
        OMV_CUDA(cudaMemcpyAsync(df, d.meshes[i].faces, sizeof(uint32_t) * 3 * (size_t)d.meshes[i].num_faces,
                                 cudaMemcpyHostToDevice, s->stream));
        geo[i].d_pos = dp;
        geo[i].d_faces = df;
        geo[i].h_pos = pos3[i].data();
        geo[i].h_faces = d.meshes[i].faces;
    }
    if (d.bvh_builder < OMV_BVH_SAH || d.bvh_builder > OMV_BVH_HOST_SAH) throw ArgError("unknown bvh_builder");
    AccelResult acc;
    build_accel(geo, igeo, static_cast<BvhBuilder>(d.bvh_builder), acc, s->stream, nparts);
    for (int p = 0; p < nparts; ++p) parts[p].tlas_root = acc.tlas_roots[p];
    s->allocs.push_back(acc.nodes);
    s->allocs.push_back(acc.tris);
    s->allocs.push_back(acc.tlas_items);
    s->device_bytes += (int64_t)acc.num_nodes * 128 + (int64_t)acc.num_tris * 48;
    s->tlas_items = acc.tlas_items;
    for (int i = 0; i < d.num_instances; ++i)
        if (insts[i].valid) insts[i].blas_root = acc.blas_root[insts[i].mesh];
    s->blas_nodes = acc.num_nodes;
    s->tlas_nodes = 0;

    DevScene& D = s->dev;
    D.nodes = reinterpret_cast<const uint4*>(acc.nodes);
    D.tlas_root = acc.tlas_root;
    D.num_instances = (uint32_t)d.num_instances;
    D.tris = acc.tris;
    D.insts = s->upload(insts);
    D.verts = s->upload(verts);
    D.faces = s->upload(faces);
    D.mats = s->upload(mats);
    D.num_materials = nmat;
    if (!uv1.empty()) {
        uv1.resize(verts.size() / 3, make_float2(0.0f, 0.0f));
        D.uv1 = s->upload(uv1);
    }
    // ---- textures (RenderScene::setTexture): one texel pool
    if (s->num_textures > 0) {
        if (!d.textures) throw ArgError("num_textures > 0 with NULL textures");
        std::vector<DevTexture> tt(s->num_textures);
        std::vector<uchar4> texels;
        for (int i = 0; i < s->num_textures; ++i) {
            const omv_texture_desc& td = d.textures[i];
            const bool ok = td.rgba && td.width > 0 && td.height > 0;
            if (ok && (int64_t)td.width * td.height > ((int64_t)1 << 28)) throw ArgError("texture too large");
            tt[i].offset = (uint32_t)texels.size();
            tt[i].width = ok ? td.width : 1;
            tt[i].height = ok ? td.height : 1;
            tt[i].present = ok ? 1 : 0;
            if (ok) {
                const uchar4* p = reinterpret_cast<const uchar4*>(td.rgba);
                texels.insert(texels.end(), p, p + (size_t)td.width * td.height);
            }
            if (texels.size() > 0xFFFFFFFFull) throw ArgError("texel pool too large");
        }
        if (texels.empty()) texels.push_back(make_uchar4(0, 0, 0, 0));
        D.texels = s->upload(texels);
        D.textures = s->upload(tt);
        D.num_textures = s->num_textures;
        s->device_bytes += (int64_t)texels.size() * 4;
    }
    s->num_materials = nmat;
    s->h_mats = mats;
    s->d_face_prefix = s->upload(s->mesh_face_prefix);

    // ---- lights (RenderLightPoint::set, DistanceRandom CDF per scene of a group)
    s->num_lights = d.num_lights;
    {
        std::vector<float4> lp(std::max(1, d.num_lights)), li(std::max(1, d.num_lights));
        std::vector<float> cdf(std::max(1, d.num_lights));
        for (ScenePart& P : parts) {
            float acc_p = 0.0f;
            for (int i = P.light_base; i < P.light_base + P.light_count; ++i) {
                const omv_light_desc& l = d.lights[i];
                lp[i] = make_float4(l.position[0], l.position[1], l.position[2], l.range > 0.0f ? l.range : kFltMax);
                li[i] = make_float4(l.intensity[0], l.intensity[1], l.intensity[2], 0.0f);
                float power = 0.2126f * l.intensity[0] + 0.7152f * l.intensity[1] + 0.0722f * l.intensity[2];
                acc_p = acc_p + power;
                cdf[i] = acc_p;
            }
            P.light_max = P.light_count > 0 ? cdf[P.light_base + P.light_count - 1] : 0.0f;
        }
        D.light_pos = s->upload(lp);
        D.light_int = s->upload(li);
        D.light_cdf = s->upload(cdf);
        // the single-frame calls render scene 0
        D.num_lights = parts[0].light_count;
        D.light_max = parts[0].light_max;
    }
    s->parts = parts;

    // ---- environment
    D.env.present = 0;
    if (d.hdri) {
        const omv_hdri_desc& h = *d.hdri;
        if (h.width <= 0 || h.height <= 0 || !h.rgb) throw ArgError("invalid HDRI description");
        std::vector<float4> tex((size_t)h.width * h.height);
        for (size_t k = 0; k < tex.size(); ++k)
            tex[k] = make_float4(h.rgb[3 * k], h.rgb[3 * k + 1], h.rgb[3 * k + 2], 0.0f);
        D.env.rgb = s->upload(tex);
        D.env.width = h.width;
        D.env.height = h.height;
        D.env.fwidth = (float)h.width;
        D.env.fheight = (float)h.height;
        D.env.half_u = 0.5f / D.env.fwidth;  // the lookup's 0.5f / (float)W, rounded alike
        D.env.half_v = 0.5f / D.env.fheight;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) D.env.rot[3 * r + c] = h.rotation[r][c];
        D.env.scale = h.scale;
        D.env.present = 1;
    }
    OMV_CUDA(cudaStreamSynchronize(s->stream));
    s->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return s.release();
}

SceneHost* scene_create_group(int num, const omv_scene_desc* descs, int device)
{
    if (num == 1) return scene_create(descs[0], device);
    std::vector<omv_mesh_desc> meshes;
    std::vector<omv_instance_desc> insts;
    std::vector<omv_material_desc> mats;
    std::vector<omv_light_desc> lights;
    std::vector<omv_texture_desc> texs;
    std::vector<int> inst_part;
    std::vector<ScenePart> parts(num);
    for (int p = 0; p < num; ++p) {
        const omv_scene_desc& d = descs[p];
        if (d.num_meshes < 0 || d.num_instances < 0 || d.num_materials < 0 || d.num_lights < 0 ||
            d.num_textures < 0)
            throw ArgError("negative element count in scene " + std::to_string(p) + " of the group");
        if ((d.num_meshes && !d.meshes) || (d.num_instances && !d.instances) || (d.num_materials && !d.materials) ||
            (d.num_lights && !d.lights) || (d.num_textures && !d.textures))
            throw ArgError("NULL array for a non-zero count in scene " + std::to_string(p) + " of the group");
        const omv_hdri_desc* h0 = descs[0].hdri;
        if ((d.hdri != nullptr) != (h0 != nullptr))
            throw ArgError("the scenes of a group share one HDRI background or none has one");
        if (h0 && d.hdri != h0) {
            const omv_hdri_desc& h = *d.hdri;
            bool same = h.width == h0->width && h.height == h0->height && h.scale == h0->scale && h.rgb && h0->rgb &&
                        std::memcmp(h.rotation, h0->rotation, sizeof(h.rotation)) == 0;
            same = same && std::memcmp(h.rgb, h0->rgb, sizeof(float) * 3 * (size_t)h.width * h.height) == 0;
            if (!same) throw ArgError("the scenes of a group share one HDRI background or none has one");
        }
        if ((d.num_lights > 0) != (descs[0].num_lights > 0))
            throw ArgError("either every scene of a group has point lights or none has");
        const int mesh_base = (int)meshes.size(), mat_base = (int)mats.size(), tex_base = (int)texs.size();
        parts[p].mat_base = mat_base;
        parts[p].mat_count = d.num_materials;
        parts[p].light_base = (int)lights.size();
        parts[p].light_count = d.num_lights;
        for (int i = 0; i < d.num_meshes; ++i) {
            omv_mesh_desc m = d.meshes[i];
            m.material = (m.material >= 0 && m.material < d.num_materials) ? mat_base + m.material : -1;
            meshes.push_back(m);
        }
        for (int i = 0; i < d.num_instances; ++i) {
            omv_instance_desc in = d.instances[i];
            in.mesh = (in.mesh >= 0 && in.mesh < d.num_meshes) ? mesh_base + in.mesh : -1;
            insts.push_back(in);
            inst_part.push_back(p);
        }
        for (int i = 0; i < d.num_materials; ++i) {
            omv_material_desc m = d.materials[i];
            for (omv_texture_ref* r : {&m.base_color_texture, &m.metallic_roughness_texture, &m.normal_texture,
                                       &m.occlusion_texture, &m.emissive_texture})
                if (r->texture > 0) r->texture += tex_base;
            mats.push_back(m);
        }
        lights.insert(lights.end(), d.lights, d.lights + d.num_lights);
        texs.insert(texs.end(), d.textures, d.textures + d.num_textures);
    }
    omv_scene_desc g{};
    g.num_meshes = (int32_t)meshes.size();
    g.meshes = meshes.data();
    g.num_instances = (int32_t)insts.size();
    g.instances = insts.data();
    g.num_materials = (int32_t)mats.size();
    g.materials = mats.data();
    g.num_lights = (int32_t)lights.size();
    g.lights = lights.data();
    g.hdri = descs[0].hdri;
    g.num_textures = (int32_t)texs.size();
    g.textures = texs.data();
    g.bvh_builder = descs[0].bvh_builder;
    return scene_create(g, device, &inst_part, &parts);
}

// ------------------------------------------------------- kernel hooks ---
namespace {

__global__ void k_hook_eval(int64_t n, const float* in, float* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* x = in + 17 * i;
    V3 r = bsdf_eval_direct(v3(x[0], x[1], x[2]), v3(x[3], x[4], x[5]), v3(x[6], x[7], x[8]), x + 9, x[13], x[14]);
    out[3 * i] = r.x;
    out[3 * i + 1] = r.y;
    out[3 * i + 2] = r.z;
}

__global__ void k_hook_sample(int64_t n, const float* in, float* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* x = in + 24 * i;
    BsdfIn d;
    d.I = v3(x[0], x[1], x[2]);
    d.N = v3(x[3], x[4], x[5]);
    d.T = v3(x[6], x[7], x[8]);
    for (int c = 0; c < 4; ++c) d.color[c] = x[9 + c];
    d.metal = x[13];
    d.alpha = x[14];
    d.eta = x[15];
    d.transmissive = x[16] != 0.0f;
    V3 O;
    V3 w = bsdf_sample_indirect(d, x[17], x[18], x[19], O);
    float* o = out + 6 * i;
    o[0] = O.x;
    o[1] = O.y;
    o[2] = O.z;
    o[3] = w.x;
    o[4] = w.y;
    o[5] = w.z;
}

__global__ void k_hook_om(int64_t n, const float* in, float* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* x = in + 7 * i;
    for (int c = 0; c < 3; ++c) out[3 * i + c] = om_channel(x[c], x[3 + c], x[6]);
}

__global__ void k_hook_camera(omv_camera cam, const float* jitter, float* rays)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cam.width * cam.height) return;
    V3 O, R;
    camera_ray(cam, p % cam.width, p / cam.width, jitter[2 * (size_t)p], jitter[2 * (size_t)p + 1], O, R);
    float* r = rays + 6 * (size_t)p;
    r[0] = O.x;
    r[1] = O.y;
    r[2] = O.z;
    r[3] = R.x;
    r[4] = R.y;
    r[5] = R.z;
}

// the correctly rounded library functions, one per launch (OMV_FN_*)
__global__ void k_hook_library(int fn, int64_t n, const float* in, float* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = in[i];
    float y = 0.0f, c = 0.0f;
    switch (fn) {
    case OMV_FN_SIN: cr::sincos_cr(x, y, c); break;
    case OMV_FN_COS: cr::sincos_cr(x, c, y); break;
    case OMV_FN_ASIN: y = cr::asin_cr(x); break;
    case OMV_FN_ACOS: y = cr::acos_cr(x); break;
    case OMV_FN_POW5: y = cr::pow5_cr(x); break;
    default: y = cr::rcp_sq_cr(x); break;
    }
    out[i] = y;
}

inline int hb(int64_t n) { return (int)std::max<int64_t>(1, (n + 255) / 256); }

}  // namespace

void hook_eval_direct(int64_t n, const float* in, float* out, cudaStream_t st)
{
    k_hook_eval<<<hb(n), 256, 0, st>>>(n, in, out);
    OMV_CUDA(cudaGetLastError());
}
void hook_sample_indirect(int64_t n, const float* in, float* out, cudaStream_t st)
{
    k_hook_sample<<<hb(n), 256, 0, st>>>(n, in, out);
    OMV_CUDA(cudaGetLastError());
}
void hook_om_fresnel(int64_t n, const float* in, float* out, cudaStream_t st)
{
    k_hook_om<<<hb(n), 256, 0, st>>>(n, in, out);
    OMV_CUDA(cudaGetLastError());
}
void hook_library_function(int fn, int64_t n, const float* in, float* out, cudaStream_t st)
{
    k_hook_library<<<hb(n), 256, 0, st>>>(fn, n, in, out);
    OMV_CUDA(cudaGetLastError());
}
void hook_camera_rays(const omv_camera& cam, const float* jitter, float* rays, cudaStream_t st)
{
    k_hook_camera<<<hb((int64_t)cam.width * cam.height), 256, 0, st>>>(cam, jitter, rays);
    OMV_CUDA(cudaGetLastError());
}

}  // namespace omv
