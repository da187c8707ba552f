/*
 * ORACLE -- test infrastructure only (see oc_core.h).  CPU restatement of the
 * reference's bidirectional render loop and everything it calls per sample.
 * Each function names the reference function it restates; the float operation
 * order follows the reference so that mode 0 of oc_render reproduces the
 * reference renderer at -C 1 bit for bit (same std::mt19937 stream, same
 * closest-hit contract through oc_bvh.c, which also backs the Embree shim).
 */
#include "oc_render.h"

#include <complex.h>
#undef I /* complex.h macro; the reference uses I for the incident direction */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#include "oc_bvh.h"
#include "oc_core.h"

#define OC_INVALID 0xFFFFFFFFu
#define OC_EPS_ACC 3.0f /* BDPTRenderer::m_fEpsAcc (BDPTRenderer.h:43) */

enum { MAT_PBR = 0, MAT_OM = 1, MAT_MISSING = 2 };

/* PbrMaterial::TextureData (PbrMaterial.h:24-34): image index (-1: none),
 * TEXCOORD set and the first two rows of the 3x3 transformation */
typedef struct oc_tref {
    int tex, ch;
    float m[2][3];
} oc_tref;

enum { TEX_BASE = 0, TEX_METROUGH = 1, TEX_NORMAL = 2, TEX_OCCLUSION = 3, TEX_EMISSIVE = 4, TEX_SLOTS = 5 };

typedef struct oc_mat {
    int type;
    float color[4];
    float metal, rough, ior;
    int alpha_mode;
    float cutoff;
    int double_sided;
    float om_n[3], om_k[3];
    int has_ior;
    oc_tref tref[TEX_SLOTS];
    float normal_scale, occl_strength, emissive[3];
} oc_mat;

/* BitmapTexture (BitmapTexture.cpp): 8-bit RGBA texels */
typedef struct oc_tex {
    int w, h;
    unsigned char* rgba;
} oc_tex;

typedef struct oc_mesh_r {
    int valid;
    int vn, fn, mat;
    uint32_t* faces;
    float* v; /* vn * 10: position, normal, tangent(4) */
    float* uv[2]; /* TEXCOORD_0 / _1: vn * 2, or NULL */
    oc_tri_mesh geo;
} oc_mesh_r;

typedef struct oc_inst_r {
    int mesh; /* -1: invalid */
    float M[4][4];
    float N[3][3];
} oc_inst_r;

struct oc_scene {
    int n_mesh;
    oc_mesh_r* meshes;
    int n_inst;
    oc_inst_r* inst;
    oc_accel accel;
    int n_mat; /* including the missing material (last) */
    oc_mat* mats;
    int n_light;
    float (*lpos)[3];
    float (*lint)[3];
    float* lrange;
    float* lcdf;
    float lmax;
    int has_bg;
    int bg_w, bg_h;
    float* bg; /* bg_w*bg_h*3 */
    float bg_R[3][3];
    float bg_scale;
    int n_tex;
    oc_tex* tex;
};

/* ------------------------------------------------------------ commit --- */

/* RenderMesh::computeNormals (RenderMesh.cpp:300-330) */
static void compute_normals(oc_mesh_r* m)
{
    for (int i = 0; i < m->vn; ++i) {
        float* cn = m->v + (size_t)i * 10 + 3;
        cn[0] = 0.0f; cn[1] = 0.0f; cn[2] = OC_EPS;
    }
    for (int i = 0; i < m->fn; ++i) {
        const uint32_t* f = m->faces + 3 * (size_t)i;
        const float* p0 = m->v + (size_t)f[0] * 10;
        const float* p1 = m->v + (size_t)f[1] * 10;
        const float* p2 = m->v + (size_t)f[2] * 10;
        float v0[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        float v1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        float N[3];
        oc_cross3(v0, v1, N);
        if (N[0] * N[0] + N[1] * N[1] + N[2] * N[2] > OC_EPS) oc_normalize3(N);
        for (int j = 0; j < 3; ++j) {
            float* cn = m->v + (size_t)f[j] * 10 + 3;
            cn[0] += N[0]; cn[1] += N[1]; cn[2] += N[2];
        }
    }
    for (int i = 0; i < m->vn; ++i) oc_normalize3(m->v + (size_t)i * 10 + 3);
}

/* RenderMesh::randomTangent (RenderMesh.cpp:418-432) */
static void random_tangent(const float* nv, float* tv)
{
    const float Zv[3] = {0.0f, 0.0f, 1.0f}, Yv[3] = {0.0f, 1.0f, 0.0f}, Xv[3] = {1.0f, 0.0f, 0.0f};
    if (nv[2] < 0.95f && nv[2] > -0.95f)
        oc_cross3(Zv, nv, tv);
    else if (nv[1] < 0.95f && nv[1] > -0.95f)
        oc_cross3(Yv, nv, tv);
    else
        oc_cross3(Xv, nv, tv);
    oc_normalize3(tv);
    tv[3] = 1.0f;
    tv[0] *= 1.0f; tv[1] *= 1.0f; tv[2] *= 1.0f;
}

/* RenderMesh::computeTangents(int) from texture coordinates (RenderMesh.cpp:332-409) */
static void compute_tangents_uv(oc_mesh_r* m, const float* uv, int uv_stride)
{
    float(*tv)[3] = (float(*)[3])calloc((size_t)m->vn, sizeof(float[3]));
    float(*bv)[3] = (float(*)[3])calloc((size_t)m->vn, sizeof(float[3]));
    for (int i = 0; i < m->fn; ++i) {
        const uint32_t* f = m->faces + 3 * (size_t)i;
        const float* X0 = m->v + (size_t)f[0] * 10;
        const float* X1 = m->v + (size_t)f[1] * 10;
        const float* X2 = m->v + (size_t)f[2] * 10;
        const float* U0 = uv + (size_t)f[0] * uv_stride;
        const float* U1 = uv + (size_t)f[1] * uv_stride;
        const float* U2 = uv + (size_t)f[2] * uv_stride;
        float v0[3] = {X1[0] - X0[0], X1[1] - X0[1], X1[2] - X0[2]};
        float v1[3] = {X2[0] - X0[0], X2[1] - X0[1], X2[2] - X0[2]};
        float t0[2] = {U1[0] - U0[0], U1[1] - U0[1]};
        float t1[2] = {U2[0] - U0[0], U2[1] - U0[1]};
        float det = t0[0] * t1[1] - t1[0] * t0[1];
        if (det < OC_EPS) continue;
        float r = 1.0f / det;
        float SI[2][2];
        SI[0][0] = r * t1[1]; SI[0][1] = -r * t1[0];
        SI[1][0] = -r * t0[1]; SI[1][1] = r * t0[0];
        float udir[3] = {v0[0] * SI[0][0] + v1[0] * SI[1][0], v0[1] * SI[0][0] + v1[1] * SI[1][0],
                         v0[2] * SI[0][0] + v1[2] * SI[1][0]};
        float vdir[3] = {v0[0] * SI[0][1] + v1[0] * SI[1][1], v0[1] * SI[0][1] + v1[1] * SI[1][1],
                         v0[2] * SI[0][1] + v1[2] * SI[1][1]};
        for (int j = 0; j < 3; ++j) {
            tv[f[0]][j] += udir[j]; tv[f[1]][j] += udir[j]; tv[f[2]][j] += udir[j];
            bv[f[0]][j] += vdir[j]; bv[f[1]][j] += vdir[j]; bv[f[2]][j] += vdir[j];
        }
    }
    for (int i = 0; i < m->vn; ++i) {
        float* tan = m->v + (size_t)i * 10 + 6;
        const float* nv = m->v + (size_t)i * 10 + 3;
        float nv_tv = oc_dot3(nv, tv[i]);
        tan[0] = tv[i][0] - nv[0] * nv_tv;
        tan[1] = tv[i][1] - nv[1] * nv_tv;
        tan[2] = tv[i][2] - nv[2] * nv_tv;
        float len = oc_length3(tan);
        if (len <= OC_EPS) {
            random_tangent(nv, tan);
        } else {
            tan[0] /= len; tan[1] /= len; tan[2] /= len;
        }
        float nvtv[3];
        oc_cross3(nv, tan, nvtv);
        tan[3] = oc_dot3(nvtv, bv[i]) < 0.0f ? -1.0f : 1.0f;
    }
    free(tv);
    free(bv);
}

/* AssetMaterialIor::getIor linear-interpolation branch + Interpolation::_get
 * (AssetMaterialIor.cpp:133-145, Interpolation.h:44-78); table sorted by x */
float oc_ior_lookup(const float* t, int32_t count, float x)
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

static const float RGB_WL[3] = {6.50000004e-07f, 5.10000007e-07f, 4.40000008e-07f};

oc_scene* oc_scene_create(const omv_scene_desc* d)
{
    oc_scene* s = (oc_scene*)calloc(1, sizeof(oc_scene));
    if (!s) return NULL;
    s->n_mat = d->num_materials + 1;
    s->mats = (oc_mat*)calloc((size_t)s->n_mat, sizeof(oc_mat));
    for (int i = 0; i < d->num_materials; ++i) {
        const omv_material_desc* md = &d->materials[i];
        oc_mat* m = &s->mats[i];
        if (md->type == OMV_MATERIAL_OPENMATERIAL) {
            m->type = MAT_OM;
            m->has_ior = md->ior_n_count >= 2 && md->ior_k_count >= 2;
            for (int c = 0; c < 3 && m->has_ior; ++c) {
                m->om_n[c] = oc_ior_lookup(md->ior_n, md->ior_n_count, RGB_WL[c]);
                m->om_k[c] = oc_ior_lookup(md->ior_k, md->ior_k_count, RGB_WL[c]);
            }
        } else {
            m->type = MAT_PBR;
            memcpy(m->color, md->base_color, sizeof(m->color));
            m->metal = md->metallic;
            m->rough = md->roughness;
            m->ior = md->ior;
            m->alpha_mode = md->alpha_mode;
            m->cutoff = md->alpha_cutoff;
            m->double_sided = md->double_sided;
            const omv_texture_ref* refs[TEX_SLOTS] = {&md->base_color_texture, &md->metallic_roughness_texture,
                                                     &md->normal_texture, &md->occlusion_texture,
                                                     &md->emissive_texture};
            for (int k = 0; k < TEX_SLOTS; ++k) {
                oc_tref* t = &m->tref[k];
                t->tex = refs[k]->texture - 1;
                t->ch = refs[k]->texcoord;
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 3; ++b)
                        t->m[a][b] = refs[k]->has_transform ? refs[k]->transform[a][b] : (a == b ? 1.0f : 0.0f);
            }
            m->normal_scale = md->normal_scale;
            m->occl_strength = md->occlusion_strength;
            memcpy(m->emissive, md->emissive_factor, sizeof(m->emissive));
        }
    }
    for (int i = 0; i < s->n_mat; ++i)
        if (s->mats[i].type != MAT_PBR)
            for (int k = 0; k < TEX_SLOTS; ++k) s->mats[i].tref[k].tex = -1;
    s->n_tex = d->num_textures > 0 ? d->num_textures : 0;
    s->tex = (oc_tex*)calloc((size_t)(s->n_tex > 0 ? s->n_tex : 1), sizeof(oc_tex));
    for (int i = 0; i < s->n_tex; ++i) {
        const omv_texture_desc* td = &d->textures[i];
        oc_tex* t = &s->tex[i];
        t->w = td->width;
        t->h = td->height;
        if (td->rgba && t->w > 0 && t->h > 0) {
            t->rgba = (unsigned char*)malloc((size_t)t->w * t->h * 4);
            memcpy(t->rgba, td->rgba, (size_t)t->w * t->h * 4);
        }
    }
    oc_mat* miss = &s->mats[s->n_mat - 1]; /* DiffuseColorMaterial(BDPT_MISSING_MATERIAL_COLOR) */
    miss->type = MAT_MISSING;
    miss->color[0] = 1000.0f; miss->color[1] = 0.0f; miss->color[2] = 1000.0f; miss->color[3] = 1.0f;

    s->n_mesh = d->num_meshes;
    s->meshes = (oc_mesh_r*)calloc((size_t)(s->n_mesh > 0 ? s->n_mesh : 1), sizeof(oc_mesh_r));
    for (int i = 0; i < s->n_mesh; ++i) {
        const omv_mesh_desc* md = &d->meshes[i];
        oc_mesh_r* m = &s->meshes[i];
        m->vn = md->num_vertices;
        m->fn = md->num_faces;
        m->mat = md->material;
        m->valid = m->vn > 0 && m->fn > 0 && md->positions && md->faces;
        if (!m->valid) continue;
        m->faces = (uint32_t*)malloc(sizeof(uint32_t) * 3 * (size_t)m->fn);
        memcpy(m->faces, md->faces, sizeof(uint32_t) * 3 * (size_t)m->fn);
        m->v = (float*)calloc((size_t)m->vn * 10, sizeof(float));
        for (int k = 0; k < m->vn; ++k) {
            memcpy(m->v + (size_t)k * 10, md->positions + (size_t)k * md->position_stride, 3 * sizeof(float));
            if (md->normals) memcpy(m->v + (size_t)k * 10 + 3, md->normals + (size_t)k * md->normal_stride, 3 * sizeof(float));
            if (md->tangents) memcpy(m->v + (size_t)k * 10 + 6, md->tangents + (size_t)k * md->tangent_stride, 4 * sizeof(float));
        }
        const float* uvs[2] = {md->texcoord0, md->texcoord0 ? md->texcoord1 : NULL};
        for (int c = 0; c < 2; ++c) {
            if (!uvs[c]) continue;
            m->uv[c] = (float*)malloc(sizeof(float) * 2 * (size_t)m->vn);
            for (int k = 0; k < m->vn; ++k)
                memcpy(m->uv[c] + 2 * (size_t)k, uvs[c] + (size_t)k * md->texcoord_stride, 2 * sizeof(float));
        }
        /* RenderScene::commitScene material resolution (RenderScene.cpp:158-176):
         * PhysicallyBasedMaterial::getNormalTextureChannel = normalTexture.texCoord */
        int norm_ch = -1;
        if (m->mat >= 0 && m->mat < s->n_mat - 1) {
            norm_ch = s->mats[m->mat].type == MAT_PBR ? d->materials[m->mat].normal_texture.texcoord : -1;
        } else {
            m->mat = s->n_mat - 1;
        }
        if (!md->normals) compute_normals(m);
        if (!md->tangents) {
            if (norm_ch >= 0 && norm_ch < 2 && m->uv[norm_ch])
                compute_tangents_uv(m, m->uv[norm_ch], 2);
            else
                for (int k = 0; k < m->vn; ++k) random_tangent(m->v + (size_t)k * 10 + 3, m->v + (size_t)k * 10 + 6);
        }
        m->geo.n_tri = m->fn;
        m->geo.idx = m->faces;
        m->geo.idx_stride = 3 * sizeof(uint32_t);
        m->geo.vtx = (const unsigned char*)m->v;
        m->geo.vtx_stride = 10 * sizeof(float);
        m->geo.geom_id = (uint32_t)i;
        oc_build_mesh_bvh(&m->geo);
    }
    s->n_inst = d->num_instances;
    s->inst = (oc_inst_r*)calloc((size_t)(s->n_inst > 0 ? s->n_inst : 1), sizeof(oc_inst_r));
    s->accel.inst = (oc_instance*)calloc((size_t)(s->n_inst > 0 ? s->n_inst : 1), sizeof(oc_instance));
    int valid = 0;
    for (int i = 0; i < s->n_inst; ++i) {
        oc_inst_r* in = &s->inst[i];
        memcpy(in->M, d->instances[i].transform, sizeof(in->M));
        float TM[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) TM[a][b] = in->M[b][a];
        oc_inverse3((const float(*)[3])TM, in->N); /* RenderInstance::computeNormalMatrix */
        int mi = d->instances[i].mesh;
        in->mesh = (mi >= 0 && mi < s->n_mesh && s->meshes[mi].valid) ? mi : -1;
        if (in->mesh < 0) continue;
        oc_instance* ai = &s->accel.inst[s->accel.n_inst++];
        ai->mesh = &s->meshes[in->mesh].geo;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 4; ++b) ai->xf[a][b] = in->M[a][b];
        ai->inst_id = (uint32_t)i;
        ++valid;
    }
    if (valid == 0) {
        oc_scene_destroy(s);
        return NULL;
    }
    oc_build_tlas(&s->accel);
    /* lights: RenderLightPoint::set + DistanceRandom CDF (RenderScene.cpp:212-220) */
    s->n_light = d->num_lights;
    if (s->n_light > 0) {
        s->lpos = (float(*)[3])malloc(sizeof(float[3]) * (size_t)s->n_light);
        s->lint = (float(*)[3])malloc(sizeof(float[3]) * (size_t)s->n_light);
        s->lrange = (float*)malloc(sizeof(float) * (size_t)s->n_light);
        s->lcdf = (float*)malloc(sizeof(float) * (size_t)s->n_light);
        float acc = 0.0f;
        for (int i = 0; i < s->n_light; ++i) {
            memcpy(s->lpos[i], d->lights[i].position, sizeof(float[3]));
            memcpy(s->lint[i], d->lights[i].intensity, sizeof(float[3]));
            s->lrange[i] = d->lights[i].range > 0.0f ? d->lights[i].range : FLT_MAX;
            float power = 0.2126f * s->lint[i][0] + 0.7152f * s->lint[i][1] + 0.0722f * s->lint[i][2];
            acc = acc + power;
            s->lcdf[i] = acc;
        }
        s->lmax = s->lcdf[s->n_light - 1];
    }
    if (d->hdri && d->hdri->rgb && d->hdri->width > 0 && d->hdri->height > 0) {
        s->has_bg = 1;
        s->bg_w = d->hdri->width;
        s->bg_h = d->hdri->height;
        size_t n = (size_t)s->bg_w * s->bg_h * 3;
        s->bg = (float*)malloc(n * sizeof(float));
        memcpy(s->bg, d->hdri->rgb, n * sizeof(float));
        memcpy(s->bg_R, d->hdri->rotation, sizeof(s->bg_R));
        s->bg_scale = d->hdri->scale;
    }
    return s;
}

void oc_scene_destroy(oc_scene* s)
{
    if (!s) return;
    for (int i = 0; i < s->n_mesh; ++i) {
        free(s->meshes[i].faces);
        free(s->meshes[i].v);
        free(s->meshes[i].uv[0]);
        free(s->meshes[i].uv[1]);
        oc_free_bvh(&s->meshes[i].geo.bvh);
    }
    free(s->meshes);
    free(s->inst);
    free(s->accel.inst);
    oc_free_bvh(&s->accel.tlas);
    free(s->mats);
    free(s->lpos);
    free(s->lint);
    free(s->lrange);
    free(s->lcdf);
    free(s->bg);
    for (int i = 0; i < s->n_tex; ++i) free(s->tex[i].rgba);
    free(s->tex);
    free(s);
}

int32_t oc_scene_mesh_info(const oc_scene* s, int32_t mesh, int32_t* vn, int32_t* fn, int32_t* mat)
{
    if (mesh < 0 || mesh >= s->n_mesh) return -1;
    *vn = s->meshes[mesh].vn;
    *fn = s->meshes[mesh].fn;
    *mat = s->meshes[mesh].mat;
    return 0;
}

int32_t oc_scene_mesh_vertices(const oc_scene* s, int32_t mesh, float* out)
{
    if (mesh < 0 || mesh >= s->n_mesh || !s->meshes[mesh].valid) return -1;
    memcpy(out, s->meshes[mesh].v, sizeof(float) * 10 * (size_t)s->meshes[mesh].vn);
    return 0;
}

int32_t oc_scene_normal_matrix(const oc_scene* s, int32_t inst, float* out9)
{
    if (inst < 0 || inst >= s->n_inst) return -1;
    memcpy(out9, s->inst[inst].N, sizeof(float) * 9);
    return 0;
}

/* ------------------------------------------------------ surface points --- */

typedef struct oc_sp {
    int inst, mesh, face;
    float bary[3];
    float pos[3], nrm[3], tan[4], bin[3];
    int is_tex_norm;
} oc_sp;

/* mirror of RTCRayHit as the reference uses it */
typedef struct oc_rh {
    float org[3], tnear, dir[3], tfar;
    uint32_t geom, inst, prim;
    float u, v;
} oc_rh;

/* RenderMesh::computeSurfacePoint (RenderMesh.cpp:159-196) */
static void mesh_surface_point(const oc_mesh_r* m, oc_sp* sp, const float M[4][4], const float N[3][3])
{
    sp->is_tex_norm = 0;
    const float* b = sp->bary;
    const uint32_t* fi = m->faces + 3 * (size_t)sp->face;
    const float* v[3] = {m->v + (size_t)fi[0] * 10, m->v + (size_t)fi[1] * 10, m->v + (size_t)fi[2] * 10};
    float pp[3], pn[3], pbn[3], pt[4];
    for (int i = 0; i < 3; ++i) {
        pp[i] = b[0] * v[0][i] + b[1] * v[1][i] + b[2] * v[2][i];
        pn[i] = b[0] * v[0][3 + i] + b[1] * v[1][3 + i] + b[2] * v[2][3 + i];
        pt[i] = b[0] * v[0][6 + i] + b[1] * v[1][6 + i] + b[2] * v[2][6 + i];
    }
    pt[3] = b[0] * v[0][9] + b[1] * v[1][9] + b[2] * v[2][9];
    pt[3] = pt[3] >= 0.0f ? 1.0f : -1.0f;
    oc_normalize_if_needed3(pn);
    float tn = oc_dot3(pn, pt);
    pt[0] -= tn * pn[0];
    pt[1] -= tn * pn[1];
    pt[2] -= tn * pn[2];
    oc_normalize_if_needed3(pt);
    oc_cross3(pn, pt, pbn);
    pbn[0] *= pt[3];
    pbn[1] *= pt[3];
    pbn[2] *= pt[3];
    oc_xform_point(M, pp, sp->pos);
    oc_mat3_vec(N, pn, sp->nrm);
    oc_mat3_vec(N, pt, sp->tan);
    oc_mat3_vec(N, pbn, sp->bin);
    oc_normalize_if_needed3(sp->nrm);
    oc_normalize_if_needed3(sp->tan);
    oc_normalize_if_needed3(sp->bin);
    sp->tan[3] = pt[3];
}

/* BDPTRenderer::computeSurfacePoint (BDPTRenderer.cpp:57-73) */
static void compute_surface_point(const oc_scene* s, const oc_rh* h, oc_sp* sp)
{
    sp->mesh = (int)h->geom;
    sp->inst = (int)h->inst;
    sp->face = (int)h->prim;
    sp->bary[0] = 1.0f - h->u - h->v;
    sp->bary[1] = h->u;
    sp->bary[2] = h->v;
    const oc_inst_r* in = &s->inst[sp->inst];
    mesh_surface_point(&s->meshes[sp->mesh], sp, (const float(*)[4])in->M, (const float(*)[3])in->N);
}

/* SurfacePoint::applyTextureNormal (SurfacePoint.cpp:19-34) */
static void apply_texture_normal(oc_sp* sp, const float* tn)
{
    if (sp->is_tex_norm) return;
    float nn[3] = {tn[0] * sp->tan[0] + tn[1] * sp->bin[0] + tn[2] * sp->nrm[0],
                   tn[0] * sp->tan[1] + tn[1] * sp->bin[1] + tn[2] * sp->nrm[1],
                   tn[0] * sp->tan[2] + tn[1] * sp->bin[2] + tn[2] * sp->nrm[2]};
    oc_normalize_if_needed3_to(nn, sp->nrm);
    oc_cross3(sp->bin, sp->nrm, sp->tan);
    oc_normalize_if_needed3(sp->tan);
    oc_cross3(sp->nrm, sp->tan, sp->bin);
    for (int i = 0; i < 3; ++i) sp->bin[i] = sp->tan[3] * sp->bin[i];
    sp->is_tex_norm = 1;
}

/* triangleNormal (UtilityFunctions.h:542-547) of the hit face, through the
 * instance normal matrix, normalised (OpenMaterial.cpp:76-86) */
static void face_normal(const oc_scene* s, const oc_sp* sp, float* tfn)
{
    const oc_mesh_r* m = &s->meshes[sp->mesh];
    const uint32_t* fi = m->faces + 3 * (size_t)sp->face;
    const float* P0 = m->v + (size_t)fi[0] * 10;
    const float* P1 = m->v + (size_t)fi[1] * 10;
    const float* P2 = m->v + (size_t)fi[2] * 10;
    const float E1[3] = {P1[0] - P0[0], P1[1] - P0[1], P1[2] - P0[2]};
    const float E2[3] = {P2[0] - P0[0], P2[1] - P0[1], P2[2] - P0[2]};
    float fn[3];
    oc_cross3(E1, E2, fn);
    oc_mat3_vec((const float(*)[3])s->inst[sp->inst].N, fn, tfn);
    oc_normalize3(tfn);
}

/* ---------------------------------------------------------- textures --- */

/* BitmapTexture::getPixCoords + texture(u, v, fvec4) (BitmapTexture.cpp:73-125):
 * bilinear, wrapping, texels scaled by 1/255 */
static void tex_sample(const oc_tex* t, float u, float v, float* out)
{
    if (!t->rgba) {
        out[0] = out[1] = out[2] = 0.5f;
        out[3] = 1.0f;
        return;
    }
    const int W = t->w, H = t->h;
    float upage = floorf(u - 0.5f / (float)W);
    float vpage = floorf(v - 0.5f / (float)H);
    u -= upage;
    v -= vpage;
    u *= (float)W;
    v *= (float)H;
    int iu = (int)u, iv = (int)v;
    float kui = u - (float)iu, kvi = v - (float)iv;
    float ku = 1.0f - kui, kv = 1.0f - kvi;
    int l = iu % W, r = (iu + 1) % W, b = iv % H, tp = (iv + 1) % H;
    const int id[4] = {b * W + l, b * W + r, tp * W + l, tp * W + r};
    const float w[4] = {ku * kv, kui * kv, ku * kvi, kui * kvi};
    const float sc = 1.0f / 255.0f;
    for (int i = 0; i < 4; ++i)
        out[i] = (float)t->rgba[4 * (size_t)id[0] + i] * w[0] * sc + (float)t->rgba[4 * (size_t)id[1] + i] * w[1] * sc +
                 (float)t->rgba[4 * (size_t)id[2] + i] * w[2] * sc + (float)t->rgba[4 * (size_t)id[3] + i] * w[3] * sc;
}

/* SurfacePoint::getTexCoords -> RenderMesh::getTexCoord (RenderMesh.cpp:146-157):
 * barycentric interpolation of the channel's coordinates; (0, 0) and false
 * when the mesh has no such channel */
static int tex_coords(const oc_scene* s, const oc_sp* sp, int ch, float* tc)
{
    tc[0] = tc[1] = 0.0f;
    const oc_mesh_r* m = &s->meshes[sp->mesh];
    if (ch < 0 || ch > 1 || !m->uv[ch] || sp->face < 0 || sp->face >= m->fn) return 0;
    const uint32_t* fi = m->faces + 3 * (size_t)sp->face;
    const float* uv[3] = {m->uv[ch] + 2 * (size_t)fi[0], m->uv[ch] + 2 * (size_t)fi[1], m->uv[ch] + 2 * (size_t)fi[2]};
    const float* bc = sp->bary;
    tc[0] = uv[0][0] * bc[0] + uv[1][0] * bc[1] + uv[2][0] * bc[2];
    tc[1] = uv[0][1] * bc[0] + uv[1][1] * bc[1] + uv[2][1] * bc[2];
    return 1;
}

static int tex_valid(const oc_scene* s, int id) { return 0 <= id && id < s->n_tex; }

/* multVector3(TM, (u, v, 1)) then BitmapTexture::texture */
static void tex_transformed(const oc_scene* s, const oc_tref* t, const float* uv, float* out)
{
    const float uu = t->m[0][0] * uv[0] + t->m[0][1] * uv[1] + t->m[0][2] * 1.0f;
    const float vv = t->m[1][0] * uv[0] + t->m[1][1] * uv[1] + t->m[1][2] * 1.0f;
    tex_sample(&s->tex[t->tex], uu, vv, out);
}

/* a texture slot as the Helper reads it: sampled only if the map exists and
 * the mesh has the slot's coordinate set */
static int tex_slot(const oc_scene* s, const oc_mat* m, int slot, const oc_sp* sp, float* out)
{
    const oc_tref* t = &m->tref[slot];
    float uv[2];
    if (!tex_valid(s, t->tex) || !tex_coords(s, sp, t->ch, uv)) return 0;
    tex_transformed(s, t, uv, out);
    return 1;
}

/* Helper::getTextureOccMetRoughValues (PhysicallyBasedMaterial.cpp:54-90) */
static void pbr_omr(const oc_scene* s, const oc_mat* m, const oc_sp* sp, float* omr)
{
    omr[0] = 1.0f;
    omr[1] = m->metal;
    omr[2] = m->rough;
    float tb[4];
    if (tex_slot(s, m, TEX_METROUGH, sp, tb)) {
        omr[0] *= tb[0];
        omr[1] *= tb[2];
        omr[2] *= tb[1];
    }
    if (m->tref[TEX_OCCLUSION].tex != m->tref[TEX_METROUGH].tex && tex_slot(s, m, TEX_OCCLUSION, sp, tb))
        omr[0] = tb[0];
}

/* PhysicallyBasedMaterial::modifyFrame (:147-167) */
static void pbr_modify_frame(const oc_scene* s, const oc_mat* m, oc_sp* sp)
{
    float tn[4] = {0.0f, 0.0f, 1.0f, 0.0f};
    if (tex_slot(s, m, TEX_NORMAL, sp, tn)) {
        if (tn[2] <= 0.5f) tn[2] = 0.5f + OC_EPS;
        for (int i = 0; i < 3; ++i) tn[i] = oc_linf(2.0f, -1.0f, tn[i]);
        for (int i = 0; i < 2; ++i) tn[i] = m->normal_scale * tn[i];
        oc_normalize3(tn);
    }
    apply_texture_normal(sp, tn);
}

/* modifyFrame of each material type (OpenMaterial.cpp:66-70, DiffuseColorMaterial.cpp:35-39) */
static void modify_frame(const oc_scene* s, const oc_mat* m, oc_sp* sp)
{
    static const float tn[3] = {0.0f, 0.0f, 1.0f};
    if (m->type == MAT_PBR)
        pbr_modify_frame(s, m, sp);
    else
        apply_texture_normal(sp, tn);
}

/* PhysicallyBasedMaterial::getEmissivity + Helper::getTextureEmissivity
 * (:96-117, :293-299) at the emissive channel's coordinates */
static void pbr_emission(const oc_scene* s, const oc_mat* m, const oc_sp* sp, float* erad)
{
    float euv[2];
    tex_coords(s, sp, m->tref[TEX_EMISSIVE].ch, euv);
    if (!(oc_length3(m->emissive) > OC_EPS)) return;
    if (!tex_valid(s, m->tref[TEX_EMISSIVE].tex)) return;
    float tb[4];
    tex_transformed(s, &m->tref[TEX_EMISSIVE], euv, tb);
    for (int i = 0; i < 3; ++i) erad[i] = tb[i] * m->emissive[i];
}

/* ------------------------------------------------------------- BRDF --- */

/* ndf::GGX::pdf / lambda, SmithG::G1 / G2 (BRDFModel.h:40-80) */
static float ggx_pdf(float cos, float alpha)
{
    float cos2 = cos * cos;
    float alpha2 = alpha * alpha;
    return alpha2 / (OC_PI * powf(oc_lerp(1.0f, alpha2, cos2), 2.0f));
}
static float ggx_lambda(float a) { return 0.5f * (sqrtf(1.0f + powf(a, -2.0f)) - 1.0f); }
static float smith_g1(float cos, float alpha)
{
    float a = cos / (alpha * sqrtf(1.0f - cos * cos));
    return (alpha > 0.0f || cos < 0.99f) ? 1.0f / (1.0f + ggx_lambda(a)) : 1.0f;
}
static float smith_g2(float shadow, float mask)
{
    float p = shadow * mask;
    return p / (shadow + mask - p);
}

typedef struct bsdf_data {
    float I[3], O[3], N[3], H[3], T[3];
    float color[4];
    int transmissive;
    float metal, rough, alpha, eta;
} bsdf_data;

static void bsdf_defaults(bsdf_data* d)
{
    memset(d, 0, sizeof(*d));
    d->color[0] = d->color[1] = d->color[2] = d->color[3] = 1.0f;
    d->metal = 0.5f;
    d->alpha = 0.25f;
    d->eta = 1.0f;
}

/* BSDFModel::evaluate (BRDFModel.h:139-207); mode 0 diffuse, 1 specular, 2 transmitted */
static void bsdf_evaluate(const float* vIn, const float* vOut, const float* norm, const float* color, float metal,
                          float alpha, float* brdf, int specular, int transmitted, const float* Hext, float p)
{
    float VdotN, LdotN, NdotH, VdotH, LdotH;
    {
        float H[3];
        if (!transmitted) {
            H[0] = vOut[0] - vIn[0]; H[1] = vOut[1] - vIn[1]; H[2] = vOut[2] - vIn[2];
            oc_normalize3(H);
        } else {
            H[0] = Hext[0]; H[1] = Hext[1]; H[2] = Hext[2];
        }
        VdotN = oc_clamp(fabsf(oc_dot3(vIn, norm)), 0.0001f, 1.0f);
        LdotN = oc_clamp(fabsf(oc_dot3(vOut, norm)), 0.0001f, 1.0f);
        NdotH = fabsf(oc_dot3(norm, H));
        VdotH = fabsf(oc_dot3(vIn, H));
        LdotH = fabsf(oc_dot3(vOut, H));
    }
    float cDiff[3], F0[3], F[3], fDiff[3], fSpec[3];
    for (int i = 0; i < 3; ++i) cDiff[i] = (1.0f - metal) * color[i];
    for (int i = 0; i < 3; ++i) F0[i] = oc_lerp(0.04f, color[i], metal);
    float P = powf(oc_clamp01(1.0f - VdotH), 5.0f);
    for (int i = 0; i < 3; ++i) F[i] = oc_lerp(P, 1.0f, F0[i]);
    for (int i = 0; i < 3; ++i) fDiff[i] = (1.0f - F[i]) * cDiff[i] / OC_PI;
    {
        float G = smith_g2(smith_g1(VdotN, alpha), smith_g1(LdotN, alpha));
        for (int i = 0; i < 3; ++i)
            fSpec[i] = oc_clamp(0.25f * (transmitted ? 1.0f - F[i] : F[i]) * G / (VdotN * LdotN), 0.0f, FLT_MAX);
    }
    if (specular) {
        float k = 4.0f * LdotH * VdotN / NdotH / LdotN / (1.0f - p);
        for (int i = 0; i < 3; ++i) brdf[i] = k * fSpec[i];
    } else if (transmitted) {
        float k = 4.0f * LdotH * VdotN / NdotH / LdotN / p;
        for (int i = 0; i < 3; ++i) brdf[i] = k * fSpec[i];
    } else {
        float k = OC_PI / LdotN / p;
        for (int i = 0; i < 3; ++i) brdf[i] = k * fDiff[i];
    }
}

/* BSDFModel::evaluateDirect (BRDFModel.h:211-261) */
static void bsdf_eval_direct(const bsdf_data* d, float* brdf)
{
    float VdotN = -oc_dot3(d->I, d->N);
    float LdotN = oc_dot3(d->O, d->N);
    float H[3] = {d->O[0] - d->I[0], d->O[1] - d->I[1], d->O[2] - d->I[2]};
    oc_normalize3(H);
    float VdotH = fabsf(oc_dot3(d->I, H));
    float NdotH = fabsf(oc_dot3(d->N, H));
    float F0[3], F[3], cDiff[3], fDiff[3], fSpec[3];
    for (int i = 0; i < 3; ++i) F0[i] = oc_lerp(0.04f, d->color[i], d->metal);
    float P = powf(oc_clamp01(1.0f - VdotH), 5.0f);
    for (int i = 0; i < 3; ++i) F[i] = oc_lerp(P, 1.0f, F0[i]);
    for (int i = 0; i < 3; ++i) cDiff[i] = (1.0f - d->metal) * d->color[i];
    if (VdotN > 0.0f && LdotN > 0.0f) {
        for (int i = 0; i < 3; ++i) fDiff[i] = (1.0f - F[i]) * cDiff[i] / OC_PI;
    } else {
        fDiff[0] = fDiff[1] = fDiff[2] = 0.0f;
    }
    if (VdotN > 0.0f && LdotN > 0.0f) {
        float D = ggx_pdf(oc_clamp01(NdotH), d->alpha);
        float G = smith_g2(smith_g1(VdotN, d->alpha), smith_g1(LdotN, d->alpha));
        for (int i = 0; i < 3; ++i) fSpec[i] = oc_clamp(0.25f * F[i] * D * G / (VdotN * LdotN), 0.0f, FLT_MAX);
    } else {
        fSpec[0] = fSpec[1] = fSpec[2] = 0.0f;
    }
    for (int i = 0; i < 3; ++i) brdf[i] = fDiff[i] + fSpec[i];
}

/* RandomSampler::GGXHemisphere / cosineSqrtHemisphere / uniformHemisphere
 * (RandomSampler.h:66-103), with the uniforms supplied */
static void ggx_hemisphere(float* v, float alpha2, float u_phi, float rnd)
{
    float phi = oc_lerp(0.0f, 2.0f * OC_PI, u_phi);
    float cth = sqrtf((1.f - rnd) / (1.f - (1.0f - alpha2) * rnd));
    float sth = sqrtf(oc_max(1.0f - cth * cth, 0.0f));
    v[0] = sth * cosf(phi); v[1] = sth * sinf(phi); v[2] = cth;
}
static void cosine_hemisphere(float* v, float u_phi, float rnd)
{
    float phi = oc_lerp(0.0f, 2.0f * OC_PI, u_phi);
    float sth = sqrtf(rnd);
    v[0] = sth * cosf(phi); v[1] = sth * sinf(phi); v[2] = sqrtf(1.0f - rnd);
}
static void uniform_hemisphere(float* v, float u_phi, float cth)
{
    float phi = oc_lerp(0.0f, 2.0f * OC_PI, u_phi);
    float sth = sqrtf(oc_max(1.0f - cth * cth, 0.0f));
    v[0] = sth * cosf(phi); v[1] = sth * sinf(phi); v[2] = cth;
}

/* draws are pulled lazily, in the reference's order */
typedef struct draw_src {
    oc_mt* mt;           /* when set: draw from the generator */
    const float* fixed;  /* otherwise: consume these in order */
    int used;
} draw_src;

static float draw(draw_src* s)
{
    if (s->mt) {
        s->used++;
        return oc_mt_uniform(s->mt);
    }
    return s->fixed[s->used++];
}

/* BSDFModel::sampleIndirect (BRDFModel.h:265-337) */
static void bsdf_sample_indirect(bsdf_data* d, draw_src* rs, float* brdf)
{
    float VdotN = -oc_dot3(d->I, d->N);
    float binorm[3];
    oc_cross3(d->N, d->T, binorm);
    const float* basis[3] = {d->T, binorm, d->N};
    if (VdotN < 0.0f) {
        if (d->transmissive) {
            const float* t = basis[0];
            basis[0] = basis[1];
            basis[1] = t;
            d->N[0] = -d->N[0]; d->N[1] = -d->N[1]; d->N[2] = -d->N[2];
        } else {
            brdf[0] = brdf[1] = brdf[2] = 0.0f;
            return;
        }
    }
    const float p = 0.8f * fabsf(VdotN) + 0.1f;
    float rd[3];
    float rnd = draw(rs);
    if (rnd < p) {
        if (rnd < p * (1.0f - d->color[3])) {
            if (VdotN < 0.0f) d->eta = 1.0f / d->eta;
            float a = draw(rs);
            float b = draw(rs);
            ggx_hemisphere(rd, powf(d->alpha, 2.0f), a, b);
            oc_to_normal_space(basis[0], basis[1], basis[2], rd, d->H);
            oc_normalize3(d->H);
            if (oc_refract3(d->I, d->H, d->eta, d->O) && oc_dot3(d->N, d->O) < 0.0f) {
                oc_normalize3(d->O);
                bsdf_evaluate(d->I, d->O, d->N, d->color, d->metal, d->alpha, brdf, 0, 1, d->H, p);
            } else {
                brdf[0] = brdf[1] = brdf[2] = 0.0f;
                return;
            }
        } else {
            float a = draw(rs);
            float b = draw(rs);
            cosine_hemisphere(rd, a, b);
            oc_to_normal_space(basis[0], basis[1], basis[2], rd, d->O);
            oc_normalize3(d->O);
            bsdf_evaluate(d->I, d->O, d->N, d->color, d->metal, d->alpha, brdf, 0, 0, d->H, p);
        }
    } else {
        float a = draw(rs);
        float b = draw(rs);
        ggx_hemisphere(rd, powf(d->alpha, 2.0f), a, b);
        oc_to_normal_space(basis[0], basis[1], basis[2], rd, d->H);
        oc_normalize3(d->H);
        oc_reflect3(d->I, d->H, d->O);
        if (oc_dot3(d->N, d->O) > 0.0f) {
            oc_normalize3(d->O);
            bsdf_evaluate(d->I, d->O, d->N, d->color, d->metal, d->alpha, brdf, 1, 0, d->H, p);
        } else {
            brdf[0] = brdf[1] = brdf[2] = 0.0f;
            return;
        }
    }
}

/* OpenMaterial.cpp:20-38 fresnelReflection, complex IOR n + ik */
static void fresnel_reflection(float n, float k, float cosTheta, float* tp, float* ts)
{
    float complex fN = CMPLXF(n, k);
    float complex fN2 = fN * fN;
    cosTheta = fabsf(cosTheta);
    const float c2 = cosTheta * cosTheta;
    const float s2 = 1.0f - c2;
    float complex num_p = fN2 * cosTheta - csqrtf(fN2 - s2);
    float complex den_p = fN2 * cosTheta + csqrtf(fN2 - s2);
    float complex ratio_p = num_p / den_p;
    *tp = crealf(ratio_p * conjf(ratio_p));
    float complex num_s = cosTheta - csqrtf(fN2 - s2);
    float complex den_s = cosTheta + csqrtf(fN2 - s2);
    float complex ratio_s = num_s / den_s;
    *ts = crealf(ratio_s * conjf(ratio_s));
}

static void om_brdf_channels(const float* n, const float* k, float fCos, float* brdf)
{
    for (int c = 0; c < 3; ++c) {
        float tp, ts;
        fresnel_reflection(n[c], k[c], fCos, &tp, &ts);
        brdf[c] = oc_lerp(tp, ts, 0.5f) / fabsf(fCos);
    }
}

/* PhysicallyBasedMaterial: BSDFData from the material factors and textures:
 * getTextureRGBA, getTextureOccMetRoughValues, occluseColor (PhysicallyBasedMaterial.cpp:27-95,
 * 178-200, 261-276) */
static void pbr_data(const oc_scene* s, const oc_mat* m, const oc_sp* sp, bsdf_data* d)
{
    float rgba[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    tex_slot(s, m, TEX_BASE, sp, rgba);
    for (int i = 0; i < 4; ++i) d->color[i] = rgba[i] * m->color[i];
    if (m->alpha_mode != OMV_ALPHA_BLEND) d->color[3] = 1.0f;
    d->transmissive = m->double_sided || d->color[3] < 1.0f;
    float omr[3];
    pbr_omr(s, m, sp, omr);
    for (int i = 0; i < 3; ++i) d->color[i] = oc_lerp(d->color[i], omr[0] * d->color[i], m->occl_strength);
    d->metal = omr[1];
    d->rough = oc_clamp(omr[2], 0.00001f, 0.99999f);
    d->alpha = powf(d->rough, 2.0f);
}

/* RenderMaterial::getBrdf of each material type, impSmpScale = false */
static void material_get_brdf(const oc_scene* s, const oc_mat* m, const float* inV, const oc_sp* sp, const float* outV,
                              float* brdf)
{
    if (m->type == MAT_PBR) { /* PhysicallyBasedMaterial::getBrdf (:178-245) */
        bsdf_data d;
        bsdf_defaults(&d);
        memcpy(d.I, inV, sizeof(d.I));
        memcpy(d.O, outV, sizeof(d.O));
        memcpy(d.N, sp->nrm, sizeof(d.N));
        pbr_data(s, m, sp, &d);
        if (oc_dot3(inV, sp->nrm) > 0.0f && d.transmissive) {
            d.N[0] = -d.N[0]; d.N[1] = -d.N[1]; d.N[2] = -d.N[2];
        }
        bsdf_eval_direct(&d, brdf);
    } else if (m->type == MAT_OM) { /* OpenMaterial::getBrdf (OpenMaterial.cpp:95-163) */
        if (!m->has_ior) {
            brdf[0] = brdf[1] = brdf[2] = 0.0f;
            return;
        }
        float fCos = -oc_dot3(inV, sp->nrm);
        if (fabsf(oc_dot3(outV, sp->nrm) - fCos) > 1e-6f) {
            brdf[0] = brdf[1] = brdf[2] = 0.0f;
            return;
        }
        om_brdf_channels(m->om_n, m->om_k, fCos, brdf);
    } else { /* DiffuseColorMaterial::getBrdf (DiffuseColorMaterial.cpp:49-108) */
        const float pdf = 1.0f / OC_PI;
        const float brdfPdf = 1.0f / (pdf * OC_PI);
        for (int i = 0; i < 3; ++i) brdf[i] = brdfPdf * m->color[i];
    }
    (void)s;
}

/* RenderMaterial::getRayAndBrdf of each material type */
static void material_ray_and_brdf(const oc_scene* s, const oc_mat* m, const float* inV, const oc_sp* sp, float* outV,
                                  float* brdf, float* erad, int inv, draw_src* rs)
{
    erad[0] = erad[1] = erad[2] = 0.0f;
    if (m->type == MAT_PBR) { /* PhysicallyBasedMaterial::getRayAndBrdf (:248-291) */
        bsdf_data d;
        bsdf_defaults(&d);
        memcpy(d.I, inV, sizeof(d.I));
        memcpy(d.N, sp->nrm, sizeof(d.N));
        memcpy(d.T, sp->tan, sizeof(d.T));
        pbr_data(s, m, sp, &d);
        d.eta = 1.0f / (m->double_sided ? 1.0f : m->ior);
        bsdf_sample_indirect(&d, rs, brdf);
        memcpy(outV, d.O, sizeof(d.O));
        pbr_emission(s, m, sp, erad);
    } else if (m->type == MAT_OM) { /* OpenMaterial::defineNextDirection + getRayAndBrdf (:72-93, :165-232) */
        oc_reflect3(inV, sp->nrm, outV);
        float tfn[3];
        face_normal(s, sp, tfn);
        float correction;
        if ((correction = oc_dot3(outV, tfn)) < 0.1f) {
            for (int i = 0; i < 3; ++i) outV[i] = oc_linf(tfn[i], outV[i], 0.1f - correction);
            oc_normalize3(outV);
        }
        if (!m->has_ior) {
            brdf[0] = brdf[1] = brdf[2] = 0.0f;
            return;
        }
        float fCos = oc_dot3(outV, sp->nrm);
        om_brdf_channels(m->om_n, m->om_k, fCos, brdf);
    } else { /* RenderMaterial::getRayAndBrdf + DiffuseColorMaterial::defineNextDirection */
        float v[3];
        float a = draw(rs);
        float b = draw(rs);
        uniform_hemisphere(v, a, b);
        oc_to_normal_space(sp->tan, sp->bin, sp->nrm, v, outV);
        if (!inv) {
            material_get_brdf(s, m, inV, sp, outV, brdf);
        } else {
            float ii[3] = {-outV[0], -outV[1], -outV[2]};
            float oo[3] = {-inV[0], -inV[1], -inV[2]};
            material_get_brdf(s, m, ii, sp, oo, brdf);
        }
    }
}

/* PhysicallyBasedMaterial::isMasked (:301-316): the base colour texture's
 * alpha at the untransformed coordinates (BitmapTexture::texture(sp, ...),
 * BitmapTexture.cpp:142-156: 1 where the mesh lacks the coordinate set) */
static int material_masked(const oc_scene* s, const oc_mat* m, const oc_sp* sp)
{
    if (m->type != MAT_PBR || m->alpha_mode != OMV_ALPHA_MASK) return 0;
    float alpha = m->color[3];
    if (alpha < m->cutoff) return 1;
    if (tex_valid(s, m->tref[TEX_BASE].tex)) {
        float tc[4] = {0.5f, 0.5f, 0.5f, 1.0f}, uv[2];
        if (tex_coords(s, sp, m->tref[TEX_BASE].ch, uv)) tex_sample(&s->tex[m->tref[TEX_BASE].tex], uv[0], uv[1], tc);
        alpha *= tc[3];
    }
    return alpha < m->cutoff;
}

/* ---------------------------------------------------------- renderer --- */

typedef struct part {
    float out_ray[3];
    oc_sp sp;
    float out_rad[3];
    float out_factor[3];
} part;

typedef struct ctx {
    const oc_scene* s;
    const omv_params* p;
    uint64_t rays;
} ctx;

static int scene_query(ctx* c, oc_rh* h)
{
    oc_ray r;
    memcpy(r.org, h->org, sizeof(r.org));
    memcpy(r.dir, h->dir, sizeof(r.dir));
    r.tnear = h->tnear;
    r.tfar = h->tfar;
    oc_hitrec hr;
    c->rays++;
    if (!oc_intersect(&c->s->accel, &r, &hr)) return 0;
    h->tfar = hr.t;
    h->u = hr.u;
    h->v = hr.v;
    h->prim = hr.prim;
    h->geom = hr.geom;
    h->inst = hr.inst;
    return 1;
}

/* BDPTRenderer::sceneIntersect (BDPTRenderer.cpp:75-102) */
static int scene_intersect(ctx* c, oc_rh* h, oc_sp* sp)
{
    float t1 = h->tfar;
    int itr = 10;
    while (itr > 0) {
        scene_query(c, h);
        if (h->geom == OC_INVALID) return 0;
        compute_surface_point(c->s, h, sp);
        const oc_mat* m = &c->s->mats[c->s->meshes[sp->mesh].mat];
        if (!material_masked(c->s, m, sp)) return 1;
        float org[3] = {h->org[0] + h->tfar * h->dir[0], h->org[1] + h->tfar * h->dir[1], h->org[2] + h->tfar * h->dir[2]};
        float v = oc_max_abs(org, 1.0f);
        v = v > h->tfar ? v : h->tfar;
        float delta = OC_EPS_ACC * OC_EPS * v;
        h->tnear = h->tfar + delta;
        h->tfar = t1;
        if (h->tfar <= h->tnear) return 0;
        --itr;
    }
    return 0;
}

/* BDPTRenderer::setRay + shiftRayAlongDirection (BDPTRenderer.cpp:42-50, 309-321) */
static void set_ray(const float* O, const float* R, oc_rh* h, float epsShift)
{
    memcpy(h->org, O, sizeof(h->org));
    memcpy(h->dir, R, sizeof(h->dir));
    float v = oc_max_abs(h->org, 1.0f);
    float delta = (OC_EPS_ACC * epsShift) * OC_EPS * v;
    h->org[0] += delta * h->dir[0];
    h->org[1] += delta * h->dir[1];
    h->org[2] += delta * h->dir[2];
    h->inst = OC_INVALID;
    h->geom = OC_INVALID;
    h->tfar = FLT_MAX;
}

/* BDPTRenderer::computeLightAttenuation (BDPTRenderer.cpp:104-126) */
static float light_attenuation(const omv_params* p, float d, float attD)
{
    if (attD >= FLT_MAX) {
        d = d < p->light_min_distance ? p->light_min_distance : d;
        switch (p->light_distance_attenuation) {
            case 1: return 1.0f / d;
            case 2: return 1.0f / (d * d);
            default: return 1.0f;
        }
    }
    float rD = oc_max(1.0f - d / attD, 0.0f);
    switch (p->light_distance_attenuation) {
        case 1: return rD;
        case 2: return sqrtf(rD);
        default: return d < attD ? 1.0f : 0.0f;
    }
}

/* BDPTRenderer::computePath (BDPTRenderer.cpp:128-192) */
static int compute_path(ctx* c, part* P, int max_n, const float* O, const float* R, float* Rad, int* n, int inv,
                        float attD, draw_src* rs)
{
    oc_rh h;
    memset(&h, 0, sizeof(h));
    h.tnear = 0.0f;
    P[0].sp.inst = -1;
    memcpy(P[0].sp.pos, O, sizeof(float[3]));
    memcpy(P[0].out_ray, R, sizeof(float[3]));
    memcpy(P[0].out_rad, Rad, sizeof(float[3]));
    P[0].out_factor[0] = P[0].out_factor[1] = P[0].out_factor[2] = 1.0f;
    float rDterm = 1.0f;
    float brdf[3], erad[3];
    *n = 1;
    int exit_ = 0;
    for (int i = 1; i < max_n; ++i) {
        set_ray(P[i - 1].sp.pos, P[i - 1].out_ray, &h, 1.0f);
        if (!scene_intersect(c, &h, &P[i].sp)) {
            exit_ = 1;
            break;
        }
        const oc_mat* m = &c->s->mats[c->s->meshes[P[i].sp.mesh].mat];
        modify_frame(c->s, m, &P[i].sp);
        material_ray_and_brdf(c->s, m, P[i - 1].out_ray, &P[i].sp, P[i].out_ray, brdf, erad, inv, rs);
        float ct = fabsf(inv ? oc_dot3(P[i].out_ray, P[i].sp.nrm) : oc_dot3(P[i - 1].out_ray, P[i].sp.nrm));
        for (int k = 0; k < 3; ++k) P[i].out_factor[k] = P[i - 1].out_factor[k] * brdf[k] * ct;
        if (inv) {
            for (int k = 0; k < 3; ++k) Rad[k] += P[i].out_factor[k] * erad[k];
            P[i].out_rad[0] = P[i].out_rad[1] = P[i].out_rad[2] = 0.0f;
        } else {
            if (i == 1) rDterm = light_attenuation(c->p, oc_distance3(P[i].sp.pos, P[i - 1].sp.pos), attD);
            for (int k = 0; k < 3; ++k) P[i].out_rad[k] = P[i].out_factor[k] * Rad[k] * rDterm;
            float curInt = oc_intensity(P[i].out_rad);
            if (curInt < c->p->ray_cut_value) break;
        }
        (*n)++;
    }
    return exit_;
}

/* BDPTRenderer::isConnected (BDPTRenderer.cpp:208-235) */
static int is_connected(ctx* c, const float* A, const float* B)
{
    float dir[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
    float len = oc_length3(dir);
    float maxsz = oc_max_abs(A, 1.0f);
    float safeD = 2.0f * OC_EPS_ACC * OC_EPS * maxsz;
    if (len <= safeD) return 1;
    dir[0] /= len; dir[1] /= len; dir[2] /= len;
    oc_rh h;
    memset(&h, 0, sizeof(h));
    h.tnear = safeD;
    set_ray(A, dir, &h, 0.0f);
    h.tfar = len + (0.1f * len > safeD ? 0.1f * len : safeD);
    oc_sp sp;
    memset(&sp, 0, sizeof(sp));
    if (!scene_intersect(c, &h, &sp)) return 1;
    float sd = oc_sqdistance3(sp.pos, B);
    maxsz = oc_max_abs(B, 1.0f);
    safeD = 10.0f * OC_EPS * maxsz;
    if (sd <= safeD * safeD) return 1;
    return 0;
}

/* HDRBackground::getRadiance (HdrBackground.cpp:55-97) */
static void background_radiance(const oc_scene* s, const float* dir, float* val)
{
    float rdir[3];
    oc_vec_mat3(dir, (const float(*)[3])s->bg_R, rdir);
    float r_xy[3] = {rdir[0], rdir[1], 0.0f};
    oc_normalize3(r_xy);
    float xang = acosf(oc_clamp(r_xy[0], -1.0f, 1.0f));
    xang = r_xy[1] < 0.0f ? 2.0f * OC_PI - xang : xang;
    float yang = asinf(oc_clamp(rdir[2], -1.0f, 1.0f));
    yang += 0.5f * OC_PI;
    float u = xang / (2.0f * OC_PI);
    float v = 1.0f - yang / OC_PI;
    const int W = s->bg_w, H = s->bg_h;
    float upage = floorf(u - 0.5f / (float)W);
    float vpage = floorf(v - 0.5f / (float)H);
    u -= upage;
    v -= vpage;
    u *= (float)W;
    v *= (float)H;
    int iu = (int)u;
    int iv = (int)v;
    float kui = u - (float)iu;
    float kvi = v - (float)iv;
    float ku = 1.0f - kui;
    float kv = 1.0f - kvi;
    int l = iu % W, r = (iu + 1) % W, b = iv % H, t = (iv + 1) % H;
    int id[4] = {b * W + l, b * W + r, t * W + l, t * W + r};
    float w[4] = {ku * kv, kui * kv, ku * kvi, kui * kvi};
    for (int i = 0; i < 3; ++i)
        val[i] = s->bg[3 * (size_t)id[0] + i] * w[0] + s->bg[3 * (size_t)id[1] + i] * w[1] +
                 s->bg[3 * (size_t)id[2] + i] * w[2] + s->bg[3 * (size_t)id[3] + i] * w[3];
    val[0] *= s->bg_scale;
    val[1] *= s->bg_scale;
    val[2] *= s->bg_scale;
}

/* PinholeCamera::getRay (PinholeCamera.cpp:80-95) with the two jitter uniforms */
static void camera_ray(const omv_camera* cam, int x, int y, float ux, float uy, float* O, float* R)
{
    float px = (float)x + 0.5f - cam->half_width;
    float py = (float)y + 0.5f - cam->half_height;
    float dx = oc_lerp(-0.5f, 0.5f, ux);
    float dy = oc_lerp(-0.5f, 0.5f, uy);
    float cray[3] = {px + dx, py + dy, cam->focus};
    oc_normalize3(cray);
    oc_mat3_vec(cam->rotation, cray, R);
    memcpy(O, cam->position, sizeof(float[3]));
}

/* DistanceRandom::getValue (DistanceRandom.h:98-115) */
static int light_pick(const oc_scene* s, float rnd)
{
    const float d = rnd * s->lmax;
    const int N = s->n_light;
    if (N <= 0) return -1;
    if (N == 1) return 0;
    if (d <= s->lcdf[0]) return 0;
    if (d >= s->lcdf[N - 2]) return N - 1;
    int L = 0, R = N - 1;
    while (L < R) {
        int C = (L + R) / 2;
        if (d <= s->lcdf[C])
            R = C;
        else
            L = C + 1;
    }
    return (L + R) / 2;
}

/* BDPTRenderer::computePaths (BDPTRenderer.cpp:237-302) */
static void compute_paths(ctx* c, const float* O, const float* R, float* radiance, part* CP, part* LP, draw_src* rs)
{
    const omv_params* p = c->p;
    const oc_scene* s = c->s;
    int light = -1;
    int lp_len = 0;
    if (s->n_light > 0) { /* tryComputeLightPath (:194-206) */
        light = light_pick(s, draw(rs));
        if (light >= 0) {
            float Rl[3], sl; /* RenderLightPoint::getRandomRay -> RandomSampler::uniformSphere */
            do {
                Rl[0] = draw(rs);
                Rl[1] = draw(rs);
                Rl[2] = draw(rs);
                sl = oc_dot3(Rl, Rl);
            } while (sl > 1.0f || sl < OC_EPS);
            float k = 1.0f / sqrtf(sl);
            for (int i = 0; i < 3; ++i) Rl[i] = k * Rl[i];
            float rad[3] = {s->lint[light][0] * p->light_scale, s->lint[light][1] * p->light_scale,
                            s->lint[light][2] * p->light_scale};
            compute_path(c, LP, p->light_bounces + 1, s->lpos[light], Rl, rad, &lp_len, 0, s->lrange[light], rs);
        }
    }
    int cp_len = 0;
    radiance[0] = radiance[1] = radiance[2] = 0.0f;
    int cp_exit = compute_path(c, CP, p->camera_bounces + 1, O, R, radiance, &cp_len, 1, FLT_MAX, rs);
    int totalPN = 0;
    if (cp_exit && s->has_bg && cp_len <= p->max_path_length) {
        float bg[3];
        background_radiance(s, CP[cp_len - 1].out_ray, bg);
        const float* kf = CP[cp_len - 1].out_factor;
        bg[0] *= kf[0]; bg[1] *= kf[1]; bg[2] *= kf[2];
        for (int k = 0; k < 3; ++k) radiance[k] = bg[k] * 1.0f + radiance[k];
        ++totalPN;
    } else if (oc_intensity(radiance) > OC_EPS) {
        ++totalPN;
    }
    if (light >= 0) {
        float LC[3], lRad[3], lcRad[3], brdf[3], outV[3];
        for (int i = 0; i < lp_len; ++i) {
            memcpy(lRad, LP[i].out_rad, sizeof(lRad));
            const float* lPos = LP[i].sp.pos;
            for (int j = 1; j < cp_len && i + j <= p->max_path_length; ++j) {
                const float* cPos = CP[j].sp.pos;
                LC[0] = cPos[0] - lPos[0]; LC[1] = cPos[1] - lPos[1]; LC[2] = cPos[2] - lPos[2];
                oc_normalize3(LC);
                if (i == 0) { /* getRadianceAlongRay + attenuation (:275-282) */
                    memcpy(lRad, s->lint[light], sizeof(lRad));
                    float lsc = light_attenuation(p, oc_distance3(cPos, lPos), s->lrange[light]);
                    lRad[0] *= p->light_scale * lsc;
                    lRad[1] *= p->light_scale * lsc;
                    lRad[2] *= p->light_scale * lsc;
                }
                float cc = fabsf(oc_dot3(LC, CP[j].sp.nrm));
                for (int k = 0; k < 3; ++k) lcRad[k] = lRad[k] * cc * CP[j - 1].out_factor[k];
                if (oc_intensity(lcRad) < p->ray_cut_value) continue;
                const oc_mat* m = &s->mats[s->meshes[CP[j].sp.mesh].mat];
                outV[0] = -CP[j - 1].out_ray[0]; outV[1] = -CP[j - 1].out_ray[1]; outV[2] = -CP[j - 1].out_ray[2];
                material_get_brdf(s, m, LC, &CP[j].sp, outV, brdf);
                brdf[0] *= cc; brdf[1] *= cc; brdf[2] *= cc;
                for (int k = 0; k < 3; ++k) lcRad[k] = brdf[k] * CP[j - 1].out_factor[k] * lRad[k];
                if (oc_intensity(lcRad) < p->ray_cut_value) continue;
                if (!is_connected(c, lPos, cPos)) continue;
                for (int k = 0; k < 3; ++k) radiance[k] = lcRad[k] * 1.0f + radiance[k];
            }
        }
    }
    float scale = totalPN ? 1.0f / (float)totalPN : 1.0f;
    for (int i = 0; i < 3; ++i) radiance[i] *= scale;
}

typedef struct job {
    const oc_scene* s;
    const omv_camera* cam;
    const omv_params* p;
    int mode;
    uint32_t seed;
    int row_end;
    atomic_int next_row;
    float* film;
    double* sumsq;
    atomic_ullong rays;
} job;

static uint32_t row_seed(uint32_t seed, int row)
{
    uint32_t h = seed ^ (0x9E3779B9u * (uint32_t)(row + 1));
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

static void render_rows(job* j, oc_mt* shared)
{
    ctx c = {j->s, j->p, 0};
    part* CP = (part*)calloc((size_t)j->p->camera_bounces + 1, sizeof(part));
    part* LP = (part*)calloc((size_t)j->p->light_bounces + 1, sizeof(part));
    oc_mt own;
    const int W = j->cam->width;
    int row;
    while ((row = atomic_fetch_add(&j->next_row, 1)) < j->row_end) {
        oc_mt* mt = shared;
        if (!mt) {
            oc_mt_seed(&own, row_seed(j->seed, row));
            mt = &own;
        }
        draw_src rs = {mt, NULL, 0};
        for (int x = 0; x < W; ++x) {
            for (int k = 0; k < j->p->samples_per_pixel; ++k) {
                float ux = draw(&rs);
                float uy = draw(&rs);
                float O[3], R[3], rad[3];
                camera_ray(j->cam, x, row, ux, uy, O, R);
                compute_paths(&c, O, R, rad, CP, LP, &rs);
                float* px = j->film + 4 * ((size_t)row * W + x); /* PinholeCamera::hit */
                px[0] = px[0] + rad[0];
                px[1] = px[1] + rad[1];
                px[2] = px[2] + rad[2];
                px[3] += 1.0f;
                if (j->sumsq) {
                    double* q = j->sumsq + 3 * ((size_t)row * W + x);
                    q[0] += (double)rad[0] * rad[0];
                    q[1] += (double)rad[1] * rad[1];
                    q[2] += (double)rad[2] * rad[2];
                }
            }
        }
    }
    atomic_fetch_add(&j->rays, c.rays);
    free(CP);
    free(LP);
}

static void* worker(void* arg)
{
    render_rows((job*)arg, NULL);
    return NULL;
}

int32_t oc_render(const oc_scene* s, const omv_camera* cam, const omv_params* p, int32_t mode, uint32_t seed,
                  int32_t threads, int32_t row_begin, int32_t row_end, float* film, double* sumsq, uint64_t* rays_out)
{
    if (!s || !cam || !p || !film) return -1;
    if (row_end > cam->height) row_end = cam->height;
    job j;
    j.s = s;
    j.cam = cam;
    j.p = p;
    j.mode = mode;
    j.seed = seed;
    j.row_end = row_end;
    atomic_init(&j.next_row, row_begin);
    j.film = film;
    j.sumsq = sumsq;
    atomic_init(&j.rays, 0ULL);
    if (mode == 0) {
        oc_mt mt;
        oc_mt_seed(&mt, seed);
        render_rows(&j, &mt);
    } else {
        if (threads < 1) threads = 1;
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
        for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, worker, &j);
        for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
        free(th);
    }
    if (rays_out) *rays_out = atomic_load(&j.rays);
    return 0;
}

void oc_film_stop(float* film, int64_t pixels)
{
    for (int64_t i = 0; i < pixels; ++i) {
        float* px = film + 4 * i;
        float scale = px[3] < 0.5f ? 1.0f : 1.0f / px[3];
        px[0] = scale * px[0];
        px[1] = scale * px[1];
        px[2] = scale * px[2];
        px[3] = 1.0f;
    }
}

static void fill_hit(const oc_scene* s, const oc_rh* h, int hit, omv_hit* out)
{
    if (!hit) {
        out->inst = out->geom = out->prim = out->material = OC_INVALID;
        out->t = out->u = out->v = 0.0f;
        out->pad = 0;
        return;
    }
    out->inst = h->inst;
    out->geom = h->geom;
    out->prim = h->prim;
    out->material = (uint32_t)s->meshes[h->geom].mat;
    out->t = h->tfar;
    out->u = h->u;
    out->v = h->v;
    out->pad = 0;
}

int32_t oc_render_ids(const oc_scene* s, const omv_camera* cam, uint32_t seed, float* rays, omv_hit* hits)
{
    oc_mt mt;
    oc_mt_seed(&mt, seed);
    draw_src rs = {&mt, NULL, 0};
    omv_params p;
    omv_params_default(&p);
    ctx c = {s, &p, 0};
    for (int y = 0; y < cam->height; ++y) {
        for (int x = 0; x < cam->width; ++x) {
            float ux = draw(&rs), uy = draw(&rs);
            float O[3], R[3];
            camera_ray(cam, x, y, ux, uy, O, R);
            size_t id = (size_t)y * cam->width + x;
            memcpy(rays + 6 * id, O, sizeof(O));
            memcpy(rays + 6 * id + 3, R, sizeof(R));
            oc_rh h;
            memset(&h, 0, sizeof(h));
            set_ray(O, R, &h, 1.0f);
            oc_sp sp;
            int hit = scene_intersect(&c, &h, &sp);
            fill_hit(s, &h, hit, &hits[id]);
            /* the false-colour getRayAndBrdf of the missing material still
             * draws a uniform-hemisphere direction (RenderMaterial.cpp:51-58) */
            if (hit && s->mats[s->meshes[sp.mesh].mat].type == MAT_MISSING) {
                draw(&rs);
                draw(&rs);
            }
        }
    }
    return 0;
}

int32_t oc_trace_rays(const oc_scene* s, int64_t n, const float* rays, omv_hit* hits)
{
    omv_params p;
    omv_params_default(&p);
    ctx c = {s, &p, 0};
    for (int64_t i = 0; i < n; ++i) {
        const float* r = rays + 8 * i;
        oc_rh h;
        memset(&h, 0, sizeof(h));
        h.org[0] = r[0]; h.org[1] = r[1]; h.org[2] = r[2];
        h.tnear = r[3];
        h.dir[0] = r[4]; h.dir[1] = r[5]; h.dir[2] = r[6];
        h.tfar = r[7];
        h.geom = h.inst = OC_INVALID;
        oc_sp sp;
        int hit = scene_intersect(&c, &h, &sp);
        fill_hit(s, &h, hit, &hits[i]);
    }
    return 0;
}

void oc_brdf_eval_direct(int64_t n, const float* in, float* out)
{
    for (int64_t i = 0; i < n; ++i) {
        const float* x = in + 17 * i;
        bsdf_data d;
        bsdf_defaults(&d);
        memcpy(d.I, x, 3 * sizeof(float));
        memcpy(d.O, x + 3, 3 * sizeof(float));
        memcpy(d.N, x + 6, 3 * sizeof(float));
        memcpy(d.color, x + 9, 4 * sizeof(float));
        d.metal = x[13];
        d.alpha = x[14];
        bsdf_eval_direct(&d, out + 3 * i);
    }
}

void oc_brdf_sample_indirect(int64_t n, const float* in, float* out)
{
    for (int64_t i = 0; i < n; ++i) {
        const float* x = in + 24 * i;
        bsdf_data d;
        bsdf_defaults(&d);
        memcpy(d.I, x, 3 * sizeof(float));
        memcpy(d.N, x + 3, 3 * sizeof(float));
        memcpy(d.T, x + 6, 3 * sizeof(float));
        memcpy(d.color, x + 9, 4 * sizeof(float));
        d.metal = x[13];
        d.alpha = x[14];
        d.eta = x[15];
        d.transmissive = x[16] != 0.0f;
        draw_src rs = {NULL, x + 17, 0};
        float brdf[3];
        bsdf_sample_indirect(&d, &rs, brdf);
        memcpy(out + 6 * i, d.O, 3 * sizeof(float));
        memcpy(out + 6 * i + 3, brdf, 3 * sizeof(float));
    }
}

void oc_om_fresnel(int64_t n, const float* in, float* out)
{
    for (int64_t i = 0; i < n; ++i) {
        const float* x = in + 7 * i;
        om_brdf_channels(x, x + 3, x[6], out + 3 * i);
    }
}

void oc_camera_rays(const omv_camera* cam, const float* jitter, float* rays)
{
    for (int y = 0; y < cam->height; ++y)
        for (int x = 0; x < cam->width; ++x) {
            size_t id = (size_t)y * cam->width + x;
            camera_ray(cam, x, y, jitter[2 * id], jitter[2 * id + 1], rays + 6 * id, rays + 6 * id + 3);
        }
}

void oc_env_radiance(const oc_scene* s, int64_t n, const float* dirs, float* rgb)
{
    for (int64_t i = 0; i < n; ++i) {
        if (!s->has_bg) {
            rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = 0.0f;
            continue;
        }
        background_radiance(s, dirs + 3 * i, rgb + 3 * i);
    }
}

void oc_mt_uniforms(uint32_t seed, int64_t n, float* out)
{
    oc_mt mt;
    oc_mt_seed(&mt, seed);
    for (int64_t i = 0; i < n; ++i) out[i] = oc_mt_uniform(&mt);
}

/* RendererParameters defaults (RendererParameters.h:56-89); the same function
 * is exported by the product library under the same name */
void omv_params_default(omv_params* p)
{
    memset(p, 0, sizeof(*p));
    p->camera_bounces = 10;
    p->light_bounces = 10;
    p->max_path_length = 8;
    p->samples_per_pixel = 20;
    p->light_distance_attenuation = 1;
    p->light_scale = 100.0f;
    p->light_min_distance = 0.01f;
    p->ray_cut_value = 0.002f;
    p->seed = 0;
    p->estimator = OMV_ESTIMATOR_REFERENCE;
}

/* ----------------------------------------------- false-colour validation --- */

/* RenderMesh::getMinMaxDensity (RenderMesh.cpp:277-297) over every instance,
 * as RenderScene::commitScene collects it (RenderScene.cpp:196-203) */
static void density_range(const oc_scene* s, float* dmin, float* dmax)
{
    float lo = INFINITY, hi = 0.0f;
    for (int i = 0; i < s->n_inst; ++i) {
        const oc_inst_r* in = &s->inst[i];
        if (in->mesh < 0) continue;
        const oc_mesh_r* m = &s->meshes[in->mesh];
        for (int f = 0; f < m->fn; ++f) {
            float V[3][3], N[3];
            for (int k = 0; k < 3; ++k)
                oc_xform_point((const float(*)[4])in->M, m->v + (size_t)m->faces[3 * (size_t)f + k] * 10, V[k]);
            const float E1[3] = {V[1][0] - V[0][0], V[1][1] - V[0][1], V[1][2] - V[0][2]};
            const float E2[3] = {V[2][0] - V[0][0], V[2][1] - V[0][1], V[2][2] - V[0][2]};
            oc_cross3(E1, E2, N);
            const float area = oc_length3(N) / 2.0f;
            if (area > OC_EPS) {
                const float d = 1.0f / (0.0f + area);
                lo = oc_min(lo, d);
                hi = oc_max(hi, d);
            }
        }
    }
    *dmin = lo;
    *dmax = hi;
}

/* the FC_VALIDATION tail of RenderMesh::computeSurfacePoint (RenderMesh.cpp:
 * 197-207, pointwise surface gradient) and of BDPTRenderer::computeSurfacePoint
 * (BDPTRenderer.cpp:68-72): relative mesh density and average gradient */
static void fc_surface_terms(const oc_scene* s, const oc_sp* sp, float dmin, float dmax, float* density,
                             float* gradient)
{
    const oc_inst_r* in = &s->inst[sp->inst];
    const oc_mesh_r* m = &s->meshes[sp->mesh];
    const uint32_t* fi = m->faces + 3 * (size_t)sp->face;
    float V[3][3], tfn[3];
    for (int k = 0; k < 3; ++k) oc_xform_point((const float(*)[4])in->M, m->v + (size_t)fi[k] * 10, V[k]);
    const float E1[3] = {V[1][0] - V[0][0], V[1][1] - V[0][1], V[1][2] - V[0][2]};
    const float E2[3] = {V[2][0] - V[0][0], V[2][1] - V[0][1], V[2][2] - V[0][2]};
    oc_cross3(E1, E2, tfn);
    float ref = 1.0f / (0.0f + oc_length3(tfn) / 2.0f);
    oc_normalize3(tfn);
    float ag = 0.0f;
    for (int k = 0; k < 3; ++k) {
        float tvn[3];
        oc_mat3_vec((const float(*)[3])in->N, m->v + (size_t)fi[k] * 10 + 3, tvn);
        oc_normalize_if_needed3(tvn);
        ag = ag + sqrtf((1.0f - oc_clamp(oc_dot3(tvn, tfn), -1.0f, 1.0f)) / 2.0f);
    }
    *gradient = powf(oc_clamp(ag / 3.0f, 1e-6f, 1.0f), 0.286f);
    *density = oc_clamp01(1.0f - logf(dmax / oc_clamp(ref, dmin, dmax)) / logf(dmax / dmin));
}

static float fc_clamped(float v) { return oc_clamp(v, 0.0f, 1.0f); } /* GenericFCArgument ClampedFloat */

static void fc_lerp_paint(float t, const float* lower, const float* upper, float* c)
{
    for (int i = 0; i < 3; ++i) c[i] = oc_lerp(lower[i], upper[i], t);
}

/* The false-colour pass of the FC_VALIDATION build (main.cpp:261-270): spp 1,
 * one bounce, no lights, no background.  Each pixel's jittered primary ray is
 * traced; the hit material's getRayAndBrdf hands the subject's argument to
 * GenericFCSubject::paint (PhysicallyBasedMaterial.cpp:202-240,
 * OpenMaterial.cpp:165-210, DiffuseColorMaterial.cpp:49-89) and the colour
 * becomes the pixel's radiance (BDPTRenderer.cpp:165-168).  Outputs per pixel
 * (each may be NULL): rgba (colour, alpha 1: the film after stop), the 4
 * argument bytes, the uniforms drawn (dx, dy, and the missing material's two
 * hemisphere draws, else 0) and the hit. */
int32_t oc_render_fc(const oc_scene* s, const omv_camera* cam, uint32_t seed, int32_t subject,
                     const uint32_t* palette, int32_t palette_size, float* rgba, uint32_t* args, float* uniforms,
                     omv_hit* hits)
{
    static const float white[3] = {1.0f, 1.0f, 1.0f}, blue[3] = {0.0f, 0.0f, 1.0f}, green[3] = {0.0f, 1.0f, 0.0f},
                       red[3] = {1.0f, 0.0f, 0.0f};
    oc_mt mt;
    oc_mt_seed(&mt, seed);
    draw_src rs = {&mt, NULL, 0};
    omv_params p;
    omv_params_default(&p);
    ctx c = {s, &p, 0};
    float dmin = 0.0f, dmax = 0.0f;
    if (subject == OMV_FC_MD) density_range(s, &dmin, &dmax);
    uint32_t face_base = 0;
    for (int y = 0; y < cam->height; ++y) {
        for (int x = 0; x < cam->width; ++x) {
            const size_t id = (size_t)y * cam->width + x;
            float u[4] = {draw(&rs), draw(&rs), 0.0f, 0.0f};
            float O[3], R[3];
            camera_ray(cam, x, y, u[0], u[1], O, R);
            oc_rh h;
            memset(&h, 0, sizeof(h));
            set_ray(O, R, &h, 1.0f);
            oc_sp sp;
            const int hit = scene_intersect(&c, &h, &sp);
            float col[3] = {0.0f, 0.0f, 0.0f};
            uint32_t arg = 0;
            if (hit) {
                const oc_mat* m = &s->mats[s->meshes[sp.mesh].mat];
                modify_frame(s, m, &sp);
                float inV[3] = {R[0], R[1], R[2]};
                if (m->type == MAT_MISSING) { /* RenderMaterial::getRayAndBrdf: hemisphere, then getBrdf(-out, -in) */
                    float v[3], outV[3];
                    u[2] = draw(&rs);
                    u[3] = draw(&rs);
                    uniform_hemisphere(v, u[2], u[3]);
                    oc_to_normal_space(sp.tan, sp.bin, sp.nrm, v, outV);
                    inV[0] = -outV[0];
                    inV[1] = -outV[1];
                    inV[2] = -outV[2];
                }
                float f = 0.0f;
                face_base = 0;
                for (int k = 0; k < sp.mesh; ++k) face_base += (uint32_t)s->meshes[k].fn;
                switch (subject) {
                case OMV_FC_PID:
                case OMV_FC_GID: {
                    arg = subject == OMV_FC_PID ? face_base + (uint32_t)sp.face : (uint32_t)sp.mesh;
                    const uint32_t n = (palette && arg < (uint32_t)palette_size) ? palette[arg] : 0u;
                    col[0] = (float)((n >> 16) & 0xFFu) / 255.0f;
                    col[1] = (float)((n >> 8) & 0xFFu) / 255.0f;
                    col[2] = (float)(n & 0xFFu) / 255.0f;
                    break;
                }
                case OMV_FC_MID:
                    if (m->type == MAT_MISSING) {
                        arg = 0xFFFFFFFFu;
                        col[0] = 1000.0f;
                        col[2] = 1000.0f;
                    } else {
                        arg = (uint32_t)s->meshes[sp.mesh].mat;
                        const uint32_t n = (palette && arg < (uint32_t)palette_size) ? palette[arg] : 0u;
                        col[1] = (float)((n >> 8) & 0xFFu) / 255.0f;
                        col[2] = (float)(n & 0xFFu) / 255.0f;
                    }
                    break;
                case OMV_FC_MMP:
                case OMV_FC_RMP:
                    if (m->type == MAT_PBR) {
                        float omr[3];
                        pbr_omr(s, m, &sp, omr);
                        f = fc_clamped(subject == OMV_FC_MMP ? omr[1] : omr[2]);
                    }
                    memcpy(&arg, &f, 4);
                    fc_lerp_paint(f, white, subject == OMV_FC_MMP ? blue : green, col);
                    break;
                case OMV_FC_MD:
                case OMV_FC_SG: {
                    float dens, grad;
                    fc_surface_terms(s, &sp, dmin, dmax, &dens, &grad);
                    f = fc_clamped(subject == OMV_FC_MD ? dens : grad);
                    memcpy(&arg, &f, 4);
                    if (subject == OMV_FC_MD)
                        fc_lerp_paint(f, white, red, col);
                    else
                        col[0] = col[1] = col[2] = 1.0f - f;
                    break;
                }
                case OMV_FC_MN: {
                    const char* nm = m->type == MAT_PBR ? "pbr" : (m->type == MAT_OM ? "om" : "mm");
                    unsigned char b[4] = {0, 0, 0, 0};
                    memcpy(b, nm, strlen(nm));
                    memcpy(&arg, b, 4);
                    if (m->type == MAT_PBR) col[2] = 1.0f;
                    else if (m->type == MAT_OM) col[1] = 1.0f;
                    else col[0] = col[2] = 1000.0f;
                    break;
                }
                case OMV_FC_IN: {
                    float tfn[3];
                    face_normal(s, &sp, tfn);
                    const int inv = oc_dot3(inV, tfn) > 0.0f;
                    arg = (uint32_t)inv;
                    col[0] = (float)inv;
                    col[1] = 1.0f - (float)inv;
                    break;
                }
                default: /* EmptySubject */
                    break;
                }
            }
            if (rgba) {
                rgba[4 * id] = col[0];
                rgba[4 * id + 1] = col[1];
                rgba[4 * id + 2] = col[2];
                rgba[4 * id + 3] = 1.0f;
            }
            if (args) args[id] = arg;
            if (uniforms) memcpy(uniforms + 4 * id, u, sizeof(u));
            if (hits) fill_hit(s, &h, hit, &hits[id]);
        }
    }
    return 0;
}

/* RenderMesh::getMinMaxDensity over all instances (for the density checks) */
void oc_density_range(const oc_scene* s, float* out2) { density_range(s, &out2[0], &out2[1]); }

/* The light-box loop (main.cpp:491-521): the views rendered one after another
 * by BDPTRenderer::render at -C 1, all drawing from the scene's one
 * mt19937(seed) generator (RenderScene.cpp:20), each film normalised by stop.
 * films: n * W*H*4 floats (every camera has the same resolution). */
int32_t oc_render_views(const oc_scene* s, int32_t n, const omv_camera* cams, const omv_params* p, uint32_t seed,
                        float* films)
{
    if (!s || !cams || !p || !films || n < 0) return -1;
    oc_mt mt;
    oc_mt_seed(&mt, seed);
    const size_t px = (size_t)cams[0].width * cams[0].height;
    for (int v = 0; v < n; ++v) {
        if ((size_t)cams[v].width * cams[v].height != px) return -1;
        job j;
        j.s = s;
        j.cam = &cams[v];
        j.p = p;
        j.mode = 0;
        j.seed = seed;
        j.row_end = cams[v].height;
        atomic_init(&j.next_row, 0);
        j.film = films + 4 * px * (size_t)v;
        memset(j.film, 0, sizeof(float) * 4 * px);
        j.sumsq = NULL;
        atomic_init(&j.rays, 0ULL);
        render_rows(&j, &mt);
        oc_film_stop(j.film, (int64_t)px);
    }
    return 0;
}

/* BitmapTexture::texture(u, v, fvec4) on one RGBA8 image for n coordinate pairs */
void oc_texture_sample(int32_t w, int32_t h, const uint8_t* rgba, int64_t n, const float* uv, float* out)
{
    oc_tex t = {w, h, (unsigned char*)rgba};
    for (int64_t i = 0; i < n; ++i) tex_sample(&t, uv[2 * i], uv[2 * i + 1], out + 4 * i);
}
