/*
 * ORACLE -- test infrastructure only (see oc_core.h and oc_bvh.h).
 * Binned-SAH binary BVH (CPU) and the watertight closest-hit query that stands
 * in for Embree's rtcIntersect1 (reference call site BDPTRenderer.cpp:84).
 */
#include "oc_bvh.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OC_LEAF_MAX 4
#define OC_BINS 16
/* relative widening of a slab exit distance: covers the three roundings of
 * (bound - org) * (1/dir) (a robust box test in the sense of PBRT's 1+2*gamma(3)) */
#define OC_BOX_WIDEN 1.00000048f

const float* oc_mesh_vertex(const oc_tri_mesh* m, uint32_t vi)
{
    return (const float*)(m->vtx + (size_t)vi * m->vtx_stride);
}

void oc_mesh_face(const oc_tri_mesh* m, int32_t f, uint32_t out[3])
{
    const uint32_t* p = (const uint32_t*)((const unsigned char*)m->idx + (size_t)f * m->idx_stride);
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
}

void oc_free_bvh(oc_bvh* b)
{
    free(b->nodes);
    free(b->items);
    b->nodes = NULL;
    b->items = NULL;
    b->n_nodes = 0;
    b->n_items = 0;
}

typedef struct build_item {
    float lo[3], hi[3], c[3];
} build_item;

static float half_area(const float* lo, const float* hi)
{
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0.0f;
    return dx * dy + dy * dz + dz * dx;
}

static void box_reset(float* lo, float* hi)
{
    lo[0] = lo[1] = lo[2] = INFINITY;
    hi[0] = hi[1] = hi[2] = -INFINITY;
}

static void box_grow(float* lo, float* hi, const float* blo, const float* bhi)
{
    for (int a = 0; a < 3; ++a) {
        if (blo[a] < lo[a]) lo[a] = blo[a];
        if (bhi[a] > hi[a]) hi[a] = bhi[a];
    }
}

/* generic binned SAH build over item boxes; items[] holds the item ids */
static int build_bvh(oc_bvh* b, const build_item* it, int32_t n, int leaf_max)
{
    b->n_items = n;
    b->items = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    b->nodes = (oc_bnode*)malloc(sizeof(oc_bnode) * (size_t)(2 * (n > 0 ? n : 1)));
    if (!b->items || !b->nodes) return -1;
    for (int32_t i = 0; i < n; ++i) b->items[i] = i;
    b->n_nodes = 1;
    if (n == 0) {
        box_reset(b->nodes[0].lo, b->nodes[0].hi);
        b->nodes[0].left = 0;
        b->nodes[0].count = 0;
        return 0;
    }
    typedef struct { int32_t node, first, count; } task;
    task* stack = (task*)malloc(sizeof(task) * (size_t)(2 * n + 2));
    if (!stack) return -1;
    int sp = 0;
    stack[sp++] = (task){0, 0, n};
    while (sp) {
        task t = stack[--sp];
        oc_bnode* nd = &b->nodes[t.node];
        float lo[3], hi[3], clo[3], chi[3];
        box_reset(lo, hi);
        box_reset(clo, chi);
        for (int32_t i = t.first; i < t.first + t.count; ++i) {
            const build_item* x = &it[b->items[i]];
            box_grow(lo, hi, x->lo, x->hi);
            box_grow(clo, chi, x->c, x->c);
        }
        memcpy(nd->lo, lo, sizeof(lo));
        memcpy(nd->hi, hi, sizeof(hi));
        int best_axis = -1, best_split = -1;
        float best_cost = INFINITY;
        if (t.count > leaf_max) {
            for (int a = 0; a < 3; ++a) {
                float ext = chi[a] - clo[a];
                if (!(ext > 0.0f)) continue;
                int cnt[OC_BINS] = {0};
                float blo[OC_BINS][3], bhi[OC_BINS][3];
                for (int k = 0; k < OC_BINS; ++k) box_reset(blo[k], bhi[k]);
                float scale = (float)OC_BINS / ext;
                for (int32_t i = t.first; i < t.first + t.count; ++i) {
                    const build_item* x = &it[b->items[i]];
                    int k = (int)((x->c[a] - clo[a]) * scale);
                    if (k >= OC_BINS) k = OC_BINS - 1;
                    if (k < 0) k = 0;
                    cnt[k]++;
                    box_grow(blo[k], bhi[k], x->lo, x->hi);
                }
                float rlo[3], rhi[3], racc[OC_BINS];
                int rcnt[OC_BINS];
                box_reset(rlo, rhi);
                int rc = 0;
                for (int k = OC_BINS - 1; k > 0; --k) {
                    box_grow(rlo, rhi, blo[k], bhi[k]);
                    rc += cnt[k];
                    racc[k] = half_area(rlo, rhi);
                    rcnt[k] = rc;
                }
                float llo[3], lhi[3];
                box_reset(llo, lhi);
                int lc = 0;
                for (int k = 0; k < OC_BINS - 1; ++k) {
                    box_grow(llo, lhi, blo[k], bhi[k]);
                    lc += cnt[k];
                    if (lc == 0 || rcnt[k + 1] == 0) continue;
                    float cost = half_area(llo, lhi) * (float)lc + racc[k + 1] * (float)rcnt[k + 1];
                    if (cost < best_cost) {
                        best_cost = cost;
                        best_axis = a;
                        best_split = k;
                    }
                }
            }
        }
        int make_leaf = (t.count <= leaf_max) || best_axis < 0;
        if (!make_leaf) {
            float leaf_cost = half_area(lo, hi) * (float)t.count;
            if (best_cost >= leaf_cost && t.count <= 2 * leaf_max) make_leaf = 1;
        }
        int32_t mid = -1;
        if (!make_leaf) {
            float ext = chi[best_axis] - clo[best_axis];
            float scale = (float)OC_BINS / ext;
            int32_t i = t.first, j = t.first + t.count - 1;
            while (i <= j) {
                const build_item* x = &it[b->items[i]];
                int k = (int)((x->c[best_axis] - clo[best_axis]) * scale);
                if (k >= OC_BINS) k = OC_BINS - 1;
                if (k < 0) k = 0;
                if (k <= best_split) {
                    ++i;
                } else {
                    int32_t tmp = b->items[i];
                    b->items[i] = b->items[j];
                    b->items[j] = tmp;
                    --j;
                }
            }
            mid = i;
            if (mid == t.first || mid == t.first + t.count) make_leaf = 1;
        }
        if (make_leaf && t.count > 255) {
            /* degenerate centroids: median split by index */
            make_leaf = 0;
            mid = t.first + t.count / 2;
        }
        if (make_leaf) {
            nd->left = t.first;
            nd->count = t.count;
        } else {
            int32_t l = b->n_nodes;
            b->n_nodes += 2;
            nd->left = l;
            nd->count = 0;
            stack[sp++] = (task){l + 1, mid, t.first + t.count - mid};
            stack[sp++] = (task){l, t.first, mid - t.first};
        }
    }
    free(stack);
    return 0;
}

int oc_build_mesh_bvh(oc_tri_mesh* m)
{
    build_item* it = (build_item*)malloc(sizeof(build_item) * (size_t)(m->n_tri > 0 ? m->n_tri : 1));
    if (!it) return -1;
    for (int32_t f = 0; f < m->n_tri; ++f) {
        uint32_t fi[3];
        oc_mesh_face(m, f, fi);
        build_item* x = &it[f];
        box_reset(x->lo, x->hi);
        for (int k = 0; k < 3; ++k) {
            const float* p = oc_mesh_vertex(m, fi[k]);
            box_grow(x->lo, x->hi, p, p);
        }
        for (int a = 0; a < 3; ++a) x->c[a] = 0.5f * (x->lo[a] + x->hi[a]);
    }
    int rc = build_bvh(&m->bvh, it, m->n_tri, OC_LEAF_MAX);
    free(it);
    return rc;
}

void oc_affine_inverse(const float xf[3][4], float inv[3][4])
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
        for (int j = 0; j < 3; ++j) inv[i][j] = (float)r[i][j];
        inv[i][3] = (float)t;
    }
}

int oc_build_tlas(oc_accel* a)
{
    build_item* it = (build_item*)malloc(sizeof(build_item) * (size_t)(a->n_inst > 0 ? a->n_inst : 1));
    if (!it) return -1;
    for (int32_t i = 0; i < a->n_inst; ++i) {
        oc_instance* in = &a->inst[i];
        oc_affine_inverse((const float(*)[4])in->xf, in->inv);
        const oc_bnode* root = &in->mesh->bvh.nodes[0];
        box_reset(in->lo, in->hi);
        if (in->mesh->n_tri > 0) {
            for (int c = 0; c < 8; ++c) {
                double p[3] = {(c & 1) ? root->hi[0] : root->lo[0], (c & 2) ? root->hi[1] : root->lo[1],
                               (c & 4) ? root->hi[2] : root->lo[2]};
                float w[3];
                for (int k = 0; k < 3; ++k)
                    w[k] = (float)((double)in->xf[k][0] * p[0] + (double)in->xf[k][1] * p[1] +
                                   (double)in->xf[k][2] * p[2] + (double)in->xf[k][3]);
                box_grow(in->lo, in->hi, w, w);
            }
            /* widen: object-space hits must never be culled in world space */
            for (int k = 0; k < 3; ++k) {
                float pad = (in->hi[k] - in->lo[k]) * 1e-5f + (fabsf(in->lo[k]) + fabsf(in->hi[k])) * 1e-5f + 1e-20f;
                in->lo[k] -= pad;
                in->hi[k] += pad;
            }
        }
        build_item* x = &it[i];
        memcpy(x->lo, in->lo, sizeof(x->lo));
        memcpy(x->hi, in->hi, sizeof(x->hi));
        for (int k = 0; k < 3; ++k) x->c[k] = 0.5f * (x->lo[k] + x->hi[k]);
        if (in->mesh->n_tri == 0)
            for (int k = 0; k < 3; ++k) x->c[k] = 0.0f;
    }
    int rc = build_bvh(&a->tlas, it, a->n_inst, 1);
    free(it);
    return rc;
}

/* ------------------------------------------------------------ queries --- */

typedef struct wt_ray {
    int kx, ky, kz;
    float Sx, Sy, Sz;
} wt_ray;

/* returns 0 for a direction that is zero or not finite (no hit possible) */
static int wt_setup(const float* d, wt_ray* w)
{
    if (!(fabsf(d[0]) <= FLT_MAX && fabsf(d[1]) <= FLT_MAX && fabsf(d[2]) <= FLT_MAX)) return 0;
    float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) { kz = 2; m = az; }
    if (!(m > 0.0f)) return 0;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    if (d[kz] < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    w->kx = kx;
    w->ky = ky;
    w->kz = kz;
    w->Sx = d[kx] / d[kz];
    w->Sy = d[ky] / d[kz];
    w->Sz = 1.0f / d[kz];
    return 1;
}

static int wt_triangle(const wt_ray* w, const float* o, const float* p0, const float* p1, const float* p2, float tnear,
                       float tfar, float* t, float* u, float* v)
{
    const float A[3] = {p0[0] - o[0], p0[1] - o[1], p0[2] - o[2]};
    const float B[3] = {p1[0] - o[0], p1[1] - o[1], p1[2] - o[2]};
    const float C[3] = {p2[0] - o[0], p2[1] - o[1], p2[2] - o[2]};
    const int kx = w->kx, ky = w->ky, kz = w->kz;
    const float Ax = A[kx] - w->Sx * A[kz];
    const float Ay = A[ky] - w->Sy * A[kz];
    const float Bx = B[kx] - w->Sx * B[kz];
    const float By = B[ky] - w->Sy * B[kz];
    const float Cx = C[kx] - w->Sx * C[kz];
    const float Cy = C[ky] - w->Sy * C[kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
        double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
        double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
        U = (float)(cxby - cybx);
        V = (float)(axcy - aycx);
        W = (float)(bxay - byax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    const float det = U + V + W;
    if (det == 0.0f) return 0;
    const float Az = w->Sz * A[kz];
    const float Bz = w->Sz * B[kz];
    const float Cz = w->Sz * C[kz];
    const float T = U * Az + V * Bz + W * Cz;
    const float rcp = 1.0f / det;
    const float tt = T * rcp;
    if (!(tt >= tnear && tt <= tfar)) return 0;
    *t = tt;
    *u = V * rcp;
    *v = W * rcp;
    return 1;
}

static int box_test(const float* lo, const float* hi, const float* o, const float* idir, float tnear, float tfar,
                    float* tentry)
{
    float t0 = tnear, t1 = tfar;
    for (int a = 0; a < 3; ++a) {
        float tn = (lo[a] - o[a]) * idir[a];
        float tf = (hi[a] - o[a]) * idir[a];
        if (tn > tf) {
            float s = tn;
            tn = tf;
            tf = s;
        }
        tf = tf * OC_BOX_WIDEN;
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return 0;
    }
    *tentry = t0;
    return 1;
}

typedef struct best_hit {
    float t;
    uint32_t inst, prim, geom;
    float u, v;
    int found;
} best_hit;

static void consider(best_hit* b, float t, float u, float v, uint32_t inst, uint32_t geom, uint32_t prim)
{
    int take = 0;
    if (!b->found || t < b->t)
        take = 1;
    else if (t == b->t && (inst < b->inst || (inst == b->inst && prim < b->prim)))
        take = 1;
    if (take) {
        b->found = 1;
        b->t = t;
        b->u = u;
        b->v = v;
        b->inst = inst;
        b->geom = geom;
        b->prim = prim;
    }
}

static void trace_blas(const oc_instance* in, const float* wo, const float* wd, float tnear, best_hit* b)
{
    const float(*M)[4] = (const float(*)[4])in->inv;
    float o[3], d[3];
    for (int i = 0; i < 3; ++i) {
        o[i] = M[i][0] * wo[0] + M[i][1] * wo[1] + M[i][2] * wo[2] + M[i][3];
        d[i] = M[i][0] * wd[0] + M[i][1] * wd[1] + M[i][2] * wd[2];
    }
    wt_ray w;
    if (!wt_setup(d, &w)) return;
    const float idir[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    const oc_tri_mesh* m = in->mesh;
    const oc_bvh* bvh = &m->bvh;
    int32_t stack[256];
    int sp = 0;
    float te;
    if (!box_test(bvh->nodes[0].lo, bvh->nodes[0].hi, o, idir, tnear, b->t, &te)) return;
    stack[sp++] = 0;
    while (sp) {
        const oc_bnode* nd = &bvh->nodes[stack[--sp]];
        if (nd->count > 0) {
            for (int32_t i = nd->left; i < nd->left + nd->count; ++i) {
                uint32_t prim = (uint32_t)bvh->items[i];
                uint32_t fi[3];
                oc_mesh_face(m, (int32_t)prim, fi);
                float t, u, v;
                if (wt_triangle(&w, o, oc_mesh_vertex(m, fi[0]), oc_mesh_vertex(m, fi[1]), oc_mesh_vertex(m, fi[2]), tnear,
                                b->t, &t, &u, &v))
                    consider(b, t, u, v, in->inst_id, m->geom_id, prim);
            }
            continue;
        }
        const oc_bnode* l = &bvh->nodes[nd->left];
        const oc_bnode* r = &bvh->nodes[nd->left + 1];
        float tl, tr;
        int hl = box_test(l->lo, l->hi, o, idir, tnear, b->t, &tl);
        int hr = box_test(r->lo, r->hi, o, idir, tnear, b->t, &tr);
        if (hl && hr) {
            if (tl <= tr) {
                stack[sp++] = nd->left + 1;
                stack[sp++] = nd->left;
            } else {
                stack[sp++] = nd->left;
                stack[sp++] = nd->left + 1;
            }
        } else if (hl) {
            stack[sp++] = nd->left;
        } else if (hr) {
            stack[sp++] = nd->left + 1;
        }
    }
}

int oc_intersect(const oc_accel* a, const oc_ray* r, oc_hitrec* h)
{
    best_hit b;
    memset(&b, 0, sizeof(b));
    b.t = r->tfar;
    if (!(r->tnear <= r->tfar) || a->n_inst == 0) return 0;
    wt_ray w0;
    if (!wt_setup(r->dir, &w0)) return 0;
    const float idir[3] = {1.0f / r->dir[0], 1.0f / r->dir[1], 1.0f / r->dir[2]};
    const oc_bvh* bvh = &a->tlas;
    int32_t stack[256];
    int sp = 0;
    float te;
    if (!box_test(bvh->nodes[0].lo, bvh->nodes[0].hi, r->org, idir, r->tnear, b.t, &te)) return 0;
    stack[sp++] = 0;
    while (sp) {
        const oc_bnode* nd = &bvh->nodes[stack[--sp]];
        if (nd->count > 0) {
            for (int32_t i = nd->left; i < nd->left + nd->count; ++i) {
                const oc_instance* in = &a->inst[bvh->items[i]];
                if (in->mesh->n_tri == 0) continue;
                float ti;
                if (!box_test(in->lo, in->hi, r->org, idir, r->tnear, b.t, &ti)) continue;
                trace_blas(in, r->org, r->dir, r->tnear, &b);
            }
            continue;
        }
        const oc_bnode* l = &bvh->nodes[nd->left];
        const oc_bnode* rr = &bvh->nodes[nd->left + 1];
        float tl, tr;
        int hl = box_test(l->lo, l->hi, r->org, idir, r->tnear, b.t, &tl);
        int hr = box_test(rr->lo, rr->hi, r->org, idir, r->tnear, b.t, &tr);
        if (hl && hr) {
            if (tl <= tr) {
                stack[sp++] = nd->left + 1;
                stack[sp++] = nd->left;
            } else {
                stack[sp++] = nd->left;
                stack[sp++] = nd->left + 1;
            }
        } else if (hl) {
            stack[sp++] = nd->left;
        } else if (hr) {
            stack[sp++] = nd->left + 1;
        }
    }
    if (!b.found) return 0;
    h->inst = b.inst;
    h->geom = b.geom;
    h->prim = b.prim;
    h->t = b.t;
    h->u = b.u;
    h->v = b.v;
    return 1;
}
