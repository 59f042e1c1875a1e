/*
 * orc.c - CPU oracle: plain-C restatement of the reference's render-path
 * arithmetic (RunningOutRate/kagayaki).  TEST INFRASTRUCTURE ONLY: used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker or the timed CPU baseline; the product never links it.
 *
 * Parity of this restatement is pinned against the reference's own source
 * compiled for the host (oracle/ref, golden fixtures in tests/golden/).
 * Operation order follows the reference expression by expression and the
 * file is built with -ffp-contract=off, so results match the reference's
 * host build bit for bit where no libm call differs.
 */
#include "orc.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Vec (struct_Vec.cuh)                                                       */
/* ------------------------------------------------------------------------ */
typedef struct { float x, y, z, a; } V;

static inline V mk(float x, float y, float z) { V r = {x, y, z, 0.0f}; return r; }
static inline V vadd(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V vsub(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V vmul(V a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline V vdivs(V a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline V vmulv(V a, V b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V vdivv(V a, V b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float absdot(V a, V b) { return fabsf(dot(a, b)); }
static inline float len2(V a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline float len(V a) { return sqrtf(len2(a)); }
static inline V cross(V a, V b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* struct_Vec.cuh:40-46: a zero vector normalises to (10000, 0, 0). */
static inline V normalize(V b) {
    if (len(b) == 0) return mk(10000, 0, 0);
    return vdivs(b, len(b));
}
/* struct_Vec.cuh:81-86 */
static void onb(V n, V *u, V *v, V *w) {
    *w = n;
    if (fabsf(w->x) > 1e-4) *u = normalize(cross(mk(0.0f, 1.0f, 0.0f), *w));
    else *u = normalize(cross(mk(1.0f, 0.0f, 0.0f), *w));
    *v = normalize(cross(*w, *u));
}

static const float sINF = 1e-4f;
static const float bINF = 1e38f;
static const float PI = 3.14159265358979323846263383f;

/* Reference struct layouts. */
typedef struct {
    V v0, v1, v2, n0, n1, n2, t0, t1, t2;
    int32_t material_id;
    unsigned char smooth;
    int32_t shape_id;
} Tri;
typedef struct {
    int32_t type, tex;
    V diffuse, emission;
    float subsurface, metallic, specular, specularTint, roughness, anisotropic, sheen, sheenTint,
          clearcoat, clearcoatGloss, IOR, mu_a, mu_s, scatter_g;
} Mat;
typedef struct { V dir, org; double pad; } Ray;
typedef struct { V org, dir; float dist; V sx, sy; float pixel; } Cam;
typedef struct { float *pixels; int32_t w, h, bpp; } Tex;

_Static_assert(sizeof(Tri) == 156, "Triangle");
_Static_assert(sizeof(Mat) == 96, "Material");
_Static_assert(sizeof(Ray) == 40, "Ray");
_Static_assert(sizeof(Cam) == 72, "Camera");
_Static_assert(sizeof(Tex) == 24, "Texture");

/* ------------------------------------------------------------------------ */
/* Threads                                                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t n, chunk;
    int64_t next;
    pthread_mutex_t mu;
    void (*fn)(void *ctx, int64_t i0, int64_t i1);
    void *ctx;
} pool_t;

static void *pool_worker(void *arg) {
    pool_t *p = (pool_t *)arg;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        int64_t i0 = p->next;
        p->next += p->chunk;
        pthread_mutex_unlock(&p->mu);
        if (i0 >= p->n) break;
        int64_t i1 = i0 + p->chunk < p->n ? i0 + p->chunk : p->n;
        p->fn(p->ctx, i0, i1);
    }
    return NULL;
}

static void parallel_for(int64_t n, int nthreads, int64_t chunk,
                         void (*fn)(void *, int64_t, int64_t), void *ctx) {
    if (nthreads <= 1 || n <= chunk) { fn(ctx, 0, n); return; }
    if (nthreads > 256) nthreads = 256;
    pool_t p;
    p.n = n; p.chunk = chunk; p.next = 0; p.fn = fn; p.ctx = ctx;
    pthread_mutex_init(&p.mu, NULL);
    pthread_t th[256];
    for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, pool_worker, &p);
    for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
    pthread_mutex_destroy(&p.mu);
}

/* ------------------------------------------------------------------------ */
/* Intersection (struct_Triangle.cuh:30-79)                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    float distance;
    V position, normal, normal_ns;
    float u, v;
} Hit;

static int isect_full(const Tri *tr, const Ray *ray, Hit *hp, float *bu, float *bv) {
    V e = cross(vsub(tr->v1, tr->v0), vsub(tr->v2, tr->v0));
    V n;
    if (len(e) == 0) n = normalize(vadd(vadd(tr->n0, tr->n1), tr->n2));
    else n = normalize(e);
    if (absdot(n, ray->dir) <= 0) return 0;
    V e2 = vsub(tr->v2, tr->v0), e1 = vsub(tr->v1, tr->v0), so = vsub(ray->org, tr->v0);
    float term1 = (1.0f / dot(cross(ray->dir, e2), e1));
    float t = term1 * dot(cross(so, e1), e2);
    float u = term1 * dot(cross(ray->dir, e2), so);
    float v = term1 * dot(cross(so, e1), ray->dir);
    if (bu) *bu = u;
    if (bv) *bv = v;
    if (u < 0 || v < 0 || u + v > 1) return 0;
    if ((double)t < 1e-5) return 0;
    if (hp) {
        V uv = vadd(vadd(vmul(tr->t1, u), vmul(tr->t2, v)), vmul(tr->t0, (1 - u - v)));
        if (uv.x < 0) uv.x += (float)((int)(-uv.x) + 1);
        else if (uv.x > 1) uv.x -= (float)((int)(uv.x));
        if (uv.y < 0) uv.y += (float)((int)(-uv.y) + 1);
        else if (uv.y > 1) uv.y -= (float)((int)(uv.y));
        hp->u = uv.x;
        hp->v = uv.y;
        hp->distance = t;
        hp->position = vadd(ray->org, vmul(ray->dir, hp->distance));
        if (!tr->smooth) hp->normal = n;
        else hp->normal = normalize(vadd(vadd(vmul(tr->n1, u), vmul(tr->n2, v)), vmul(tr->n0, (1 - u - v))));
        hp->normal_ns = n;
    }
    return 1;
}

static int isect_t(const Tri *tr, const Ray *ray, float *t_out, float *u_out, float *v_out) {
    V e = cross(vsub(tr->v1, tr->v0), vsub(tr->v2, tr->v0));
    V n;
    if (len(e) == 0) n = normalize(vadd(vadd(tr->n0, tr->n1), tr->n2));
    else n = normalize(e);
    if (absdot(n, ray->dir) <= 0) return 0;
    V e2 = vsub(tr->v2, tr->v0), e1 = vsub(tr->v1, tr->v0), so = vsub(ray->org, tr->v0);
    float term1 = (1.0f / dot(cross(ray->dir, e2), e1));
    float t = term1 * dot(cross(so, e1), e2);
    float u = term1 * dot(cross(ray->dir, e2), so);
    float v = term1 * dot(cross(so, e1), ray->dir);
    if (t_out) *t_out = t;
    if (u_out) *u_out = u;
    if (v_out) *v_out = v;
    if (u < 0 || v < 0 || u + v > 1) return 0;
    if ((double)t < 1e-5) return 0;
    return 1;
}

int orc_intersect_ref(const void *tri, const void *ray, float *t, float *u, float *v) {
    return isect_t((const Tri *)tri, (const Ray *)ray, t, u, v);
}

/* ------------------------------------------------------------------------ */
/* Brute-force closest hit                                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    const Tri *tris;
    int64_t n;
    const Ray *rays;
    int32_t *id;
    float *t;
} brute_ctx;

static void brute_chunk(void *c_, int64_t i0, int64_t i1) {
    brute_ctx *c = (brute_ctx *)c_;
    for (int64_t i = i0; i < i1; ++i) {
        float best = bINF;
        int32_t bid = -1;
        for (int64_t k = 0; k < c->n; ++k) {
            float t;
            if (isect_t(&c->tris[k], &c->rays[i], &t, NULL, NULL) && best > t) {
                best = t;
                bid = (int32_t)k;
            }
        }
        c->id[i] = bid;
        c->t[i] = best;
    }
}

void orc_closest_brute(const void *tris, int64_t n, const void *rays, int64_t nrays,
                       int32_t *face_id, float *t, int nthreads) {
    brute_ctx c = {(const Tri *)tris, n, (const Ray *)rays, face_id, t};
    parallel_for(nrays, nthreads, 256, brute_chunk, &c);
}

/* ------------------------------------------------------------------------ */
/* Fragility classification                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    const Tri *tris;
    int64_t n;
    const Ray *rays;
    const int32_t *id;
    const float *t;
    uint8_t *flags;
} cls_ctx;

static int near_zero(float x) { return fabsf(x) <= 4.0f * 1.1920929e-7f; }

static void cls_chunk(void *c_, int64_t i0, int64_t i1) {
    cls_ctx *c = (cls_ctx *)c_;
    for (int64_t i = i0; i < i1; ++i) {
        uint8_t f = 0;
        float tbest = c->id[i] >= 0 ? c->t[i] : bINF;
        for (int64_t k = 0; k < c->n; ++k) {
            float t, u, v;
            int hit = isect_t(&c->tris[k], &c->rays[i], &t, &u, &v);
            if (hit && k != c->id[i] && t == tbest) f |= 1;
            /* only triangles that could displace or become the answer */
            if (!(t <= tbest * (1.0f + 1e-5f)) || !(t > 0)) continue;
            float w = 1.0f - u - v;
            int inside_loose = u >= -1e-5f && v >= -1e-5f && w >= -1e-5f;
            if (inside_loose && (near_zero(u) || near_zero(v) || near_zero(w))) f |= 2;
            if (inside_loose && fabsf(t - 1e-5f) <= 4.0f * 1.1920929e-7f * 1e-5f) f |= 2;
        }
        c->flags[i] = f;
    }
}

void orc_classify(const void *tris, int64_t n, const void *rays, int64_t nrays,
                  const int32_t *face_id, const float *t, uint8_t *flags, int nthreads) {
    cls_ctx c = {(const Tri *)tris, n, (const Ray *)rays, face_id, t, flags};
    parallel_for(nrays, nthreads, 256, cls_chunk, &c);
}

/* ------------------------------------------------------------------------ */
/* CPU BVH with conservative culling (equals brute force)                     */
/* ------------------------------------------------------------------------ */
typedef struct { float lo[3], hi[3]; int32_t left, count; /* leaf: left = first */ } bnode;
struct orc_bvh {
    const Tri *tris;
    int64_t n;
    int32_t *idx;
    bnode *nodes;
    int64_t nn;
};

typedef struct { float lo[3], hi[3], c[3]; } pbox;

static void box_grow(float *lo, float *hi, const float *plo, const float *phi) {
    for (int a = 0; a < 3; ++a) {
        if (plo[a] < lo[a]) lo[a] = plo[a];
        if (phi[a] > hi[a]) hi[a] = phi[a];
    }
}
static float box_area(const float *lo, const float *hi) {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0) return 0;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

#define ORC_BINS 16
static int64_t bvh_build_rec(orc_bvh *b, pbox *pb, int64_t first, int64_t count, int depth) {
    int64_t me = b->nn++;
    bnode *nd = &b->nodes[me];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = first; i < first + count; ++i) {
        pbox *p = &pb[b->idx[i]];
        box_grow(lo, hi, p->lo, p->hi);
        box_grow(clo, chi, p->c, p->c);
    }
    memcpy(b->nodes[me].lo, lo, sizeof lo);
    memcpy(b->nodes[me].hi, hi, sizeof hi);
    if (count <= 4 || depth > 60) {
        b->nodes[me].left = (int32_t)first;
        b->nodes[me].count = (int32_t)count;
        return me;
    }
    int best_axis = -1, best_bin = -1;
    float best_cost = INFINITY;
    for (int a = 0; a < 3; ++a) {
        float ext = chi[a] - clo[a];
        if (!(ext > 0)) continue;
        int cnt[ORC_BINS] = {0};
        float blo[ORC_BINS][3], bhi[ORC_BINS][3];
        for (int k = 0; k < ORC_BINS; ++k)
            for (int q = 0; q < 3; ++q) { blo[k][q] = INFINITY; bhi[k][q] = -INFINITY; }
        for (int64_t i = first; i < first + count; ++i) {
            pbox *p = &pb[b->idx[i]];
            int k = (int)((p->c[a] - clo[a]) / ext * ORC_BINS);
            if (k >= ORC_BINS) k = ORC_BINS - 1;
            if (k < 0) k = 0;
            cnt[k]++;
            box_grow(blo[k], bhi[k], p->lo, p->hi);
        }
        float rlo[3] = {INFINITY, INFINITY, INFINITY}, rhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        float rarea[ORC_BINS];
        int rcnt[ORC_BINS];
        int acc = 0;
        for (int k = ORC_BINS - 1; k > 0; --k) {
            box_grow(rlo, rhi, blo[k], bhi[k]);
            acc += cnt[k];
            rarea[k] = box_area(rlo, rhi);
            rcnt[k] = acc;
        }
        float llo[3] = {INFINITY, INFINITY, INFINITY}, lhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        int lc = 0;
        for (int k = 0; k < ORC_BINS - 1; ++k) {
            box_grow(llo, lhi, blo[k], bhi[k]);
            lc += cnt[k];
            if (lc == 0 || rcnt[k + 1] == 0) continue;
            float cost = box_area(llo, lhi) * lc + rarea[k + 1] * rcnt[k + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = k; }
        }
    }
    int64_t mid;
    if (best_axis < 0) {
        mid = first + count / 2; /* all centroids coincide: split by index */
    } else {
        float ext = chi[best_axis] - clo[best_axis];
        int64_t i = first, j = first + count - 1;
        while (i <= j) {
            pbox *p = &pb[b->idx[i]];
            int k = (int)((p->c[best_axis] - clo[best_axis]) / ext * ORC_BINS);
            if (k >= ORC_BINS) k = ORC_BINS - 1;
            if (k < 0) k = 0;
            if (k <= best_bin) ++i;
            else { int32_t tmp = b->idx[i]; b->idx[i] = b->idx[j]; b->idx[j] = tmp; --j; }
        }
        mid = i;
        if (mid == first || mid == first + count) mid = first + count / 2;
    }
    int64_t l = bvh_build_rec(b, pb, first, mid - first, depth + 1);
    int64_t r = bvh_build_rec(b, pb, mid, first + count - mid, depth + 1);
    (void)r;
    b->nodes[me].left = (int32_t)l;
    b->nodes[me].count = 0; /* inner: children are l and r = next after l's subtree */
    b->nodes[me].count = -(int32_t)r;
    return me;
}

orc_bvh *orc_bvh_build(const void *tris_, int64_t n) {
    const Tri *tris = (const Tri *)tris_;
    orc_bvh *b = (orc_bvh *)calloc(1, sizeof(orc_bvh));
    b->tris = tris;
    b->n = n;
    b->idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    b->nodes = (bnode *)malloc(sizeof(bnode) * (size_t)(2 * n + 1));
    pbox *pb = (pbox *)malloc(sizeof(pbox) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        const float *p0 = &tris[i].v0.x, *p1 = &tris[i].v1.x, *p2 = &tris[i].v2.x;
        for (int a = 0; a < 3; ++a) {
            float lo = fminf(p0[a], fminf(p1[a], p2[a])), hi = fmaxf(p0[a], fmaxf(p1[a], p2[a]));
            pb[i].lo[a] = lo;
            pb[i].hi[a] = hi;
            pb[i].c[a] = 0.5f * (lo + hi);
        }
        b->idx[i] = (int32_t)i;
    }
    if (n > 0) bvh_build_rec(b, pb, 0, n, 0);
    free(pb);
    return b;
}

void orc_bvh_free(orc_bvh *b) {
    if (!b) return;
    free(b->idx);
    free(b->nodes);
    free(b);
}

/* Slab test in double with a relative widening: never rejects a box that a
 * reference hit point (within its own rounding) could lie in. */
static int slab(const bnode *nd, const double *o, const double *inv, double tmax) {
    double t0 = -1e300, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        double ext = (double)nd->hi[a] - (double)nd->lo[a];
        double pad = 1e-5 * (ext + fabs((double)nd->hi[a]) + fabs((double)nd->lo[a])) + 1e-7;
        double lo = nd->lo[a] - pad, hi = nd->hi[a] + pad;
        if (inv[a] == INFINITY || inv[a] == -INFINITY) {
            if (o[a] < lo || o[a] > hi) return 0;
            continue;
        }
        double ta = (lo - o[a]) * inv[a], tb = (hi - o[a]) * inv[a];
        if (ta > tb) { double s = ta; ta = tb; tb = s; }
        if (ta > t0) t0 = ta;
        if (tb < t1) t1 = tb;
        if (t0 > t1) return 0;
    }
    return t1 >= 0;
}

static void bvh_closest_one(const orc_bvh *b, const Ray *r, int32_t *id_out, float *t_out) {
    int32_t stack[256];
    {
        double o[3] = {r->org.x, r->org.y, r->org.z};
        double d[3] = {r->dir.x, r->dir.y, r->dir.z};
        double inv[3];
        for (int a = 0; a < 3; ++a) inv[a] = 1.0 / d[a];
        float best = bINF;
        int32_t bid = -1;
        int sp = 0;
        if (b->n > 0) stack[sp++] = 0;
        while (sp > 0) {
            const bnode *nd = &b->nodes[stack[--sp]];
            if (!slab(nd, o, inv, (double)best * (1.0 + 1e-6) + 1e-6)) continue;
            if (nd->count > 0) {
                for (int32_t k = 0; k < nd->count; ++k) {
                    int32_t ti = b->idx[nd->left + k];
                    float t;
                    if (isect_t(&b->tris[ti], r, &t, NULL, NULL) &&
                        (t < best || (t == best && ti < bid))) {
                        best = t;
                        bid = ti;
                    }
                }
            } else if (sp + 2 <= 256) {
                stack[sp++] = -nd->count;
                stack[sp++] = nd->left;
            }
        }
        *id_out = bid;
        *t_out = best;
    }
}

typedef struct { const orc_bvh *b; const Ray *rays; int32_t *id; float *t; } bvhq_ctx;

static void bvhq_chunk(void *c_, int64_t i0, int64_t i1) {
    bvhq_ctx *c = (bvhq_ctx *)c_;
    for (int64_t i = i0; i < i1; ++i) bvh_closest_one(c->b, &c->rays[i], &c->id[i], &c->t[i]);
}

void orc_bvh_closest(const orc_bvh *b, const void *rays, int64_t nrays, int32_t *face_id,
                     float *t, int nthreads) {
    bvhq_ctx c = {b, (const Ray *)rays, face_id, t};
    parallel_for(nrays, nthreads, 256, bvhq_chunk, &c);
}

/* ------------------------------------------------------------------------ */
/* RNG (struct_Xorshift.cuh)                                                  */
/* ------------------------------------------------------------------------ */
uint64_t orc_xorshift(uint64_t seed) {
    if (seed == 0) seed++;
    seed = seed ^ (seed << 5);
    seed = seed ^ (seed >> 41);
    seed = seed ^ (seed << 20);
    return seed;
}

float orc_random_range(uint64_t *seed, float lo, float hi) {
    *seed = orc_xorshift(*seed);
    float mid = (hi + lo) * 0.5f;
    float r = (hi - lo) * 0.5f;
    float ret = 2 * ((float)*seed / (float)UINT64_MAX - 0.5f);
    ret = r * ret + mid;
    return ret;
}
#define RND(s, lo, hi) orc_random_range((s), (lo), (hi))

/* ------------------------------------------------------------------------ */
/* Camera (struct_Camera.cuh:27-45, matrix.cuh:11-38)                         */
/* ------------------------------------------------------------------------ */
static void matmul4(const float A[4][4], const float *b, float *out) {
    for (int i = 0; i < 4; ++i) {
        float acc = 0.0f;
        for (int l = 0; l < 4; ++l) acc += A[i][l] * b[l];
        out[i] = acc;
    }
}

static V rotate3(float x, float y, float z, V init) {
    float rx[4][4] = {{1, 0, 0, 0}, {0, cosf(x), -sinf(x), 0}, {0, sinf(x), cosf(x), 0}, {0, 0, 0, 1}};
    float ry[4][4] = {{cosf(y), 0, sinf(y), 0}, {0, 1, 0, 0}, {-sinf(y), 0, cosf(y), 0}, {0, 0, 0, 1}};
    float rz[4][4] = {{cosf(z), -sinf(z), 0, 0}, {sinf(z), cosf(z), 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    float b[4] = {init.x, init.y, init.z, 1}, t1[4], t2[4], t3[4];
    matmul4(rx, b, t1);
    matmul4(ry, t1, t2);
    matmul4(rz, t2, t3);
    return normalize(mk(t3[0], t3[1], t3[2]));
}

void orc_camera_setup(const float *org, float dist, float rx, float ry, float rz,
                      int image_height, void *out_) {
    const float D2R = 0.01745329f;
    V up = rotate3(D2R * rx, D2R * ry, D2R * rz, normalize(mk(0.0f, 1.0f, 0.0f)));
    V dir = rotate3(D2R * rx, D2R * ry, D2R * rz, normalize(mk(0.0f, 0.0f, -1.0f)));
    Cam c;
    memset(&c, 0, sizeof c);
    c.org = mk(org[0], org[1], org[2]);
    c.dir = dir;
    c.dist = dist;
    c.sx = cross(dir, up);
    c.sy = up;
    c.pixel = 36.0f / (float)image_height;
    memcpy(out_, &c, sizeof c);
}

/* ------------------------------------------------------------------------ */
/* Tone map (FileIO/IO_save_png.cuh)                                          */
/* ------------------------------------------------------------------------ */
static float clampf(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

void orc_tonemap_rgba8(const float *img, int64_t npx, uint8_t *out) {
    for (int64_t i = 0; i < npx; ++i) {
        for (int c = 0; c < 3; ++c) {
            float g = powf(img[4 * i + c], 1 / 2.2f);
            g = clampf(g, 0.0f, 1.0f);
            out[4 * i + c] = (uint8_t)(g * 255);
        }
        out[4 * i + 3] = 255;
    }
}

/* ------------------------------------------------------------------------ */
/* Light CDFs                                                                 */
/* ------------------------------------------------------------------------ */
static float tri_area(const Tri *t) { return 0.5f * len(cross(vsub(t->v1, t->v0), vsub(t->v2, t->v0))); }

void orc_light_cdf(const void *tris_, int64_t n, const void *mats_, float *cdf) {
    const Tri *tris = (const Tri *)tris_;
    const Mat *mats = (const Mat *)mats_;
    if (n <= 0) return;
    cdf[0] = tri_area(&tris[0]) * len(mats[tris[0].material_id].emission);
    for (int64_t i = 1; i < n; ++i)
        cdf[i] = cdf[i - 1] + tri_area(&tris[i]) * len(mats[tris[i].material_id].emission);
}

void orc_env_cdf(const float *px, int w, int h, int bpp, float *cdf) {
    const int64_t n = (int64_t)w * h;
    if (n == 0) return;
    const float PIH = 3.14159265358979323846263383f;
    float v = 1.0;
    cdf[0] = len(mk(px[0], px[1], px[2])) * cosf((v - 0.5f) * PIH);
    for (int64_t i = 1; i < n; ++i) {
        v = 1.0f - (float)(i / w) / (float)h;
        cdf[i] = cdf[i - 1] + len(mk(px[bpp * i], px[bpp * i + 1], px[bpp * i + 2])) * cosf((v - 0.5f) * PIH);
    }
}

/* ------------------------------------------------------------------------ */
/* Compat estimator                                                           */
/* ------------------------------------------------------------------------ */
typedef struct {
    const Tri *tris;
    int64_t n;
    const Mat *mats;
    const Tex *tex;
    const float *hdr;
    int hw, hh, hbpp;
    const float *lss;
    int64_t lss_n;
    const float *lssh;
    int64_t lssh_n;
    int no_light, no_hdr;
    Cam cam;
    int W, H, frames;
    uint64_t *seeds;
    float *out;
    int64_t *rays; /* per-thread-chunk counts accumulate here under lock */
    pthread_mutex_t mu;
    const orc_bvh *bvh;      /* NULL: brute-force closest hits */
    const int32_t *px_list;  /* NULL: all pixels but 0 */
    int64_t n_px;
} rctx;

/* Algorithms.cuh:6-20 */
static int lower_bound_f(const float *a, int64_t n, float k) {
    int64_t ng = -1, ok = n - 1;
    while (ok - ng > 1) {
        int64_t mid = (ok + ng) / 2;
        if (a[mid] >= k) ok = mid;
        else ng = mid;
    }
    return (int)ok;
}

static int closest(const rctx *c, const Ray *r, Hit *out, int *id) {
    if (c->bvh) {
        int32_t bid;
        float bt;
        bvh_closest_one(c->bvh, r, &bid, &bt);
        *id = bid;
        if (bid < 0) { out->distance = bINF; return 0; }
        isect_full(&c->tris[bid], r, out, NULL, NULL);
        return 1;
    }
    float best = bINF;
    int bid = -1;
    Hit h;
    for (int64_t k = 0; k < c->n; ++k) {
        if (isect_full(&c->tris[k], r, &h, NULL, NULL)) {
            if (best > h.distance) {
                best = h.distance;
                bid = (int)k;
                *out = h;
            }
        }
    }
    *id = bid;
    if (bid < 0) out->distance = bINF;
    return bid >= 0;
}

/* ImageBasedLighting.cuh:6-31 */
static V uv_sphere(V d) {
    float theta, phi;
    phi = asinf(d.z);
    if ((double)fabsf(d.z) >= 1.0 - (double)sINF) theta = 0.0f;
    else if (fabsf(d.x) <= sINF) theta = d.y > 0 ? PI / 2 : -PI / 2;
    else {
        if (d.x > 0) theta = asinf(d.y / sqrtf(1 - d.z * d.z));
        else if (d.x < 0 && d.y > 0) theta = PI - asinf(d.y / sqrtf(1 - d.z * d.z));
        else theta = -1 * PI - asinf(d.y / sqrtf(1 - d.z * d.z));
    }
    theta = clampf(theta / (2 * PI) + 0.5f, 0.0f, 1.0f);
    phi = clampf(phi / PI + 0.5f, 0.0f, 1.0f);
    return mk(theta, phi, 0.0f);
}

static V hdr_emission(const rctx *c, V d) {
    V uv = uv_sphere(d);
    int idx = c->hw * (int)((float)(c->hh - 1) * (1 - uv.y)) + (int)((float)(c->hw - 1) * (1 - uv.x));
    /* a NaN direction (a degenerate sample) indexes nothing in the reference's
     * defined behaviour; clamp like the device code */
    if (idx < 0 || idx >= c->hw * c->hh) idx = idx < 0 ? 0 : c->hw * c->hh - 1;
    idx *= c->hbpp;
    return mk(c->hdr[idx], c->hdr[idx + 1], c->hdr[idx + 2]);
}

static V hdr_index_to_dir(const rctx *c, int index, float *pdf) {
    float u = 1.0f - (float)(index % c->hw) / (float)c->hw;
    float v = 1.0f - (float)(index / c->hw) / (float)c->hh;
    float theta = (u - 0.5f) * 2 * PI;
    float phi = (v - 0.5f) * PI;
    if (fabsf(cosf(phi)) < sINF) *pdf *= 1.0f / (2.0f * PI * PI * sINF);
    else *pdf *= 1.0f / (2.0f * PI * PI * cosf(phi));
    *pdf *= (float)(c->hw * c->hh);
    return mk((float)cosf(phi) * cosf(theta), (float)cosf(phi) * sinf(theta), (float)sinf(phi));
}

static float hdr_pdf(const rctx *c, V d) {
    V uv = uv_sphere(d);
    int idx = (c->hw * (int)((float)c->hh * (1.0f - uv.y)) + (int)((float)c->hw * (uv.x)));
    if (idx >= c->hw * c->hh) idx = c->hw * c->hh - 1; /* reference reads one past the end */
    if (idx < 0) idx = 0;
    if (idx == 0) return c->lssh[0] / c->lssh[c->lssh_n - 1];
    return (c->lssh[idx] - c->lssh[idx - 1]) / c->lssh[c->lssh_n - 1];
}

/* Disney_BRDF.cuh */
static float sqrf(float a) { return a * a; }
static float schlick(float u) { float m = 1 - u; return m * m * m * m * m; }
static V fr_schlick(V F, V n, V Vv) {
    float p = (float)pow((double)(1 - dot(Vv, n)), 5);
    return vadd(F, vmul(vsub(mk(1, 1, 1), F), p));
}
static float d_gtr2(V h, float ax, float ay, V u, V v, V w) {
    float hu = dot(h, u), hv = dot(h, v), hw = dot(h, w);
    double p = pow((double)((hu * hu) / (ax * ax) + (hv * hv) / (ay * ay) + hw * hw), 2);
    return (float)(1 / ((double)(PI * ax * ay) * p));
}
static float d_berry(V h, V n, float alpha) {
    alpha = clampf(alpha, 0.0001f, 0.9999f);
    return ((alpha * alpha - 1) / (2 * PI * logf(alpha))) / ((alpha * alpha - 1) * absdot(h, n) * absdot(h, n) + 1);
}
static float g_lambda(V w, V h, float ax, float ay) {
    V wx, wy, wz;
    onb(h, &wx, &wy, &wz);
    float a = dot(wx, w), b = dot(wy, w), cz = dot(wz, w);
    return 0.5f * (-1 + sqrtf(1 + (ax * ax * a * a + ay * ay * b * b) / (cz * cz)));
}
static float g_ggx(V in, V out, float ax, float ay) {
    V h = normalize(vadd(out, in));
    return 1 / (1 + g_lambda(in, h, ax, ay) + g_lambda(out, h, ax, ay));
}
static float smith_g(float NdotV, float alphaG) {
    float a = alphaG * alphaG, b = NdotV * NdotV;
    return 1 / (NdotV + sqrtf(a + b - a * b));
}
static V brdf_diffuse(const Mat *m, V out, V in, V n) {
    float FL = schlick(dot(n, in)), FV = schlick(dot(n, out));
    V h = normalize(vadd(out, in));
    float fd90 = 0.5f + 2 * m->roughness * absdot(h, in) * absdot(h, in);
    float fd = ((1 - FL) + FL * fd90) * ((1 - FV) + FV * fd90);
    return vmul(vdivs(m->diffuse, PI), fd);
}
static V brdf_subsurface(const Mat *m, V out, V in, V n) {
    V h = normalize(vadd(out, in));
    float FL = schlick(dot(n, in)), FV = schlick(dot(n, out));
    float fss90 = m->roughness * dot(h, in) * dot(h, in);
    float fss = ((1 - FL) + FL * fss90) * ((1 - FV) + FV * fss90);
    return vmul(vmul(vdivs(m->diffuse, PI), 1.25f), (fss * (1 / (dot(n, in) + dot(n, out)) - 0.5f) + 0.5f));
}
static V brdf_sheen(const Mat *m, V out, V in, V n) {
    (void)n;
    V rho = vadd(vmul(mk(1, 1, 1), (1 - m->sheenTint)), vmul(normalize(m->diffuse), m->sheenTint));
    V h = normalize(vadd(out, in));
    float p = (float)pow((double)(1 - dot(h, in)), 5);
    return vmul(vmul(rho, m->sheen), p);
}
static V brdf_specular(const Mat *m, V out, V in, V n, V u, V v, V w, float ax, float ay) {
    V rho = vadd(vmul(mk(1, 1, 1), (1 - m->specularTint)), vmul(normalize(m->diffuse), m->specularTint));
    V h = normalize(vadd(out, in));
    V f0 = vadd(vmul(rho, (1.0f - m->metallic) * 0.08f * m->specular), vmul(m->diffuse, m->metallic));
    V r = vmul(fr_schlick(f0, n, h), d_gtr2(h, ax, ay, u, v, w));
    r = vmul(r, g_ggx(in, out, ax, ay));
    return vdivs(r, (4 * absdot(in, n) * absdot(out, n)));
}
static V brdf_clearcoat(const Mat *m, V out, V in, V n, float ac) {
    V h = normalize(vadd(out, in));
    float ni = dot(n, in), no = dot(n, out);
    V r = vmul(fr_schlick(mk(0.04f, 0.04f, 0.04f), n, h), 0.25f * m->clearcoat);
    r = vmul(r, d_berry(h, n, ac));
    r = vmul(r, smith_g(ni, .25f));
    return vmul(r, smith_g(no, .25f));
}
static V disney_eval(const float *wt, const Mat *m, V out, V in, V n, V u, V v, V w, float ax,
                     float ay, float ac) {
    V b = mk(0, 0, 0);
    if (dot(n, in) < 0 || dot(n, out) < 0) return b;
    b = vadd(b, vmul(brdf_diffuse(m, out, in, n), wt[0]));
    b = vadd(b, vmul(brdf_subsurface(m, out, in, n), wt[1]));
    b = vadd(b, vmul(brdf_sheen(m, out, in, n), wt[2]));
    b = vadd(b, vmul(brdf_specular(m, out, in, n, u, v, w, ax, ay), wt[3]));
    b = vadd(b, vmul(brdf_clearcoat(m, out, in, n, ac), wt[4]));
    return b;
}
static float disney_pdf(const float *wt, V in, V out, V n, V u, V v, V w, float ax, float ay,
                        float ac) {
    float sw = 0, pdf = 0;
    V h = normalize(vadd(out, in));
    for (int i = 0; i < 5; ++i) sw += wt[i];
    pdf += (wt[0] + wt[1] + wt[2]) * (fmaxf(dot(n, out), 0.0f) / PI);
    pdf += wt[3] * (d_gtr2(h, ax, ay, u, v, w) * absdot(n, h) / (4 * absdot(n, out)));
    pdf += wt[4] * (d_berry(h, n, ac) * absdot(n, h) / (4 * absdot(n, out)));
    pdf /= sw;
    return pdf;
}

/* LambertBRDF_sampling.cuh:10-29 */
static V sample_cos(uint64_t *s, V u, V v, V w) {
    float R1 = RND(s, 0, 1.0f);
    float R2 = RND(s, 0, 0.9999f);
    float theta = acosf(sqrtf(1.0f - R2));
    float phi = 2 * PI * R1;
    return normalize(vadd(vadd(vmul(vmul(u, sinf(theta)), cosf(phi)), vmul(vmul(v, sinf(theta)), sinf(phi))),
                          vmul(w, cosf(theta))));
}

/* Disney_BRDF_sampling.cuh */
static V sample_gtr2(uint64_t *s, V u, V v, V w, float ax, float ay) {
    float R1 = RND(s, 0.0001f, 0.9999f);
    float R2 = RND(s, 0.0001f, 0.9999f);
    V a = vmul(u, ax * cosf(2 * PI * R1));
    V b = vmul(v, ay * sinf(2 * PI * R1));
    V h = vadd(vmul(vadd(a, b), sqrtf(R2 / (1 - R2))), w);
    return normalize(h);
}
static V sample_gtr1(uint64_t *s, V u, V v, V w, float alpha) {
    float R1 = RND(s, 0.0001f, 0.9999f);
    float cosphi = cosf(2 * PI * R1);
    float sinphi = sqrtf(1 - cosphi * cosphi);
    float R2 = RND(s, 0.0001f, 0.9999f);
    alpha = clampf(alpha, -0.9999f, 0.9999f);
    float costheta = sqrtf((1 - powf(alpha, 2 * (1 - R2))) / (1 - alpha * alpha));
    float sintheta = sqrtf(1 - costheta * costheta);
    return vadd(vadd(vmul(u, sintheta * cosphi), vmul(v, sintheta * sinphi)), vmul(w, costheta));
}

/* sampling.cuh:11-26 in its zero-initialised reading: Sum = {w0, w0, w1, w2, w3}. */
static int sample_bxdf(uint64_t *s, const float *w) {
    float R = RND(s, 0.0f, 1.0f);
    float sum[5] = {0, 0, 0, 0, 0};
    sum[0] = w[0];
    for (int i = 1; i < 5; ++i) sum[i] += w[i - 1];
    R *= sum[4];
    return lower_bound_f(sum, 5, R);
}

/* Argument order of SamplePointOnTriangle(random, random, tri) in the host
 * build: g++ evaluates the call's arguments right to left, so the second
 * random number is drawn first. */
static int g_point_args_rtl = 1;

static V sample_point_on_tri(float r1, float r2, const Tri *t) {
    float t1 = r1 / 2.0f, t2 = r2 / 2.0f;
    float off = t2 - t1;
    if (off > 0) t2 += off;
    else t1 -= off;
    return vadd(vadd(vmul(t->v0, t1), vmul(t->v1, t2)), vmul(t->v2, (1 - t1 - t2)));
}

typedef struct {
    float aspect, a_sheen, ax, ay, ac;
    float wt[5];
} DisneyP;

static void disney_params(const Mat *m, DisneyP *p) {
    p->aspect = sqrtf(1.0f - 0.9f * m->anisotropic);
    p->a_sheen = m->roughness * m->roughness;
    p->ax = fmaxf(0.001f, m->roughness * m->roughness / p->aspect);
    p->ay = fmaxf(0.001f, m->roughness * m->roughness * p->aspect);
    p->ac = (1.0f - m->clearcoatGloss) * 0.1f + m->clearcoatGloss * 0.001f;
    p->wt[0] = (1 - m->subsurface) * (1 - m->metallic);
    p->wt[1] = m->subsurface * (1 - m->metallic);
    p->wt[2] = 1 - m->metallic;
    p->wt[3] = 1.0f;
    p->wt[4] = 1.0f;
}

static void bsdf_and_pdf(const Mat *m, const DisneyP *p, V n, V in_neg_ray, V out, V *bsdf, float *pdf) {
    if (m->type == 0) {
        *bsdf = vdivs(m->diffuse, PI);
        *pdf = fmaxf(dot(n, out), 0.0f) / PI;
    } else if (m->type == 1) {
        V u, v, w;
        onb(n, &u, &v, &w);
        *bsdf = disney_eval(p->wt, m, out, in_neg_ray, n, u, v, w, p->ax, p->ay, p->ac);
        *pdf = disney_pdf(p->wt, in_neg_ray, out, n, u, v, w, p->ax, p->ay, p->ac);
    } else {
        *bsdf = mk(0, 0, 0);
        *pdf = 0;
    }
}

/* NextEventEstimation_FaceLight.cuh:47-120 */
static void nee_face(const rctx *c, V *rad, V T, uint64_t *s, const Ray *ray, const Mat *m,
                     const DisneyP *p, const Hit *hp, V n, int64_t *nr) {
    if (len(m->emission) != 0 || m->type >= 2 || c->lss_n == 0) return;
    float R = RND(s, 0, 1);
    int id;
    if (c->no_light) id = -1;
    else id = lower_bound_f(c->lss, c->lss_n, R * c->lss[c->lss_n - 1]);
    float r1, r2;
    if (g_point_args_rtl) { r2 = RND(s, 0, 1); r1 = RND(s, 0, 1); }
    else { r1 = RND(s, 0, 1); r2 = RND(s, 0, 1); }
    /* no face light: the reference samples Objects[-1] (undefined); here the
     * step draws its three numbers and contributes nothing */
    if (id < 0) return;
    V P = sample_point_on_tri(r1, r2, &c->tris[id]);
    V L = normalize(vsub(P, hp->position));
    float dist = len(vsub(P, hp->position));
    Ray sr;
    sr.dir = L; sr.org = hp->position; sr.pad = 0;
    if (dot(L, n) <= 0) return;
    Hit sh;
    int sid;
    ++*nr;
    if (!closest(c, &sr, &sh, &sid) || sid != id) return;
    float cos1 = fabsf(dot(hp->normal, L)), cos2 = fabsf(dot(sh.normal, vmul(L, -1.0f)));
    float G = cos1 * cos2 / (dist * dist);
    float pdf_nee;
    if (id == 0) pdf_nee = (c->lss[0] / c->lss[c->lss_n - 1]) * (1.0f / tri_area(&c->tris[0]));
    else pdf_nee = ((c->lss[id] - c->lss[id - 1]) / c->lss[c->lss_n - 1]) * (1.0f / tri_area(&c->tris[id]));
    float p_pt = 0, p_face = pdf_nee, p_hdr = 0;
    if (!c->no_hdr) p_hdr = hdr_pdf(c, sr.dir);
    V bsdf;
    bsdf_and_pdf(m, p, n, vmul(ray->dir, -1.0f), sr.dir, &bsdf, &p_pt);
    p_pt *= G / fabsf(dot(sr.dir, hp->normal));
    float mis = p_face / (p_pt + p_face + p_hdr);
    V r = vmulv(vdivs(vmul(bsdf, G), pdf_nee), c->mats[c->tris[id].material_id].emission);
    r = vmul(r, mis);
    *rad = vadd(*rad, vmulv(T, r));
}

/* NextEventEstimation_HDR.cuh:4-58 */
static void nee_hdr(const rctx *c, V *rad, V T, uint64_t *s, const Ray *ray, const Mat *m,
                    const DisneyP *p, const Hit *hp, V n, int64_t *nr) {
    if (c->no_hdr) return;
    float R = RND(s, 0, 1);
    int pix = lower_bound_f(c->lssh, c->lssh_n, R * c->lssh[c->lssh_n - 1]);
    float pdf;
    if (pix == 0) pdf = c->lssh[0] / c->lssh[c->lssh_n - 1];
    else pdf = (c->lssh[pix] - c->lssh[pix - 1]) / c->lssh[c->lssh_n - 1];
    V d = hdr_index_to_dir(c, pix, &pdf);
    Ray sr;
    sr.dir = d; sr.org = hp->position; sr.pad = 0;
    if (dot(d, n) <= 0) return;
    Hit sh;
    int sid;
    ++*nr;
    if (closest(c, &sr, &sh, &sid)) return;
    V Le = mk(c->hdr[pix * c->hbpp], c->hdr[pix * c->hbpp + 1], c->hdr[pix * c->hbpp + 2]);
    V bsdf;
    float p_pt;
    bsdf_and_pdf(m, p, n, vmul(ray->dir, -1.0f), d, &bsdf, &p_pt);
    float mis = pdf / (p_pt + pdf);
    V r = vmul(vmulv(bsdf, vdivs(Le, pdf)), dot(n, d));
    r = vmul(r, mis);
    *rad = vadd(*rad, vmulv(r, T));
}

/* sampling.cuh:28-64; returns the next ray, updates T */
static Ray sample_next(uint64_t *s, V *T, const Mat *m, const DisneyP *p, const Ray *ray,
                       const Hit *hp, V n) {
    Ray nr;
    memset(&nr, 0, sizeof nr);
    V u, v, w;
    onb(n, &u, &v, &w);
    if (m->type == 0) {
        nr.dir = sample_cos(s, u, v, w);
        nr.org = hp->position;
        *T = vmulv(m->diffuse, *T);
    } else if (m->type == 1) {
        int lobe = sample_bxdf(s, p->wt);
        if (lobe <= 2) {
            nr.dir = sample_cos(s, u, v, w);
        } else if (lobe == 3) {
            V h = sample_gtr2(s, u, v, w, p->ax, p->ay);
            nr.dir = normalize(vsub(ray->dir, vmul(h, 2 * dot(ray->dir, h))));
        } else {
            V h = sample_gtr1(s, u, v, w, p->ac);
            nr.dir = normalize(vsub(ray->dir, vmul(h, 2 * dot(ray->dir, h))));
        }
        nr.org = hp->position;
        V b = disney_eval(p->wt, m, nr.dir, vmul(ray->dir, -1.0f), n, u, v, w, p->ax, p->ay, p->ac);
        float pdf = disney_pdf(p->wt, vmul(ray->dir, -1.0f), nr.dir, n, u, v, w, p->ax, p->ay, p->ac);
        *T = vmulv(*T, vdivs(vmul(b, absdot(n, nr.dir)), pdf));
    }
    return nr;
}

static V tex_color(const Tex *t, float u, float v) {
    int idx = (t->w * (int)((float)t->h * (1 - v)) + (int)((float)t->w * u));
    int np = t->w * t->h;
    if (idx >= np) idx = np - 1; /* reference reads past the end for v == 0 */
    if (idx < 0) idx = 0;
    idx *= t->bpp;
    return mk(t->pixels[idx], t->pixels[idx + 1], t->pixels[idx + 2]);
}

/* RayTrace.cuh:9-109 */
static V raytrace(const rctx *c, Ray ray, uint64_t *s, int64_t *nr) {
    int depth = -1;
    V T = mk(1, 1, 1);
    V rad = mk(sINF, sINF, sINF);
    for (;;) {
        depth++;
        Hit hp;
        int id;
        ++*nr;
        if (!closest(c, &ray, &hp, &id)) {
            if (c->no_hdr) rad = vadd(rad, vmulv(T, mk(1, 1, 1)));
            else rad = vadd(rad, vmulv(T, hdr_emission(c, ray.dir)));
            break;
        }
        const Tri *face = &c->tris[id];
        Mat m = c->mats[face->material_id];
        V n = dot(hp.normal, ray.dir) > 0.0 ? vmul(hp.normal, -1.0f) : hp.normal;
        if (m.tex != -1) m.diffuse = tex_color(&c->tex[m.tex], hp.u, hp.v);
        if ((double)len(m.diffuse) < 1e-5) m.diffuse = mk(sINF, sINF, sINF);
        if (depth == 0) ++*nr; /* reprojection traversal of the G-buffer */
        DisneyP p;
        disney_params(&m, &p);
        /* Russian roulette (RayTrace_Russian_Roulette.cuh:4-36), (2, 3) */
        {
            float prr = fmaxf(m.diffuse.x, fmaxf(m.diffuse.y, m.diffuse.z));
            if (prr == 0) prr = sINF;
            float rnd = RND(s, 0, 1);
            if (depth > 3) prr /= (float)(depth * depth);
            if (depth > 2) {
                if (prr < rnd) {
                    rad = vadd(rad, vmulv(T, m.emission));
                    break;
                }
            } else {
                prr = 1.0f;
            }
            if (depth == 0) rad = vadd(rad, vmulv(T, m.emission));
            T = vdivs(T, prr);
        }
        nee_face(c, &rad, T, s, &ray, &m, &p, &hp, n, nr);
        nee_hdr(c, &rad, T, s, &ray, &m, &p, &hp, n, nr);
        if (m.type == 0) { /* NextEventEstimation_PathTracing.cuh: draws, traces, adds 0 */
            V T2 = T;
            Ray pr = sample_next(s, &T2, &m, &p, &ray, &hp, n);
            if (dot(pr.dir, n) > 0) ++*nr;
        }
        ray = sample_next(s, &T, &m, &p, &ray, &hp, n);
    }
    return rad;
}

/* struct_Camera.cuh:38-45 */
static Ray primary(const Cam *cam, int x, int y, int W, int H) {
    V d = vadd(vadd(vmul(cam->dir, cam->dist),
                    vmul(vmul(cam->sx, ((float)x - W / 2.0f)), cam->pixel)),
               vmul(vmul(cam->sy, (H / 2.0f - (float)y)), cam->pixel));
    Ray r;
    r.dir = normalize(d);
    r.org = cam->org;
    r.pad = 0;
    return r;
}

static void render_chunk(void *c_, int64_t i0, int64_t i1) {
    rctx *c = (rctx *)c_;
    int64_t nr = 0;
    const int64_t npx = (int64_t)c->W * c->H;
    for (int64_t i = i0; i < i1; ++i) {
        int pos = c->px_list ? (int)c->px_list[i] : (int)(i + 1);
        if (pos <= 0 || pos >= npx) continue;
        int X = pos % c->W, Y = pos / c->W;
        uint64_t s = c->seeds[pos];
        for (int f = 0; f < c->frames; ++f) {
            /* render.cuh:29: int arithmetic (142857*pos wraps), added to u64 */
            int32_t m1 = (int32_t)((uint32_t)142857u * (uint32_t)pos);
            uint64_t seed = s + (uint64_t)(int64_t)m1 + (uint64_t)(int64_t)(998244353 / pos) +
                            (uint64_t)(int64_t)(1000000007 % pos);
            Ray r = primary(&c->cam, X, Y, c->W, c->H);
            V v = raytrace(c, r, &seed, &nr);
            s = seed;
            float *o = c->out + ((size_t)f * npx + pos) * 3;
            o[0] = v.x;
            o[1] = v.y;
            o[2] = v.z;
        }
        c->seeds[pos] = s;
    }
    pthread_mutex_lock(&c->mu);
    *c->rays += nr;
    pthread_mutex_unlock(&c->mu);
}

int64_t orc_render_compat(const void *tris, int64_t n, const void *mats, int64_t nm,
                          const void *textures, int n_tex, const float *hdr, int hdr_w,
                          int hdr_h, int hdr_bpp, const void *cam, int width, int height,
                          int frames, int nthreads, float *out) {
    (void)nm;
    (void)n_tex;
    rctx c;
    memset(&c, 0, sizeof c);
    c.tris = (const Tri *)tris;
    c.n = n;
    c.mats = (const Mat *)mats;
    c.tex = (const Tex *)textures;
    c.hdr = hdr;
    c.hw = hdr_w;
    c.hh = hdr_h;
    c.hbpp = hdr_bpp;
    float *lss = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    orc_light_cdf(tris, n, mats, lss);
    c.lss = lss;
    c.lss_n = n;
    c.no_light = n > 0 && lss[n - 1] == 0;
    float *lssh = NULL;
    c.no_hdr = hdr == NULL;
    if (hdr) {
        lssh = (float *)malloc(sizeof(float) * (size_t)hdr_w * hdr_h);
        orc_env_cdf(hdr, hdr_w, hdr_h, hdr_bpp, lssh);
        c.lssh = lssh;
        c.lssh_n = (int64_t)hdr_w * hdr_h;
    }
    memcpy(&c.cam, cam, sizeof(Cam));
    c.W = width;
    c.H = height;
    c.frames = frames;
    const int64_t npx = (int64_t)width * height;
    c.seeds = (uint64_t *)calloc((size_t)npx, sizeof(uint64_t));
    c.out = out;
    int64_t rays = 0;
    c.rays = &rays;
    pthread_mutex_init(&c.mu, NULL);
    for (int f = 0; f < frames; ++f) out[(size_t)f * npx * 3] = out[(size_t)f * npx * 3 + 1] =
        out[(size_t)f * npx * 3 + 2] = NAN;
    parallel_for(npx - 1, nthreads, 16, render_chunk, &c);
    pthread_mutex_destroy(&c.mu);
    free(c.seeds);
    free(lss);
    free(lssh);
    return rays;
}

/* Test hook: selects the argument order of SamplePointOnTriangle's random
 * numbers (1 = right to left, the host build's order). */
void orc_set_point_arg_order(int rtl) { g_point_args_rtl = rtl; }

/* evaluate_Disney_BRDF / _pdf for one material and n direction triples,
 * parameters as RayTrace.cuh:85-92 (test hook mirroring ref_disney_eval). */
void orc_disney_eval(const void *mat, int n, const float *wo, const float *wi, const float *nrm,
                     float *brdf, float *pdf) {
    const Mat *m = (const Mat *)mat;
    DisneyP p;
    disney_params(m, &p);
    for (int i = 0; i < n; ++i) {
        V o = mk(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        V in = mk(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        V N = mk(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        V u, v, w;
        onb(N, &u, &v, &w);
        V b = disney_eval(p.wt, m, o, in, N, u, v, w, p.ax, p.ay, p.ac);
        brdf[3 * i] = b.x;
        brdf[3 * i + 1] = b.y;
        brdf[3 * i + 2] = b.z;
        pdf[i] = disney_pdf(p.wt, in, o, N, u, v, w, p.ax, p.ay, p.ac);
    }
}

/* The compat estimator over a list of pixels (1..W*H-1) of a W x H frame,
 * one sample each, with closest hits from a CPU BVH (orc_bvh_build); for
 * scenes too large for brute force.  out = n_px * 3 floats (pixel order of
 * the list).  Returns the number of traversal calls. */
int64_t orc_render_compat_px(const void *tris, int64_t n, const void *mats, const orc_bvh *bvh,
                             const float *hdr, int hdr_w, int hdr_h, int hdr_bpp, const void *cam,
                             int width, int height, const int32_t *px_list, int64_t n_px, int nthreads,
                             float *out) {
    rctx c;
    memset(&c, 0, sizeof c);
    c.tris = (const Tri *)tris;
    c.n = n;
    c.mats = (const Mat *)mats;
    c.hdr = hdr;
    c.hw = hdr_w;
    c.hh = hdr_h;
    c.hbpp = hdr_bpp;
    float *lss = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    orc_light_cdf(tris, n, mats, lss);
    c.lss = lss;
    c.lss_n = n;
    c.no_light = n > 0 && lss[n - 1] == 0;
    float *lssh = NULL;
    c.no_hdr = hdr == NULL;
    if (hdr) {
        lssh = (float *)malloc(sizeof(float) * (size_t)hdr_w * hdr_h);
        orc_env_cdf(hdr, hdr_w, hdr_h, hdr_bpp, lssh);
        c.lssh = lssh;
        c.lssh_n = (int64_t)hdr_w * hdr_h;
    }
    memcpy(&c.cam, cam, sizeof(Cam));
    c.W = width;
    c.H = height;
    c.frames = 1;
    const int64_t npx = (int64_t)width * height;
    c.seeds = (uint64_t *)calloc((size_t)npx, sizeof(uint64_t));
    float *full = (float *)calloc((size_t)npx * 3, sizeof(float));
    c.out = full;
    int64_t rays = 0;
    c.rays = &rays;
    c.bvh = bvh;
    c.px_list = px_list;
    c.n_px = n_px;
    pthread_mutex_init(&c.mu, NULL);
    parallel_for(n_px, nthreads, 4, render_chunk, &c);
    pthread_mutex_destroy(&c.mu);
    for (int64_t k = 0; k < n_px; ++k) {
        int64_t p = px_list[k];
        if (p <= 0 || p >= npx) continue;
        out[3 * k] = full[3 * p];
        out[3 * k + 1] = full[3 * p + 1];
        out[3 * k + 2] = full[3 * p + 2];
    }
    free(full);
    free(c.seeds);
    free(lss);
    free(lssh);
    return rays;
}

/* ------------------------------------------------------------------------ */
/* SVGF, race-free reading (SVGF.cuh:10-522)                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    V albedo, emission, normal, history;
    int32_t object_id, material_id;
    int32_t pos_i[2];
    float pos_f[2];
    int32_t sample_num;
    float m1, m2, variance, depth;
    unsigned char atrous, temporal;
    unsigned char pad[2];
} SB;
_Static_assert(sizeof(SB) == 112, "SVGFBuffer");

static void sb_init(SB *b) { /* struct_SVGFBuffers.cuh:31-47 */
    b->albedo = mk(0, 0, 0);
    b->emission = mk(0, 0, 0);
    b->normal = mk(0, 0, 0);
    b->history = mk(0, 0, 0);
    b->object_id = -1;
    b->material_id = -1;
    b->pos_i[0] = b->pos_i[1] = -1;
    b->pos_f[0] = b->pos_f[1] = -1;
    b->sample_num = 0;
    b->m1 = -1.0f;
    b->m2 = -1.0f;
    b->variance = 0.0f;
    b->depth = 0.0f;
    b->atrous = 1;
    b->temporal = 0;
}

static float lum(V c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
static float depth_w(float d, float nd, int dx, int dy, float gx, float gy) {
    float top = -1.0f * fabsf(d - nd);
    float bottom = 1.0f * fabsf((float)dx * gx + (float)dy * gy) + sINF;
    return expf(top / bottom);
}
static float normal_w(V n, V nn) {
    float c = fmaxf(0.0f, dot(n, nn));
    c *= c; c *= c; c *= c; c *= c; c *= c; c *= c; c *= c;
    return c;
}
static float lum_w(float l, float nl, float sd) {
    float top = -1.0f * fabsf(l - nl);
    float bottom = 4.0f * sd + sINF;
    return expf(top / bottom);
}

/* One ApplySVGF call over all pixels with a full barrier at every
 * __syncthreads.  result/filtered: npx Vec (4 floats); prev/cur: npx SB. */
void orc_svgf_compat(int W, int H, float *result_, float *filtered_, void *prev_, void *cur_, int frame) {
    const int npx = W * H;
    V *R = (V *)result_, *F = (V *)filtered_;
    SB *P = (SB *)prev_, *C = (SB *)cur_;
    float *M1 = (float *)calloc((size_t)npx, sizeof(float));
    float *M2 = (float *)calloc((size_t)npx, sizeof(float));
    float *sd = (float *)calloc((size_t)npx, sizeof(float));
    unsigned char *spatial = (unsigned char *)calloc((size_t)npx, 1);
    float *sw = (float *)calloc((size_t)npx, sizeof(float));
    float *s1 = (float *)calloc((size_t)npx, sizeof(float));
    float *s2 = (float *)calloc((size_t)npx, sizeof(float));
    V *R2 = (V *)calloc((size_t)npx, sizeof(V));
    float *var2 = (float *)calloc((size_t)npx, sizeof(float));
    float *gz = (float *)calloc((size_t)npx * 2, sizeof(float));
    /* ApplySVGF prologue (SVGF.cuh:498-511) */
    for (int p = 0; p < npx; ++p) {
        if (!isfinite(len(R[p]))) R[p] = mk(0.0f, 0.0f, 0.0f);
        if (frame == 0) sb_init(&P[p]);
        if (P[p].m1 == -1.0f) {
            V c = vdivv(R[p], C[p].albedo);
            C[p].m1 = lum(c);
            C[p].m2 = C[p].m1 * C[p].m1;
        }
        F[p] = mk(0, 0, 0);
    }
    /* TemporalAccumulation (SVGF.cuh:50-98) */
    for (int p = 0; p < npx; ++p) {
        if (len(C[p].emission) != 0) continue;
        int px = C[p].pos_i[0], py = C[p].pos_i[1];
        float s = C[p].pos_f[0] - (float)px, t = C[p].pos_f[1] - (float)py;
        int off[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
        float w[4] = {(1 - s) * (1 - t), s * (1 - t), (1 - s) * t, s * t};
        V sum = mk(0, 0, 0);
        float swt = 0.0f;
        for (int i = 0; i < 4; ++i) {
            int qx = px + off[i][0], qy = py + off[i][1];
            if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
            int q = W * qy + qx;
            if (P[q].material_id == C[p].material_id && P[q].temporal) {
                sum = vadd(sum, vmul(P[q].history, w[i]));
                swt += w[i];
            }
        }
        if (swt == 0.0f) continue;
        V hist = vdivs(sum, swt);
        R[p] = vadd(vmul(R[p], 0.2f), vmul(hist, (float)0.8));
    }
    /* VarianceEstimation (SVGF.cuh:112-275), phase by phase */
    for (int p = 0; p < npx; ++p) {
        int x = p % W, y = p / W;
        V dc = vdivv(R[p], vadd(C[p].albedo, mk(sINF, sINF, sINF)));
        float l = lum(dc);
        M1[p] = l;
        M2[p] = l * l;
        int prev = W * C[p].pos_i[1] + C[p].pos_i[0];
        spatial[p] = C[p].pos_i[0] == -1 || P[prev].sample_num < 3;
        int dx = x < W / 2 ? 1 : -1, dy = y < H / 2 ? 1 : -1;
        float d = C[p].depth;
        gz[2 * p] = (C[W * y + x + dx].depth - d) / (float)dx;
        gz[2 * p + 1] = (C[W * (y + dy) + x].depth - d) / (float)dy;
    }
    for (int p = 0; p < npx; ++p) {
        if (spatial[p]) continue;
        int prev = W * C[p].pos_i[1] + C[p].pos_i[0];
        C[p].sample_num = P[prev].sample_num + 1;
        float cw = 1.0f / 5.0f;
        if (C[p].sample_num < 5) cw = 1.0f / (float)C[p].sample_num;
        C[p].m1 = (1.0f - cw) * P[prev].m1 + cw * M1[p];
        C[p].m2 = (1.0f - cw) * P[prev].m2 + cw * M2[p];
        M1[p] = C[p].m1;
        M2[p] = C[p].m2;
    }
    static const float K7[7] = {0.00598f, 0.060626f, 0.241843f, 0.383103f, 0.241843f, 0.060626f, 0.00598f};
    for (int p = 0; p < npx; ++p) {
        sw[p] = s1[p] = s2[p] = 0.0f;
        if (!spatial[p]) continue;
        int x = p % W, y = p / W;
        float a = 0, b = 0, c = 0;
        for (int kx = -3; kx <= 3; ++kx) {
            int nx = x + kx;
            if (nx < 0 || nx >= W) continue;
            float hx = K7[kx + 3];
            for (int ky = -3; ky <= 3; ++ky) {
                int ny = y + ky;
                if (ny < 0 || ny >= H) continue;
                float hy = K7[ky + 3];
                if (kx == 0 && ky == 0) {
                    a += hx * hy * M1[p];
                    b += hx * hy * M2[p];
                    c += hx * hy;
                    continue;
                }
                int q = W * ny + nx;
                if (C[q].object_id == -1) continue;
                float wm = C[p].material_id == C[q].material_id ? 1.0f : 0.0f;
                float wz = depth_w(C[p].depth, C[q].depth, kx, ky, gz[2 * p], gz[2 * p + 1]);
                float wn = normal_w(C[p].normal, C[q].normal);
                float wt = hx * hy * wz * wn * wm;
                a += wt * M1[q];
                b += wt * M2[q];
                c += wt;
            }
        }
        s1[p] = a;
        s2[p] = b;
        sw[p] = c;
    }
    for (int p = 0; p < npx; ++p) {
        int prev = W * C[p].pos_i[1] + C[p].pos_i[0];
        if (C[p].object_id == -1) {
            F[p] = R[p];
            sb_init(&C[p]);
            C[p].atrous = 0;
        } else if (spatial[p] && sw[p] == 0) {
            F[p] = R[p];
            sb_init(&C[p]);
            C[p].atrous = 0;
        } else if (spatial[p]) {
            C[p].m1 = s1[p] / sw[p];
            C[p].m2 = s2[p] / sw[p];
            if (C[p].pos_i[0] == -1) C[p].sample_num = 1;
            else C[p].sample_num = P[prev].sample_num + 1;
        }
    }
    for (int p = 0; p < npx; ++p) {
        if (C[p].object_id == -1) continue;
        C[p].variance = fmaxf(0.0f, C[p].m2 - C[p].m1 * C[p].m1);
        if (C[p].variance > 1000) C[p].variance = 1000;
    }
    /* ApplyGaussianFilterToVar (SVGF.cuh:277-344) */
    static const float KG[3] = {1 / 4.0f, 1 / 2.0f, 1 / 4.0f};
    for (int p = 0; p < npx; ++p) {
        int x = p % W, y = p / W;
        float sv = 0, swt = 0;
        for (int kx = -1; kx <= 1; ++kx) {
            float hx = KG[kx + 1];
            int nx = x + kx;
            if (nx < 0 || nx >= W) continue;
            for (int ky = -1; ky <= 1; ++ky) {
                float hy = KG[ky + 1];
                int ny = y + ky;
                if (ny < 0 || ny >= H) continue;
                int q = W * ny + nx;
                if (C[q].object_id == -1) continue;
                float wt = hx * hy;
                sv += wt * C[q].variance;
                swt += wt;
            }
        }
        s1[p] = sv;
        sw[p] = swt;
    }
    for (int p = 0; p < npx; ++p) {
        sd[p] = 0.0f;
        if (s1[p] == 0 && sw[p] != 0) {
            F[p] = R[p];
            C[p].atrous = 0;
        } else if (sw[p] == 0) {
            C[p].m1 = -1.0f;
            C[p].m2 = -1.0f;
            C[p].sample_num = 0;
            C[p].atrous = 0;
        } else {
            C[p].variance = s1[p] / sw[p];
            sd[p] = sqrtf(s1[p] / sw[p]);
        }
    }
    /* 5 x 5 a-trous stages (SVGF.cuh:347-474, 486-491) */
    static const float KW[25] = {1 / 256.0f, 4 / 256.0f, 6 / 256.0f, 4 / 256.0f, 1 / 256.0f,
                                 4 / 256.0f, 16 / 256.0f, 24 / 256.0f, 16 / 256.0f, 4 / 256.0f,
                                 6 / 256.0f, 24 / 256.0f, 36 / 256.0f, 24 / 256.0f, 6 / 256.0f,
                                 4 / 256.0f, 16 / 256.0f, 24 / 256.0f, 16 / 256.0f, 4 / 256.0f,
                                 1 / 256.0f, 4 / 256.0f, 6 / 256.0f, 4 / 256.0f, 1 / 256.0f};
    for (int k = 0; k < 5; ++k) {
        for (int stage = 0; stage < 5; ++stage) {
            for (int p = 0; p < npx; ++p) {
                R2[p] = R[p];
                var2[p] = C[p].variance;
            }
            for (int p = 0; p < npx; ++p) {
                int x = p % W, y = p / W;
                V dc = vdivv(R2[p], vadd(C[p].albedo, mk(sINF, sINF, sINF)));
                float l = lum(dc);
                float d = C[p].depth;
                int dx = x < W / 2 ? 1 : -1, dy = y < H / 2 ? 1 : -1;
                float gx = (C[W * y + x + dx].depth - d) / (float)dx;
                float gy = (C[W * (y + dy) + x].depth - d) / (float)dy;
                V srad = mk(0.0f, 0.0f, 0.0f);
                float svar = 0.0f, swt = 0.0f;
                for (int ki = 0; ki < 25; ++ki) {
                    float h = KW[ki];
                    int ox = ki % 5 - 2, oy = ki / 5 - 2;
                    int qx = x + (ox * (1 << stage)), qy = y + (oy * (1 << stage));
                    if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
                    int q = W * qy + qx;
                    if (ki == 12) {
                        svar += h * h * var2[p];
                        srad = vadd(srad, vmul(dc, h));
                        swt += h;
                        continue;
                    }
                    if (C[q].object_id == -1) continue;
                    V nr = vdivv(R2[q], vadd(C[q].albedo, mk(sINF, sINF, sINF)));
                    float nl = lum(nr);
                    if (((double)l > 0.5 && nl > 5 * l) || ((double)l > 0.1 && nl > 50 * l) ||
                        (l > sINF && nl > 100 * l))
                        continue;
                    float wm = C[p].material_id == C[q].material_id ? 1 : 0;
                    float wz = depth_w(d, C[q].depth, qx, qy, gx, gy);
                    float wn = normal_w(C[p].normal, C[q].normal);
                    float wl = lum_w(l, nl, sd[p]);
                    float wt = C[p].atrous ? h * wz * wn * wl * wm : h * wz * wn * wm;
                    srad = vadd(srad, vmul(nr, wt));
                    svar += wt * wt * var2[q];
                    swt += wt;
                }
                if (C[p].object_id == -1) continue;
                if (swt < 1e-6f || swt * swt < 1e-6f) {
                    F[p] = R2[p];
                    C[p].temporal = 1;
                    continue;
                }
                V fl = vdivs(srad, swt);
                float fv = svar / (swt * swt);
                float cw = 0.2f;
                V out = vadd(vmul(vmulv(fl, C[p].albedo), cw), vmul(R2[p], (1 - cw)));
                F[p] = out;
                R[p] = out;
                if (C[p].atrous) C[p].variance = cw * var2[p] + (1 - cw) * fv;
                if (stage == 0) {
                    C[p].history = out;
                    C[p].temporal = 1;
                }
            }
        }
    }
    for (int p = 0; p < npx; ++p) R[p] = C[p].history;
    free(M1); free(M2); free(sd); free(spatial); free(sw); free(s1); free(s2);
    free(R2); free(var2); free(gz);
}
