/*
 * nbvh_oracle.c -- TEST INFRASTRUCTURE ONLY (see nbvh_oracle.h).
 *
 * CPU restatement of the reference's N-BVH ray-query path. Each function cites the reference
 * file:line it follows (paths relative to the reference project root). Parity: UNPINNED -- the
 * reference has no golden vectors and cannot be built here; see nbvh_oracle.h.
 *
 * Compile with -ffp-contract=off -fno-fast-math: every FP32 operation below is rounded on its
 * own, in the order written, which is the order glm evaluates the reference expressions in
 * (dot = (x*x' + y*y') + z*z', cross = (a.y*b.z - b.y*a.z, ...), min(a,b) = b < a ? b : a,
 * max(a,b) = a < b ? b : a, normalize(v) = v * (1 / sqrt(dot(v, v)))).
 */
#include "nbvh_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------------ */
/* glm-semantics FP32 vector helpers                                                          */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    float x, y, z;
} v3;

static inline v3 mk(float x, float y, float z)
{
    v3 r = {x, y, z};
    return r;
}
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vdiv(v3 a, v3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 vscale(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 vadds(v3 a, float s) { return mk(a.x + s, a.y + s, a.z + s); }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b)
{
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline float gmin(float a, float b) { return (b < a) ? b : a; }
static inline float gmax(float a, float b) { return (a < b) ? b : a; }
static inline v3 vmin(v3 a, v3 b) { return mk(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
static inline v3 vmax(v3 a, v3 b) { return mk(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
static inline float cmax(v3 v) { return gmax(gmax(v.x, v.y), v.z); } /* common.cuh:38-41 */
static inline float cmin(v3 v) { return gmin(gmin(v.x, v.y), v.z); } /* common.cuh:43-46 */
static inline v3 vnormalize(v3 v) { return vscale(v, 1.0f / sqrtf(vdot(v, v))); }
static inline float vlength(v3 v) { return sqrtf(vdot(v, v)); }
static inline float gclamp01(float x) { return gmin(gmax(x, 0.0f), 1.0f); }

static inline v3 load3(const float *p) { return mk(p[0], p[1], p[2]); }
static inline float u2f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static inline uint32_t f2u(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

/* ------------------------------------------------------------------------------------------ */
/* RNG: include/cuda/utils/lcg_rng.cuh                                                        */
/* ------------------------------------------------------------------------------------------ */

uint32_t orc_murmur_mix(uint32_t hash, uint32_t k) /* lcg_rng.cuh:12-29 */
{
    k *= 0xcc9e2d51u;
    k = (k << 15) | (k >> 17);
    k *= 0x1b873593u;
    hash ^= k;
    hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
    return hash;
}

uint32_t orc_murmur_finalize(uint32_t hash) /* lcg_rng.cuh:31-40 */
{
    hash ^= hash >> 16;
    hash *= 0x85ebca6bu;
    hash ^= hash >> 13;
    hash *= 0xc2b2ae35u;
    hash ^= hash >> 16;
    return hash;
}

uint32_t orc_lcg_seed(uint32_t index, uint32_t frame, uint32_t linear) /* lcg_rng.cuh:65-72 */
{
    uint32_t s = orc_murmur_mix(0u, linear);
    s = orc_murmur_mix(s, 512u * frame + index);
    return orc_murmur_finalize(s);
}

float orc_lcg_randomf(uint32_t *state) /* lcg_rng.cuh:42-53: ldexp((float)u32, -32) */
{
    *state = *state * 1664525u + 1013904223u;
    return (float)(*state) * 0x1p-32f;
}

/* sin(2 pi u), cos(2 pi u): octant reduction on u (exact in FP32), then Taylor series of degree
 * 11 (sin) and 12 (cos) on [0, pi/4] evaluated with fused multiply-adds. The reference calls
 * sin/cos of 2*PI*u (sampling.cuh:8-14); this is a deterministic replacement that the device code
 * evaluates with the same operations, so oracle and GPU agree bit for bit. */
void orc_sincos_turns(float u, float *s, float *c)
{
    float y = u * 8.0f;
    float o = floorf(y);
    float f = y - o;
    int oct = ((int)o) & 7;
    float g = (oct & 1) ? (1.0f - f) : f;
    float x = g * 0.785398163397448310f;
    float x2 = x * x;
    float ps = fmaf(x2, -2.50521084e-08f, 2.75573192e-06f);
    ps = fmaf(x2, ps, -1.98412698e-04f);
    ps = fmaf(x2, ps, 8.33333333e-03f);
    ps = fmaf(x2, ps, -1.66666667e-01f);
    ps = fmaf(x2, ps, 1.0f);
    float sn = x * ps;
    float pc = fmaf(x2, 2.08767570e-09f, -2.75573192e-07f);
    pc = fmaf(x2, pc, 2.48015873e-05f);
    pc = fmaf(x2, pc, -1.38888889e-03f);
    pc = fmaf(x2, pc, 4.16666667e-02f);
    pc = fmaf(x2, pc, -0.5f);
    float cs = fmaf(x2, pc, 1.0f);
    float rs, rc;
    switch (oct) {
    case 0: rs = sn; rc = cs; break;
    case 1: rs = cs; rc = sn; break;
    case 2: rs = cs; rc = -sn; break;
    case 3: rs = sn; rc = -cs; break;
    case 4: rs = -sn; rc = -cs; break;
    case 5: rs = -cs; rc = -sn; break;
    case 6: rs = -cs; rc = sn; break;
    default: rs = -sn; rc = cs; break;
    }
    *s = rs;
    *c = rc;
}

/* square_to_uniform_sphere, include/cuda/utils/sampling.cuh:8-14 */
static v3 uniform_sphere(float sx, float sy)
{
    float sp, cp;
    orc_sincos_turns(sx, &sp, &cp);
    float cos_theta = sy * 2.0f - 1.0f;
    float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
    return mk(sin_theta * cp, sin_theta * sp, cos_theta);
}

/* ------------------------------------------------------------------------------------------ */
/* Classic BVH2: include/base/accel/bvh.h:66-154, include/cuda/accel/bvh.cuh:98-136,           */
/* include/cuda/accel/bvh2.cuh:12-88                                                           */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    v3 o;
    float mint;
    v3 d;
    float maxt;
} ray3;

static inline ray3 load_ray(const float *r)
{
    ray3 ray;
    ray.o = load3(r);
    ray.mint = r[3];
    ray.d = load3(r + 4);
    ray.maxt = r[7];
    return ray;
}

static inline v3 node_min(const uint32_t *node) { return mk(u2f(node[0]), u2f(node[1]), u2f(node[2])); }
static inline v3 node_max(const uint32_t *node) { return mk(u2f(node[4]), u2f(node[5]), u2f(node[6])); }

/* BVH2Node::intersect, bvh.h:121-133: entry distance inside (ray.mint, ray.maxt) or FLT_MAX */
static inline float box_entry(v3 bmin, v3 bmax, const ray3 *ray)
{
    v3 t0 = vdiv(vsub(bmin, ray->o), ray->d);
    v3 t1 = vdiv(vsub(bmax, ray->o), ray->d);
    v3 ts = vmin(t0, t1);
    v3 tb = vmax(t0, t1);
    float mint = gmax(ray->mint, cmax(ts));
    float maxt = gmin(ray->maxt, cmin(tb));
    return (mint <= maxt) ? mint : FLT_MAX;
}

/* BaseCudaBLAS::intersect_triangle, bvh.cuh:98-136 (Moller-Trumbore). Returns 1 on hit. */
static inline int tri_intersect(const orc_classic_scene *s, const ray3 *ray, uint32_t prim, float *t_out,
                                float *u_out, float *v_out)
{
    const uint32_t *ix = s->indices + 3u * prim;
    v3 v0 = load3(s->vertices + 3u * ix[0]);
    v3 v1 = load3(s->vertices + 3u * ix[1]);
    v3 v2 = load3(s->vertices + 3u * ix[2]);
    v3 e1 = vsub(v1, v0);
    v3 e2 = vsub(v2, v0);
    v3 pvec = vcross(ray->d, e2);
    float det = vdot(e1, pvec);
    if (det > -1e-8f && det < 1e-8f)
        return 0;
    float inv_det = 1.0f / det;
    v3 tvec = vsub(ray->o, v0);
    float u = vdot(tvec, pvec) * inv_det;
    if (u < 0.0f || u > 1.0f)
        return 0;
    v3 qvec = vcross(tvec, e1);
    float v = vdot(ray->d, qvec) * inv_det;
    if (v < 0.0f || (u + v) > 1.0f)
        return 0;
    float t = vdot(e2, qvec) * inv_det;
    if (t < ray->mint || t >= ray->maxt)
        return 0;
    *t_out = t;
    *u_out = u;
    *v_out = v;
    return 1;
}

/* CudaBVH2::intersect<ShadowRay>, bvh2.cuh:12-88. Fills t,u,v,prim (prim = UINT32_MAX on miss). */
static void classic_intersect(const orc_classic_scene *s, ray3 ray, int any_hit, float *t_o, float *u_o,
                              float *v_o, uint32_t *prim_o, uint32_t *boxes, uint32_t *tris)
{
    float best_t = FLT_MAX, best_u = 0.f, best_v = 0.f;
    uint32_t best_prim = 0xFFFFFFFFu;
    uint32_t stack[32];
    int sp = 0;
    uint32_t node_idx = 0;
    uint32_t nb = 0, nt = 0;
    for (;;) {
        const uint32_t *node = s->nodes + 8u * node_idx;
        if (node[3] > 0u) { /* leaf */
            uint32_t start = node[7], end = node[7] + node[3];
            int done = 0;
            for (uint32_t pid = start; pid < end; pid++) {
                uint32_t prim = s->prim_indices[pid];
                float t, u, v;
                nt++;
                if (tri_intersect(s, &ray, prim, &t, &u, &v) && t < ray.maxt) {
                    best_t = t;
                    best_u = u;
                    best_v = v;
                    best_prim = prim;
                    if (any_hit) {
                        done = 1;
                        break;
                    }
                    ray.maxt = t;
                }
            }
            if (done || sp == 0)
                break;
            node_idx = stack[--sp];
            continue;
        }
        uint32_t c1 = node[7], c2 = node[7] + 1u;
        const uint32_t *n1 = s->nodes + 8u * c1;
        const uint32_t *n2 = s->nodes + 8u * c2;
        float d1 = box_entry(node_min(n1), node_max(n1), &ray);
        float d2 = box_entry(node_min(n2), node_max(n2), &ray);
        nb += 2;
        if (d1 > d2) {
            float td = d1;
            d1 = d2;
            d2 = td;
            uint32_t tc = c1;
            c1 = c2;
            c2 = tc;
        }
        if (d1 == FLT_MAX) {
            if (sp == 0)
                break;
            node_idx = stack[--sp];
        } else {
            node_idx = c1;
            if (d2 != FLT_MAX)
                stack[sp++] = c2; /* depth of the build is below 32 (checked by the builder) */
        }
    }
    *t_o = best_t;
    *u_o = best_u;
    *v_o = best_v;
    *prim_o = best_prim;
    if (boxes)
        *boxes = nb;
    if (tris)
        *tris = nt;
}

typedef struct {
    const orc_classic_scene *scene;
    const float *rays;
    uint32_t begin, end;
    int any_hit;
    uint32_t *hits;
    uint32_t *stats;
} classic_job;

static void *classic_worker(void *arg)
{
    classic_job *j = (classic_job *)arg;
    for (uint32_t i = j->begin; i < j->end; i++) {
        float t, u, v;
        uint32_t prim, nb, nt;
        classic_intersect(j->scene, load_ray(j->rays + 8u * i), j->any_hit, &t, &u, &v, &prim, &nb, &nt);
        j->hits[4u * i + 0] = f2u(t);
        j->hits[4u * i + 1] = f2u(u);
        j->hits[4u * i + 2] = f2u(v);
        j->hits[4u * i + 3] = prim;
        if (j->stats) {
            j->stats[2u * i] = nb;
            j->stats[2u * i + 1] = nt;
        }
    }
    return NULL;
}

void orc_classic_query(const orc_classic_scene *scene, const float *rays, uint32_t n, int any_hit,
                       uint32_t *hits, uint32_t *stats, int n_threads)
{
    if (n_threads < 1)
        n_threads = 1;
    if (n_threads > 256)
        n_threads = 256;
    pthread_t th[256];
    classic_job jobs[256];
    uint32_t chunk = (n + (uint32_t)n_threads - 1u) / (uint32_t)n_threads;
    for (int k = 0; k < n_threads; k++) {
        uint32_t b = (uint32_t)k * chunk, e = b + chunk;
        if (b > n)
            b = n;
        if (e > n)
            e = n;
        jobs[k] = (classic_job){scene, rays, b, e, any_hit, hits, stats};
        if (n_threads == 1)
            classic_worker(&jobs[k]);
        else
            pthread_create(&th[k], NULL, classic_worker, &jobs[k]);
    }
    if (n_threads > 1)
        for (int k = 0; k < n_threads; k++)
            pthread_join(th[k], NULL);
}

void orc_fp64_closest(const orc_classic_scene *s, const float *rays, uint32_t n, double *t_out,
                      uint32_t *prim_out)
{
    for (uint32_t i = 0; i < n; i++) {
        const float *r = rays + 8u * i;
        double o[3] = {r[0], r[1], r[2]}, d[3] = {r[4], r[5], r[6]};
        double tmin = r[3], tmax = r[7];
        double best = 1e300;
        uint32_t bp = 0xFFFFFFFFu;
        for (uint32_t p = 0; p < s->n_triangles; p++) {
            const uint32_t *ix = s->indices + 3u * p;
            double v0[3], e1[3], e2[3];
            for (int k = 0; k < 3; k++) {
                v0[k] = s->vertices[3u * ix[0] + k];
                e1[k] = s->vertices[3u * ix[1] + k] - v0[k];
                e2[k] = s->vertices[3u * ix[2] + k] - v0[k];
            }
            double pv[3] = {d[1] * e2[2] - e2[1] * d[2], d[2] * e2[0] - e2[2] * d[0], d[0] * e2[1] - e2[0] * d[1]};
            double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
            if (det == 0.0)
                continue;
            double tv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
            double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) / det;
            if (u < 0.0 || u > 1.0)
                continue;
            double qv[3] = {tv[1] * e1[2] - e1[1] * tv[2], tv[2] * e1[0] - e1[2] * tv[0], tv[0] * e1[1] - e1[0] * tv[1]};
            double v = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) / det;
            if (v < 0.0 || u + v > 1.0)
                continue;
            double t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) / det;
            if (t < tmin || t >= tmax)
                continue;
            if (t < best || (t == best && p < bp)) {
                best = t;
                bp = p;
            }
        }
        t_out[i] = best;
        prim_out[i] = bp;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Neural BVH2: include/cuda/neural/accel/neural_bvh2.cuh                                      */
/* ------------------------------------------------------------------------------------------ */

#define ORC_NEURAL_STACK 24 /* NEURAL_STACK_SIZE, neural_bvh.cuh:22 */
#define NO_NEURAL_CHILD 0xFFFFFFFFu

/* dilated box: BVH2Node::bbox_center = min + extent * 0.5 (bvh.h:235-243) and
 * neural_bvh2.cuh:80-86 */
static inline void dilated_box(const uint32_t *node, float dil, v3 *bmin, v3 *bmax)
{
    v3 mn = node_min(node), mx = node_max(node);
    if (dil != 0.0f) {
        v3 ext = vsub(mx, mn);
        v3 center = vadd(mn, vscale(ext, 0.5f));
        v3 next = vscale(ext, 1.0f + dil);
        *bmin = vsub(center, vscale(next, 0.5f));
        *bmax = vadd(center, vscale(next, 0.5f));
    } else {
        *bmin = mn;
        *bmax = mx;
    }
}

/* intersect_bbox_min_max without ray bounds (ray.cuh:111-132 / bvh.h:137-154) */
static inline int slab_min_max(v3 bmin, v3 bmax, v3 o, v3 d, float *mint, float *maxt)
{
    v3 t0 = vdiv(vsub(bmin, o), d);
    v3 t1 = vdiv(vsub(bmax, o), d);
    *mint = cmax(vmin(t0, t1));
    *maxt = cmin(vmax(t0, t1));
    return *mint <= *maxt;
}

/* intersect_traversal_bbox, neural_bvh2.cuh:94-115 (check_ray_bounds = true) */
static inline float traversal_entry(const uint32_t *node, float dil, v3 o, v3 d, float rmint, float rmaxt)
{
    v3 bmin, bmax;
    dilated_box(node, dil, &bmin, &bmax);
    v3 t0 = vdiv(vsub(bmin, o), d);
    v3 t1 = vdiv(vsub(bmax, o), d);
    float mint = gmax(rmint, cmax(vmin(t0, t1)));
    float maxt = gmin(rmaxt, cmin(vmax(t0, t1)));
    return (mint <= maxt) ? mint : FLT_MAX;
}

static inline int is_leaf_at_lod(const uint32_t *node, uint32_t lod) /* neural_bvh2.cuh:124-128 */
{
    return node[3] > 0u && node[3] <= 2u + lod;
}

/* NeuralBVH2::intersect, neural_bvh2.cuh:170-292. Returns 1 with the next entered leaf segment,
 * 0 when the stack is exhausted, -1 on stack overflow (the reference prints and returns false). */
static int neural_intersect(const uint32_t *nodes, uint32_t lod, v3 o, v3 d, uint32_t *stack, int *sp,
                            int inference, const orc_neural_consts *c, float current_maxt, float dil,
                            float *seg_mint, float *seg_maxt, uint32_t *seg_node)
{
    const float rmint = -FLT_MAX, rmaxt = current_maxt;
    uint32_t node_idx = stack[--(*sp)];
    for (;;) {
        const uint32_t *node = nodes + 8u * node_idx;
        if (is_leaf_at_lod(node, lod) || node[7] == NO_NEURAL_CHILD) {
            v3 bmin, bmax;
            float mint, maxt;
            dilated_box(node, dil, &bmin, &bmax);
            if (slab_min_max(bmin, bmax, o, d, &mint, &maxt)) {
                float maxt_eps = inference ? c->inference_maxt_epsilon : c->learning_maxt_epsilon;
                float mint_eps = inference ? c->inference_mint_epsilon : c->learning_mint_epsilon;
                int valid = mint < rmaxt;
                if (mint < 0.0f)
                    valid &= maxt > maxt_eps;
                else
                    valid &= mint > mint_eps;
                if (valid) {
                    *seg_mint = mint;
                    *seg_maxt = maxt;
                    *seg_node = node_idx;
                    return 1;
                }
            }
            if (*sp == 0)
                return 0;
            node_idx = stack[--(*sp)];
            continue;
        }
        uint32_t c1 = node[7], c2 = node[7] + 1u;
        float d1 = traversal_entry(nodes + 8u * c1, dil, o, d, rmint, rmaxt);
        float d2 = traversal_entry(nodes + 8u * c2, dil, o, d, rmint, rmaxt);
        if (d1 > d2) {
            float td = d1;
            d1 = d2;
            d2 = td;
            uint32_t tc = c1;
            c1 = c2;
            c2 = tc;
        }
        if (d1 == FLT_MAX) {
            if (*sp == 0)
                return 0;
            node_idx = stack[--(*sp)];
        } else {
            node_idx = c1;
            if (d2 != FLT_MAX) {
                stack[(*sp)++] = c2;
                if (*sp >= ORC_NEURAL_STACK)
                    return -1;
            }
        }
    }
}

void orc_neural_segments(const uint32_t *nodes, const orc_neural_consts *c, const float *rays, uint32_t n,
                         uint32_t max_segments, uint32_t *segs, uint32_t *counts)
{
    for (uint32_t i = 0; i < n; i++) {
        ray3 r = load_ray(rays + 8u * i);
        uint32_t stack[ORC_NEURAL_STACK];
        int sp = 1;
        stack[0] = 0;
        uint32_t cnt = 0;
        while (sp > 0) {
            float mint, maxt;
            uint32_t nd;
            int res = neural_intersect(nodes, c->bvh_lod, r.o, r.d, stack, &sp, 1, c, FLT_MAX,
                                       c->fixed_node_dilation, &mint, &maxt, &nd);
            if (res != 1)
                break;
            if (cnt < max_segments) {
                uint32_t *s = segs + 4u * ((size_t)i * max_segments + cnt);
                s[0] = f2u(mint);
                s[1] = f2u(maxt);
                s[2] = nd;
                s[3] = 0;
            }
            cnt++;
        }
        counts[i] = cnt;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* FP16                                                                                       */
/* ------------------------------------------------------------------------------------------ */

uint16_t orc_f32_to_f16(float f) /* IEEE binary16, round to nearest even */
{
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t absx = x & 0x7FFFFFFFu;
    if (absx >= 0x7F800000u) /* inf or nan */
        return (uint16_t)(sign | 0x7C00u | (absx > 0x7F800000u ? 0x200u : 0u));
    if (absx >= 0x477FF000u) /* >= 65520 rounds to inf */
        return (uint16_t)(sign | 0x7C00u);
    if (absx < 0x38800000u) { /* below the smallest normal 2^-14: subnormal or zero */
        if (absx < 0x33000000u) /* < 2^-25 rounds to zero */
            return (uint16_t)sign;
        uint32_t mant = (absx & 0x7FFFFFu) | 0x800000u;
        int e = (int)(absx >> 23); /* biased */
        int shift = 126 - e;       /* value = mant * 2^(e-150); half subnormal unit 2^-24 */
        /* result = mant * 2^(e-150) / 2^-24 = mant >> (126 - e) */
        uint32_t q = mant >> shift;
        uint32_t rem = mant & ((1u << shift) - 1u);
        uint32_t halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (q & 1u)))
            q++;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (absx >> 23) - 112u; /* rebias 127 -> 15 */
    uint32_t mant = absx & 0x7FFFFFu;
    uint32_t q = (e << 10) | (mant >> 13);
    uint32_t rem = mant & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u)))
        q++;
    return (uint16_t)(sign | q);
}

float orc_f16_to_f32(uint16_t h)
{
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = ((uint32_t)h >> 10) & 0x1Fu;
    uint32_t m = (uint32_t)h & 0x3FFu;
    if (e == 0) {
        float v = (float)m * 0x1p-24f;
        return sign ? -v : v;
    }
    if (e == 31)
        return u2f(sign | 0x7F800000u | (m << 13));
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

static inline float round_f16(float x) { return orc_f16_to_f32(orc_f32_to_f16(x)); }

/* bfloat16: the upper 16 bits of the binary32 value, rounded to nearest even (finite inputs) */
uint16_t orc_f32_to_bf16(float f)
{
    uint32_t u = f2u(f);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
float orc_bf16_to_f32(uint16_t b) { return u2f((uint32_t)b << 16); }
static inline float round_bf16(float x) { return orc_bf16_to_f32(orc_f32_to_bf16(x)); }

/* rounding of an MLP operand in the network's precision */
static inline float round_mlp(const orc_network *net, float x) { return net->bf16 ? round_bf16(x) : round_f16(x); }

/* FP8 E4M3: 4 exponent bits (bias 7), 3 mantissa bits, max 448, no infinity */
float orc_e4m3_round(float x)
{
    uint32_t b = f2u(x);
    const uint32_t sign = b & 0x80000000u;
    uint32_t a = b & 0x7FFFFFFFu;
    if (a > 0x7F800000u)
        return x;
    float r;
    if (a >= 0x43E00000u) {
        r = u2f(0x43E00000u);
    } else if (a < 0x3C800000u) {
        r = rintf(u2f(a) * 512.0f) * (1.0f / 512.0f);
    } else {
        const uint32_t lsb = (a >> 20) & 1u;
        a = (a + 0x7FFFFu + lsb) & 0xFFF00000u;
        if (a > 0x43E00000u)
            a = 0x43E00000u;
        r = u2f(a);
    }
    return u2f(f2u(r) | sign);
}

/* index range of the hidden 64x64 matrices in the network parameters */
static inline int fp8_weight(const orc_network *net, size_t i)
{
    const size_t lo = (size_t)net->n_neurons * net->n_inputs;
    const size_t hi = lo + (size_t)(net->n_hidden_layers - 1u) * net->n_neurons * net->n_neurons;
    return net->fp8 && i >= lo && i < hi;
}
static inline float net_round(const orc_network *net, float x) { return net->exact ? x : round_mlp(net, x); }
static inline float net_w(const orc_network *net, size_t i)
{
    if (net->exact)
        return net->weights_f32[i];
    if (fp8_weight(net, i))
        return orc_e4m3_round(net->weights_f32[i] * 64.0f) * (1.0f / 64.0f);
    return net->bf16 ? orc_bf16_to_f32(net->weights_f16[i]) : orc_f16_to_f32(net->weights_f16[i]);
}
static inline float net_g(const orc_network *net, size_t i)
{
    return net->exact ? net->grid_f32[i] : orc_f16_to_f32(net->grid_f16[i]);
}

/* ------------------------------------------------------------------------------------------ */
/* Multiresolution hash grid (tcnn GridEncoding behaviour; Muller et al. 2022, Instant NGP)    */
/* ------------------------------------------------------------------------------------------ */

/* Level l (tcnn grid_scale): scale = exp2f(l * log2f(per_level_scale)) * base_resolution - 1 in
 * single precision, resolution = ceil(scale) + 1, entries = min(roundup8(res^3), 2^log2T). */
void orc_grid_layout(uint32_t n_levels, uint32_t log2_hashmap_size, uint32_t base_resolution,
                     float per_level_scale, uint32_t *offset, uint32_t *size, uint32_t *resolution,
                     float *scale, uint32_t *total_entries)
{
    uint64_t off = 0;
    uint64_t hashmap = 1ull << log2_hashmap_size;
    const float log2_scale = log2f(per_level_scale);
    for (uint32_t l = 0; l < n_levels; l++) {
        const float grow = exp2f((float)l * log2_scale);
        float s = grow * (float)base_resolution - 1.0f;
        uint32_t res = (uint32_t)ceilf(s) + 1u;
        uint64_t dense = (uint64_t)res * res * res;
        dense = (dense + 7u) & ~7ull;
        uint64_t sz = dense < hashmap ? dense : hashmap;
        offset[l] = (uint32_t)off;
        size[l] = (uint32_t)sz;
        resolution[l] = res;
        scale[l] = s;
        off += sz;
    }
    *total_entries = (uint32_t)off;
}

/* grid_index: dense index x + y*res + z*res^2 while res^3 fits the level, else the coherent prime
 * hash x*1 ^ y*2654435761 ^ z*805459861; both modulo the level size. */
static inline uint32_t grid_index(uint32_t level_size, uint32_t res, uint32_t x, uint32_t y, uint32_t z)
{
    uint64_t dense = (uint64_t)res * res * res;
    uint32_t idx;
    if (dense <= (uint64_t)level_size)
        idx = x + y * res + z * res * res;
    else
        idx = x ^ (y * 2654435761u) ^ (z * 805459861u);
    return idx % level_size;
}

/* number of features per level (entries hold that many FP16 values); 2 when unset */
static inline uint32_t net_features(const orc_network *net) { return net->n_features ? net->n_features : 2u; }

/* features of one point for one level (F values), fused multiply-add accumulation over the 8
 * corners in order c = 0..7 (bit d of c selects the upper corner along axis d), feature f of
 * corner c accumulated as f_acc = fma(w_c, entry_c[f], f_acc) */
static void encode_level(const orc_network *net, uint32_t l, v3 p, float *f, uint32_t *cidx, float *cw)
{
    const uint32_t F = net_features(net);
    float s = net->level_scale[l];
    float pos[3] = {fmaf(p.x, s, 0.5f), fmaf(p.y, s, 0.5f), fmaf(p.z, s, 0.5f)};
    uint32_t g[3];
    float fr[3];
    for (int d = 0; d < 3; d++) {
        float fl = floorf(pos[d]);
        g[d] = (uint32_t)(int32_t)fl;
        fr[d] = pos[d] - fl;
    }
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (uint32_t c = 0; c < 8; c++) {
        float wx = (c & 1u) ? fr[0] : 1.0f - fr[0];
        float wy = (c & 2u) ? fr[1] : 1.0f - fr[1];
        float wz = (c & 4u) ? fr[2] : 1.0f - fr[2];
        float w = (wx * wy) * wz;
        uint32_t idx = grid_index(net->level_size[l], net->level_resolution[l], g[0] + (c & 1u),
                                  g[1] + ((c >> 1) & 1u), g[2] + ((c >> 2) & 1u));
        uint32_t e = net->level_offset[l] + idx;
        for (uint32_t k = 0; k < F; k++)
            acc[k] = fmaf(w, net_g(net, (size_t)F * e + k), acc[k]);
        if (cidx) {
            cidx[c] = e;
            cw[c] = w;
        }
    }
    for (uint32_t k = 0; k < F; k++)
        f[k] = acc[k];
}

/* features of one point: level l's F values at l * F (tcnn GridEncoding output order) */
static void encode_point(const orc_network *net, v3 p, float *f, uint32_t (*cidx)[8], float (*cw)[8])
{
    const uint32_t F = net_features(net);
    for (uint32_t l = 0; l < net->n_levels; l++)
        encode_level(net, l, p, f + (size_t)F * l, cidx ? cidx[l] : NULL, cw ? cw[l] : NULL);
}

void orc_encode(const orc_network *net, const float *positions, uint32_t n, float *features)
{
    const uint32_t F = net_features(net);
    for (uint32_t i = 0; i < n; i++)
        for (uint32_t k = 0; k < net->n_points; k++) {
            v3 p = load3(positions + 3u * ((size_t)i * net->n_points + k));
            encode_point(net, p, features + (size_t)i * net->n_inputs + (size_t)k * net->n_levels * F, NULL, NULL);
        }
}

/* offsets of the network matrices in the parameter vector */
static void matrix_offsets(const orc_network *net, uint32_t *off, uint32_t *rows, uint32_t *cols, uint32_t *n_mat)
{
    uint32_t nm = net->n_hidden_layers + 1u, o = 0;
    for (uint32_t m = 0; m < nm; m++) {
        rows[m] = (m == nm - 1u) ? 16u : net->n_neurons;
        cols[m] = (m == 0) ? net->n_inputs : net->n_neurons;
        off[m] = o;
        o += rows[m] * cols[m];
    }
    *n_mat = nm;
}

/* forward of one row: x (FP16-rounded features) -> outputs (16, sigmoid). acts (optional) receives
 * the FP16 activations entering every layer (n_mat x 128 max) and pre (optional) the output
 * pre-activations. */
static void mlp_row(const orc_network *net, const float *x_in, float *out, float *acts, double *pre_out)
{
    uint32_t off[16], rows[16], cols[16], nm;
    matrix_offsets(net, off, rows, cols, &nm);
    float a[128], b[128];
    for (uint32_t i = 0; i < net->n_inputs; i++)
        a[i] = net_round(net, x_in[i]);
    for (uint32_t m = 0; m < nm; m++) {
        if (acts)
            memcpy(acts + 128u * m, a, sizeof(float) * cols[m]);
        for (uint32_t r = 0; r < rows[m]; r++) {
            double acc = 0.0;
            const size_t wo = off[m] + (size_t)r * cols[m];
            for (uint32_t k = 0; k < cols[m]; k++)
                acc += (double)net_w(net, wo + k) * (double)a[k];
            if (m == nm - 1u) {
                if (pre_out)
                    pre_out[r] = acc;
                out[r] = (float)(1.0 / (1.0 + exp(-acc)));
            } else if (net->fp8 && !net->exact && m + 2u < nm) {
                /* input of a hidden matrix (m + 1 <= nm - 2) in FP8 mode */
                b[r] = orc_e4m3_round((acc > 0.0 ? (float)acc : 0.0f) * 128.0f) * (1.0f / 128.0f);
            } else {
                b[r] = net_round(net, acc > 0.0 ? (float)acc : 0.0f);
            }
        }
        if (m != nm - 1u)
            memcpy(a, b, sizeof(float) * rows[m]);
    }
}

typedef struct {
    const orc_network *net;
    const float *positions;
    float *outputs;
    uint32_t begin, end;
} infer_job;

static void *infer_worker(void *arg)
{
    infer_job *j = (infer_job *)arg;
    float feat[128];
    for (uint32_t i = j->begin; i < j->end; i++) {
        orc_encode(j->net, j->positions + (size_t)i * j->net->n_points * 3u, 1, feat);
        mlp_row(j->net, feat, j->outputs + 16u * (size_t)i, NULL, NULL);
    }
    return NULL;
}

void orc_network_inference(const orc_network *net, const float *positions, uint32_t n, float *outputs,
                           int n_threads)
{
    if (n_threads < 1)
        n_threads = 1;
    if (n_threads > 256)
        n_threads = 256;
    pthread_t th[256];
    infer_job jobs[256];
    uint32_t chunk = (n + (uint32_t)n_threads - 1u) / (uint32_t)n_threads;
    for (int k = 0; k < n_threads; k++) {
        uint32_t b = (uint32_t)k * chunk, e = b + chunk;
        if (b > n)
            b = n;
        if (e > n)
            e = n;
        jobs[k] = (infer_job){net, positions, outputs, b, e};
        if (n_threads == 1)
            infer_worker(&jobs[k]);
        else
            pthread_create(&th[k], NULL, infer_worker, &jobs[k]);
    }
    if (n_threads > 1)
        for (int k = 0; k < n_threads; k++)
            pthread_join(th[k], NULL);
}

/* ------------------------------------------------------------------------------------------ */
/* Segment encoding: src/cuda/neural/neural_bvh_module_kernels.cu:10-97, 266-303              */
/* ------------------------------------------------------------------------------------------ */

static void encode_segment(const orc_neural_scene *sc, const orc_neural_consts *c, v3 wpo, v3 wpi,
                           uint32_t *rng, float *pts)
{
    v3 smin = load3(sc->scene_min), smax = load3(sc->scene_max);
    float dilation = 1.0f + c->node_extent_dilation + c->fixed_node_dilation;
    v3 ext = vscale(vsub(smax, smin), dilation);
    v3 center = vscale(vadd(smax, smin), 0.5f);
    v3 epo = vadds(vdiv(vsub(wpo, center), ext), 0.5f);
    v3 epi = vadds(vdiv(vsub(wpi, center), ext), 0.5f);
    int np = c->input_segment_points;
    float delta, offset;
    if (c->segment_distribution == 1) { /* EquidistantExterior */
        delta = 1.0f / (float)(np - 1);
        offset = 0.0f;
        if (np == 1)
            delta = 1.0f;
    } else {
        delta = 1.0f / (float)np;
        offset = 0.5f;
    }
    for (int k = 0; k < np; k++) {
        float t = (c->segment_distribution == 2) ? orc_lcg_randomf(rng) : delta * ((float)k + offset);
        v3 p = vadd(vscale(epo, 1.0f - t), vscale(epi, t));
        pts[3 * k + 0] = p.x;
        pts[3 * k + 1] = p.y;
        pts[3 * k + 2] = p.z;
    }
}

static inline v3 ray_at(v3 o, v3 d, float t) { return vadd(o, vscale(d, t)); }

/* decode_depth_estimate, LocalT branch, neural_bvh_module_common.cuh:23-58 */
static float decode_local_t(const orc_neural_consts *c, float out_depth, float mint, float maxt, int inside)
{
    float seg_len = maxt - mint;
    float u = gclamp01(out_depth);
    float depth = FLT_MAX;
    if (inside) {
        if (c->depth_epsilon != 1.0f) {
            float inward = (float)((double)u * ((double)seg_len + 1e-3));
            if (inward < maxt - seg_len * c->depth_epsilon - c->fixed_depth_epsilon)
                depth = maxt - inward;
        }
    } else {
        depth = (float)((double)u * ((double)seg_len + 1e-3) + (double)mint);
    }
    return depth;
}

float orc_decode_local_t(float out_depth, float mint, float maxt, int inside, float depth_epsilon,
                         float fixed_depth_epsilon)
{
    orc_neural_consts c;
    memset(&c, 0, sizeof(c));
    c.depth_epsilon = depth_epsilon;
    c.fixed_depth_epsilon = fixed_depth_epsilon;
    return decode_local_t(&c, out_depth, mint, maxt, inside);
}

typedef struct {
    const orc_neural_scene *scene;
    const orc_network *net;
    const orc_neural_consts *c;
    const orc_classic_scene *classic;
    float margin;
    const float *rays;
    uint32_t begin, end, depth;
    int vis_only;
    uint32_t *hits;
} nq_job;

static void neural_query_one(const nq_job *j, uint32_t i)
{
    const orc_neural_consts *c = j->c;
    ray3 r = load_ray(j->rays + 8u * i);
    uint32_t *h = j->hits + 12u * (size_t)i;
    float best_t = r.maxt; /* init_neural_traversal_result(current_t) */
    int valid = 0;
    v3 normal = mk(0, 0, 0), albedo = mk(0, 0, 0);
    float vis_acc = 0.0f;
    uint32_t flags = 0, segments = 0;
    int fallback = 0;
    uint32_t rng = orc_lcg_seed(0u, 0u, i);

    uint32_t stack[ORC_NEURAL_STACK];
    int sp = 1;
    stack[0] = 0;
    float mint, maxt;
    uint32_t node;
    int res = neural_intersect(j->scene->neural_nodes, c->bvh_lod, r.o, r.d, stack, &sp, 1, c, FLT_MAX,
                               c->fixed_node_dilation, &mint, &maxt, &node);
    float thr = j->depth == 1u ? c->primary_visibility_threshold : c->secondary_visibility_threshold;
    uint32_t step = 0;
    while (res == 1) {
        if (j->scene->non_neural && j->scene->non_neural[node]) {
            fallback = 1;
            break;
        }
        if (step > c->max_traversal_steps) {
            flags |= 0x4u;
            break;
        }
        step++;
        /* encode_bvh_network_input_data: swap for a negative mint (kernels.cu:281-286) */
        float a = mint, b = maxt;
        if (a < 0.0f) {
            float t = a;
            a = b;
            b = t;
        }
        float pts[3 * 16], feat[128], out[16];
        encode_segment(j->scene, c, ray_at(r.o, r.d, a), ray_at(r.o, r.d, b), &rng, pts);
        for (int k = 0; k < c->input_segment_points; k++)
            encode_point(j->net, load3(pts + 3 * k), &feat[(size_t)k * j->net->n_levels * net_features(j->net)],
                         NULL, NULL);
        mlp_row(j->net, feat, out, NULL, NULL);
        segments++;
        if (j->margin > 0.0f && fabsf(out[0] - thr) < j->margin) {
            fallback = 1;
            break;
        }
        /* process_neural_bvh_traversal_step, path_inference_kernels.cu:61-131 */
        float new_depth = best_t;
        int stop = 0;
        if (out[0] > thr) {
            int inside = mint < 0.0f;
            if (j->vis_only && !inside) {
                valid = 1;
                vis_acc = out[0];
                stop = 1;
            } else {
                float de = decode_local_t(c, out[1], mint, maxt, inside);
                if (de != FLT_MAX) {
                    if (j->vis_only) {
                        valid = 1;
                        vis_acc = out[0];
                        stop = 1;
                    } else if (de < best_t) {
                        valid = 1;
                        best_t = de;
                        new_depth = de;
                        vis_acc = out[0];
                        normal = vnormalize(mk(out[2] * 2.0f - 1.0f, out[3] * 2.0f - 1.0f, out[4] * 2.0f - 1.0f));
                        albedo = mk(out[5], out[6], out[7]);
                    }
                }
            }
        }
        if (stop)
            break;
        /* process_bvh_network_output_and_intersect_neural_bvh, common.cuh:496-550 */
        if (sp == 0)
            break;
        res = neural_intersect(j->scene->neural_nodes, c->bvh_lod, r.o, r.d, stack, &sp, 1, c, new_depth,
                               c->fixed_node_dilation, &mint, &maxt, &node);
    }
    if (res == -1)
        flags |= 0x8u;
    if (fallback && j->classic) {
        float t, u, v;
        uint32_t prim;
        ray3 cr = r;
        classic_intersect(j->classic, cr, j->vis_only, &t, &u, &v, &prim, NULL, NULL);
        h[0] = f2u(t);
        for (int k = 1; k < 8; k++)
            h[k] = 0;
        h[8] = (prim != 0xFFFFFFFFu ? 0x1u : 0u) | 0x2u | flags;
        h[9] = segments;
        h[10] = prim;
        h[11] = 0;
        return;
    }
    if (!valid)
        best_t = FLT_MAX;
    h[0] = f2u(valid ? best_t : FLT_MAX);
    h[1] = f2u(normal.x);
    h[2] = f2u(normal.y);
    h[3] = f2u(normal.z);
    h[4] = f2u(albedo.x);
    h[5] = f2u(albedo.y);
    h[6] = f2u(albedo.z);
    h[7] = f2u(valid ? vis_acc : 0.0f);
    h[8] = (valid ? 0x1u : 0u) | flags;
    h[9] = segments;
    h[10] = 0xFFFFFFFFu;
    h[11] = 0;
}

static void *nq_worker(void *arg)
{
    nq_job *j = (nq_job *)arg;
    for (uint32_t i = j->begin; i < j->end; i++)
        neural_query_one(j, i);
    return NULL;
}

void orc_neural_query(const orc_neural_scene *scene, const orc_network *net, const orc_neural_consts *c,
                      const orc_classic_scene *classic, float fallback_margin, const float *rays, uint32_t n,
                      uint32_t depth, int visibility_only, uint32_t *hits, int n_threads)
{
    if (n_threads < 1)
        n_threads = 1;
    if (n_threads > 256)
        n_threads = 256;
    pthread_t th[256];
    nq_job jobs[256];
    uint32_t chunk = (n + (uint32_t)n_threads - 1u) / (uint32_t)n_threads;
    for (int k = 0; k < n_threads; k++) {
        uint32_t b = (uint32_t)k * chunk, e = b + chunk;
        if (b > n)
            b = n;
        if (e > n)
            e = n;
        jobs[k] = (nq_job){scene, net, c, classic, fallback_margin, rays, b, e, depth, visibility_only, hits};
        if (n_threads == 1)
            nq_worker(&jobs[k]);
        else
            pthread_create(&th[k], NULL, nq_worker, &jobs[k]);
    }
    if (n_threads > 1)
        for (int k = 0; k < n_threads; k++)
            pthread_join(th[k], NULL);
}

/* ------------------------------------------------------------------------------------------ */
/* Training samples: neural_bvh_module_kernels.cu:119-264 (n_sub_batch = 1),                  */
/* stack_based_sample_uniform_bvh_density common.cuh:703-781, sample_bbox_position 635-660,    */
/* generate_single_bvh_network_output_reference 783-861, compute_depth_or_position_output      */
/* 586-629 (LocalT)                                                                             */
/* ------------------------------------------------------------------------------------------ */

static v3 cube_pos_on_face(int face, float u, float v) /* sampling.cuh:85-94 */
{
    switch (face) {
    case 0: return mk(1.0f, u, v);
    case 1: return mk(0.0f, u, v);
    case 2: return mk(u, 1.0f, v);
    case 3: return mk(u, 0.0f, v);
    case 4: return mk(u, v, 1.0f);
    default: return mk(u, v, 0.0f);
    }
}

/* NeuralTreeCutData::compute_loss_heuristic, include/cuda/neural/neural_bvh_renderer.h:36-47 */
float orc_loss_heuristic(const uint32_t *stats)
{
    float loss;
    memcpy(&loss, stats, 4);
    const uint32_t alive = stats[1], samples = stats[3];
    if (samples == 0u)
        return -FLT_MAX;
    return loss / ((float)alive * sqrtf((float)samples / (float)alive));
}

void orc_generate_training_batch(const orc_neural_scene *sc, const orc_classic_scene *classic,
                                 const float *albedo, const orc_neural_consts *c, uint32_t training_step,
                                 uint32_t batch_size, uint32_t n, float *positions, float *targets,
                                 uint32_t *nodes_out)
{
    orc_generate_training_batch_rr(sc, classic, albedo, c, training_step, batch_size, n, positions, targets,
                                   nodes_out, NULL);
}

void orc_generate_training_batch_rr(const orc_neural_scene *sc, const orc_classic_scene *classic,
                                    const float *albedo, const orc_neural_consts *c, uint32_t training_step,
                                    uint32_t batch_size, uint32_t n, float *positions, float *targets,
                                    uint32_t *nodes_out, const orc_node_survival *rr)
{
    v3 smin = load3(sc->scene_min), smax = load3(sc->scene_max);
    const uint32_t *nodes = sc->neural_nodes;
    const uint32_t learned_lod = rr ? rr->current_learned_lod : ORC_NUM_BVH_LODS - 1u;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t rng = orc_lcg_seed(training_step * batch_size, 0u, i);
        /* stack_based_sample_uniform_bvh_density */
        float sx = orc_lcg_randomf(&rng);
        float sy = orc_lcg_randomf(&rng);
        v3 dir = uniform_sphere(sx, sy);
        /* sampled LoD among the ones learned so far (common.cuh:719-721) */
        const uint32_t n_lods = ORC_NUM_BVH_LODS - learned_lod;
        uint32_t lod_pick = (uint32_t)(orc_lcg_randomf(&rng) * (float)n_lods);
        const uint32_t sampled_lod = learned_lod + (lod_pick < n_lods - 1u ? lod_pick : n_lods - 1u);
        float dil = c->fixed_node_dilation + orc_lcg_randomf(&rng) * c->node_extent_dilation;
        uint32_t stack[ORC_NEURAL_STACK];
        int sp = 0;
        int valid = 0;
        v3 o = mk(0, 0, 0), d = dir;
        float mint = 0.f, maxt = 0.f;
        uint32_t node = 0;
        uint32_t guard = 0;
        do {
            if (!valid) {
                stack[0] = 0;
                sp = 1;
                float px = orc_lcg_randomf(&rng);
                float py = orc_lcg_randomf(&rng);
                float pz = orc_lcg_randomf(&rng);
                v3 ps = vsub(vscale(mk(px, py, pz), c->sampling_bbox_scaling),
                             mk((c->sampling_bbox_scaling - 1.0f) * 0.5f, (c->sampling_bbox_scaling - 1.0f) * 0.5f,
                                (c->sampling_bbox_scaling - 1.0f) * 0.5f));
                o = vadd(vmul(ps, vsub(smax, smin)), smin); /* Bbox::local_to_bbox, bbox.h:93-97 */
                d = dir;
            }
            int res = neural_intersect(nodes, sampled_lod, o, d, stack, &sp, 0, c, FLT_MAX, dil, &mint, &maxt, &node);
            valid = (res == 1);
            if (res == -1)
                sp = 0;
        } while (!valid && ++guard < 100000u);
        if (c->leaf_boundary_sampling_ratio != 0.0f &&
            orc_lcg_randomf(&rng) <= c->leaf_boundary_sampling_ratio) {
            /* sample_bbox_position, common.cuh:635-660 */
            int f1 = (int)(orc_lcg_randomf(&rng) * 6.0f);
            f1 = f1 < 5 ? f1 : 5;
            int f2;
            do {
                f2 = (int)(orc_lcg_randomf(&rng) * 6.0f);
                f2 = f2 < 5 ? f2 : 5;
            } while (f1 == f2);
            float u1 = orc_lcg_randomf(&rng), v1 = orc_lcg_randomf(&rng);
            v3 lp1 = cube_pos_on_face(f1, u1, v1);
            float u2 = orc_lcg_randomf(&rng), v2 = orc_lcg_randomf(&rng);
            v3 lp2 = cube_pos_on_face(f2, u2, v2);
            const uint32_t *nd = nodes + 8u * node;
            v3 mn = node_min(nd), mx = node_max(nd);
            v3 ext = vsub(mx, mn);
            v3 center = vadd(mn, vscale(ext, 0.5f));
            v3 next = vscale(ext, 1.0f + dil);
            v3 nmin = vsub(center, vscale(next, 0.5f));
            v3 entry = vadd(nmin, vmul(lp1, next));
            v3 exitp = vadd(nmin, vmul(lp2, next));
            o = entry;
            d = vnormalize(vsub(exitp, entry));
            mint = 0.0f;
            maxt = vlength(vsub(exitp, entry));
        }
        if (nodes_out)
            nodes_out[i] = node;
        if (rr && rr->enabled) {
            /* node survival (neural_bvh_module_kernels.cu:184-199): a rejected sample leaves its
             * slot's previous input and target in place; its node index is already written */
            const float estimate = orc_loss_heuristic(rr->stats + 4u * node);
            float kept = fmaxf(rr->min_survival_prob, estimate / rr->current_max_loss);
            if (!(estimate <= rr->current_max_loss))
                kept = 1.0f;
            if (rr->survival_probability_scale * kept < orc_lcg_randomf(&rng))
                continue;
        }
        float pts[48];
        encode_segment(sc, c, ray_at(o, d, mint), ray_at(o, d, maxt), &rng, pts);
        memcpy(positions + (size_t)i * 3u * (uint32_t)c->input_segment_points, pts,
               sizeof(float) * 3u * (uint32_t)c->input_segment_points);
        /* labels from the classic BLAS on [mint, maxt] */
        ray3 lr;
        lr.o = o;
        lr.d = d;
        lr.mint = mint;
        lr.maxt = maxt;
        float t, u, v;
        uint32_t prim;
        classic_intersect(classic, lr, 0, &t, &u, &v, &prim, NULL, NULL);
        float *tg = targets + 8u * (size_t)i;
        int hit = t != FLT_MAX;
        tg[0] = hit ? 1.0f : 0.0f;
        tg[1] = hit ? (float)((double)(t - mint) / ((double)(maxt - mint) + 1e-3)) : 0.0f;
        if (hit) {
            const uint32_t *ix = classic->indices + 3u * prim;
            v3 v0 = load3(classic->vertices + 3u * ix[0]);
            v3 va = load3(classic->vertices + 3u * ix[1]);
            v3 vb = load3(classic->vertices + 3u * ix[2]);
            v3 gn = vnormalize(vcross(vsub(va, v0), vsub(vb, v0))); /* compute_its_data, bvh.cuh:69 */
            v3 nn = vscale(vadds(gn, 1.0f), 0.5f);
            tg[2] = nn.x;
            tg[3] = nn.y;
            tg[4] = nn.z;
            if (albedo) {
                tg[5] = albedo[3u * prim];
                tg[6] = albedo[3u * prim + 1u];
                tg[7] = albedo[3u * prim + 2u];
            } else {
                tg[5] = tg[6] = tg[7] = 0.9f;
            }
        } else {
            for (int k = 2; k < 8; k++)
                tg[k] = 0.0f;
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Loss: include/cuda/neural/utils/loss_gradient.cuh:25-94, pt_composite_loss.cuh:18-123       */
/* ------------------------------------------------------------------------------------------ */

static void loss_and_gradient(int type, float target, float pred, float *loss, float *grad)
{
    switch (type) {
    case 0: { /* RelativeL2 */
        float diff = pred - target;
        float denom = pred * pred + 1e-2f;
        *loss = diff * diff / denom;
        *grad = 2.0f * diff / denom;
        break;
    }
    case 2: { /* RelativeL1 */
        float scale = 1.0f / (fabsf(pred) + 1e-2f);
        float diff = pred - target;
        *loss = fabsf(diff) * scale;
        *grad = copysignf(scale, diff);
        break;
    }
    case 3: { /* L1 */
        float diff = pred - target;
        *loss = fabsf(diff);
        *grad = copysignf(1.0f, diff);
        break;
    }
    case 5: { /* BinaryCrossEntropy */
        const float eps = 1e-5f;
        float p = fminf(fmaxf(pred, eps), 1.0f - eps);
        *loss = -(target * logf(p) + (1.0f - target) * logf(1.0f - p));
        *grad = -(target - p) / (p - (p * p));
        break;
    }
    case 6: { /* LogL2 */
        float diff = logf(1.0f + pred) - logf(1.0f + target);
        *loss = diff * diff;
        *grad = 2.0f * diff / (pred + 1.0f);
        break;
    }
    case 7: { /* LHalf */
        float sd = sqrtf(fabsf(pred - target));
        *loss = sd;
        *grad = 1.0f / (2.0f * sd + 1e-5f);
        break;
    }
    default: { /* L2 */
        float diff = pred - target;
        *loss = diff * diff;
        *grad = 2.0f * diff;
        break;
    }
    }
}

void orc_composite_loss(const orc_loss_consts *lc, const float *predictions, const float *targets, uint32_t n,
                        float loss_scale, float *values, float *gradients)
{
    uint32_t dims = 2u + (lc->learn_normal ? 3u : 0u) + (lc->learn_albedo ? 3u : 0u);
    float n_total = (float)(n * dims);
    for (uint32_t i = 0; i < n; i++)
        for (uint32_t ch = 0; ch < 16; ch++) {
            float pred = predictions[16u * i + ch];
            float loss = 0.f, grad = 0.f;
            const float *tg = targets + 8u * i;
            int ignore = lc->visibility_masking_loss ? (tg[0] < 0.5f) : 0;
            if (ch == 0) {
                loss_and_gradient(lc->visibility_loss, tg[0], pred, &loss, &grad);
                loss *= lc->visibility_loss_scale;
                grad *= lc->visibility_loss_scale;
            } else if (ch == 1 && !ignore) {
                loss_and_gradient(lc->depth_loss, tg[1], pred, &loss, &grad);
                loss *= lc->depth_loss_scale;
                grad *= lc->depth_loss_scale;
            } else if (ch >= 2 && ch < 5 && !ignore && lc->learn_normal) {
                if (lc->output_normal_linear_activation) {
                    float n_length = 0.1f;
                    float n_axis = (pred * 2.0f - 1.0f) / n_length;
                    float lin = n_axis * 0.5f + 0.5f;
                    loss_and_gradient(lc->normal_loss, tg[ch], lin, &loss, &grad);
                    grad *= 1.0f / n_length;
                } else {
                    loss_and_gradient(lc->normal_loss, tg[ch], pred, &loss, &grad);
                }
                loss *= lc->normal_loss_scale;
                grad *= lc->normal_loss_scale;
            } else if (ch >= 5 && ch < 8 && !ignore && lc->learn_albedo) {
                if (lc->output_albedo_linear_activation) {
                    float n_length = 0.1f;
                    float lin = pred / n_length;
                    loss_and_gradient(lc->albedo_loss, tg[ch], lin, &loss, &grad);
                    grad *= 1.0f / n_length;
                } else {
                    loss_and_gradient(lc->albedo_loss, tg[ch], pred, &loss, &grad);
                }
                loss *= lc->albedo_loss_scale;
                grad *= lc->albedo_loss_scale;
            }
            values[16u * i + ch] = loss / n_total;
            gradients[16u * i + ch] = loss_scale * grad / n_total;
        }
}

/* ------------------------------------------------------------------------------------------ */
/* Backward pass (gradient of the mean loss), FP64 accumulation                               */
/* ------------------------------------------------------------------------------------------ */

void orc_compute_gradients(const orc_network *net, const orc_loss_consts *lc, const float *positions,
                           const float *targets, uint32_t n, float loss_scale, double *gradients,
                           double *mean_loss, int fp16_backward)
{
    uint32_t off[16], rows[16], cols[16], nm;
    matrix_offsets(net, off, rows, cols, &nm);
    uint32_t n_net = off[nm - 1u] + rows[nm - 1u] * cols[nm - 1u];
    uint32_t n_grid = net->level_offset[net->n_levels - 1u] + net->level_size[net->n_levels - 1u];
    const uint32_t F = net_features(net);
    memset(gradients, 0, sizeof(double) * ((size_t)n_net + (size_t)F * n_grid));
    double total_loss = 0.0;
    float *acts = (float *)malloc(sizeof(float) * 128u * 16u);
    double dz[128], da[128];
    for (uint32_t i = 0; i < n; i++) {
        float feat[128], out[16], vals[16], grads[16];
        double pre[16];
        const float *pos = positions + (size_t)i * net->n_points * 3u;
        /* forward, keeping the corner indices and weights for the grid backward */
        uint32_t cidx[16][32][8];
        float cw[16][32][8];
        for (uint32_t k = 0; k < net->n_points; k++)
            encode_point(net, load3(pos + 3u * k), &feat[k * net->n_levels * F], cidx[k], cw[k]);
        mlp_row(net, feat, out, acts, pre);
        orc_composite_loss(lc, out, targets + 8u * (size_t)i, 1, loss_scale, vals, grads);
        /* the per-row loss values are normalised by n_total of a batch of one; rescale to n */
        for (uint32_t ch = 0; ch < 16; ch++) {
            total_loss += (double)vals[ch] / (double)n;
            float g = grads[ch] / (float)n;
            if (fp16_backward)
                g = round_mlp(net, g);
            double s = 1.0 / (1.0 + exp(-pre[ch]));
            dz[ch] = (double)g * s * (1.0 - s);
            if (fp16_backward)
                dz[ch] = (double)round_mlp(net, (float)dz[ch]);
        }
        /* layers backward */
        for (int m = (int)nm - 1; m >= 0; m--) {
            const float *a = acts + 128u * (uint32_t)m;
            double *gw = gradients + off[m];
            for (uint32_t r = 0; r < rows[m]; r++) {
                if (dz[r] == 0.0)
                    continue;
                for (uint32_t k = 0; k < cols[m]; k++)
                    gw[(size_t)r * cols[m] + k] += dz[r] * (double)a[k];
            }
            for (uint32_t k = 0; k < cols[m]; k++) {
                double s = 0.0;
                for (uint32_t r = 0; r < rows[m]; r++)
                    s += dz[r] * (double)net_w(net, off[m] + (size_t)r * cols[m] + k);
                da[k] = s;
            }
            if (m > 0) {
                for (uint32_t k = 0; k < cols[m]; k++) {
                    double g = a[k] > 0.0f ? da[k] : 0.0; /* ReLU of the previous layer */
                    if (fp16_backward)
                        g = (double)round_mlp(net, (float)g);
                    dz[k] = g;
                }
            }
        }
        /* grid backward: d feature = da (input gradient of the first layer) */
        double *gg = gradients + n_net;
        for (uint32_t k = 0; k < net->n_points; k++)
            for (uint32_t l = 0; l < net->n_levels; l++)
                for (uint32_t q = 0; q < F; q++) {
                    double gq = da[(k * net->n_levels + l) * F + q];
                    if (fp16_backward)
                        gq = (double)round_mlp(net, (float)gq);
                    for (uint32_t cc = 0; cc < 8; cc++)
                        gg[(size_t)F * cidx[k][l][cc] + q] += (double)cw[k][l][cc] * gq;
                }
    }
    free(acts);
    for (size_t p = 0; p < (size_t)n_net + (size_t)F * n_grid; p++)
        gradients[p] /= (double)loss_scale;
    *mean_loss = total_loss;
}

/* ------------------------------------------------------------------------------------------ */
/* Adam with ExponentialDecay (Kingma & Ba 2015, Algorithm 1, bias correction folded into the  */
/* step size); decay as configured at neural_bvh_module.cu:146-150                             */
/* ------------------------------------------------------------------------------------------ */

void orc_adam_step(float *params, float *m, float *v, const float *grad, uint32_t n, uint32_t step, float lr,
                   float beta1, float beta2, float eps, float l2_reg, int32_t decay_start, int32_t decay_interval,
                   float decay_base)
{
    double lr_s = (double)lr;
    if ((int64_t)step >= (int64_t)decay_start && decay_interval > 0)
        lr_s *= pow((double)decay_base, (double)(((int64_t)step - decay_start) / decay_interval));
    double t = (double)step + 1.0;
    float lr_t = (float)(lr_s * sqrt(1.0 - pow((double)beta2, t)) / (1.0 - pow((double)beta1, t)));
    float omb1 = 1.0f - beta1, omb2 = 1.0f - beta2;
    for (uint32_t i = 0; i < n; i++) {
        float w = params[i];
        float g = grad[i] + l2_reg * w;
        float mi = beta1 * m[i] + omb1 * g;
        float vi = beta2 * v[i] + omb2 * (g * g);
        m[i] = mi;
        v[i] = vi;
        params[i] = w - lr_t * (mi / (sqrtf(vi) + eps));
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Camera rays: CudaBackend::update_camera cuda_backend.cpp:595-611, camera_raygen             */
/* renderer_kernels.cuh:74-79, jitter from get_lcg_rng(sample_idx, offset, pixel)              */
/* neural_bvh_module_common.cuh:222-228                                                         */
/* ------------------------------------------------------------------------------------------ */

void orc_camera_basis(uint32_t width, uint32_t height, const float *origin, const float *target, const float *up,
                      float yfov_degrees, float *du_out, float *dv_out, float *tl_out)
{
    float ipy = 2.0f * tanf((0.5f * yfov_degrees) * 0.0174532925199432958f);
    float aspect = (float)width / (float)height;
    float ipx = ipy * aspect;
    v3 org = load3(origin);
    v3 dir = vnormalize(vsub(load3(target), org));
    v3 upv = vnormalize(load3(up));
    v3 du = vscale(vnormalize(vcross(dir, upv)), ipx);
    v3 dv = vscale(vnormalize(vcross(du, dir)), -ipy);
    v3 tl = vsub(vsub(dir, vscale(du, 0.5f)), vscale(dv, 0.5f));
    du_out[0] = du.x, du_out[1] = du.y, du_out[2] = du.z;
    dv_out[0] = dv.x, dv_out[1] = dv.y, dv_out[2] = dv.z;
    tl_out[0] = tl.x, tl_out[1] = tl.y, tl_out[2] = tl.z;
}

void orc_camera_rays(uint32_t width, uint32_t height, uint32_t sample_idx, uint32_t sample_offset,
                     const float *origin, const float *target, const float *up, float yfov_degrees, float *rays)
{
    float ipy = 2.0f * tanf((0.5f * yfov_degrees) * 0.0174532925199432958f);
    float aspect = (float)width / (float)height;
    float ipx = ipy * aspect;
    v3 org = load3(origin);
    v3 dir = vnormalize(vsub(load3(target), org));
    v3 upv = vnormalize(load3(up));
    v3 du = vscale(vnormalize(vcross(dir, upv)), ipx);
    v3 dv = vscale(vnormalize(vcross(du, dir)), -ipy);
    v3 tl = vsub(vsub(dir, vscale(du, 0.5f)), vscale(dv, 0.5f));
    for (uint32_t p = 0; p < width * height; p++) {
        uint32_t px = p % width, py = p / width;
        uint32_t rng = orc_lcg_seed(sample_idx, sample_offset, p);
        float jx = orc_lcg_randomf(&rng);
        float jy = orc_lcg_randomf(&rng);
        float xf = ((float)px + jx) / (float)width;
        float yf = ((float)py + jy) / (float)height;
        v3 d = vnormalize(vadd(vadd(vscale(du, xf), vscale(dv, yf)), tl));
        float *r = rays + 8u * (size_t)p;
        r[0] = org.x;
        r[1] = org.y;
        r[2] = org.z;
        r[3] = 1e-4f;
        r[4] = d.x;
        r[5] = d.y;
        r[6] = d.z;
        r[7] = FLT_MAX;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Learned tree cut: include/cuda/neural/utils/bvh_split_scheduler.h:13-145,                  */
/* src/cuda/neural/neural_bvh_renderer_kernels.cu:202-287,                                     */
/* src/cuda/neural/neural_bvh_renderer_accel.cpp:256-441                                       */
/* ------------------------------------------------------------------------------------------ */

void orc_tree_cut_accumulate(uint32_t *stats, const float *values, const uint32_t *sample_nodes, uint32_t n,
                             uint32_t dims)
{
    /* update_neural_tree_cut_loss: every output channel's loss value goes to its sample's node */
    for (uint32_t i = 0; i < n; i++) {
        uint32_t *st = stats + 4u * sample_nodes[i];
        float loss;
        memcpy(&loss, st, 4);
        for (uint32_t ch = 0; ch < dims; ch++)
            loss += values[(size_t)i * dims + ch];
        memcpy(st, &loss, 4);
        st[3] += dims;
    }
}

static int node_has_child(const uint32_t *nd) { return nd[7] != ORC_NO_NEURAL_CHILD; }

void orc_tree_cut_decisions(const uint32_t *nodes, uint32_t n_nodes, uint32_t *stats, uint32_t k,
                            float *max_losses, uint32_t *split_indices)
{
    /* the k + 1 launches of update_neural_tree_cut_decisions, run in node order */
    for (uint32_t j = 0; j < k; j++) {
        max_losses[j] = 0.0f;
        split_indices[j] = 0u;
    }
    for (uint32_t j = 0; j <= k; j++) {
        for (uint32_t i = 0; i < n_nodes; i++) {
            const uint32_t *nd = nodes + 8u * i;
            if (node_has_child(nd))
                continue;
            uint32_t *st = stats + 4u * i;
            if (j == 0)
                st[1] += 1u;
            if (nd[3] == ORC_LEAF_FINAL)
                continue;
            const float candidate = orc_loss_heuristic(st);
            if (j > 0) {
                const float prev = max_losses[j - 1u];
                if (candidate >= prev) {
                    if (candidate == prev)
                        split_indices[j - 1u] = i;
                    continue;
                }
            }
            if (j == k)
                continue;
            max_losses[j] = fmaxf(candidate, max_losses[j]);
        }
    }
}

uint32_t orc_tree_cut_split(uint32_t *nodes, uint32_t *n_nodes, uint32_t capacity, uint32_t *stats,
                            uint32_t *node_map, const uint32_t *classic_nodes, const uint32_t *split_indices,
                            uint32_t k, uint32_t current_lod)
{
    /* split_neural_bvh_at: the first min(#leaves, k) indices, unique, ascending (std::set) */
    uint32_t n = *n_nodes;
    const uint32_t n_leaves = (n + 1u) / 2u;
    const uint32_t m = k < n_leaves ? k : n_leaves;
    uint8_t *chosen = (uint8_t *)calloc(n, 1);
    for (uint32_t j = 0; j < m; j++)
        if (split_indices[j] < n)
            chosen[split_indices[j]] = 1u;
    uint32_t splits = 0;
    for (uint32_t i = 0; i < *n_nodes; i++) {
        if (!chosen[i])
            continue;
        const uint32_t *parent = classic_nodes + 8u * node_map[i];
        if (parent[3] > 0u) /* classic leaf: no split */
            continue;
        uint32_t *nd = nodes + 8u * i;
        if (node_has_child(nd))
            continue;
        if (n + 2u > capacity)
            break;
        const uint32_t cl = parent[7];
        const uint32_t left = n++, right = n++;
        node_map[left] = cl;
        node_map[right] = cl + 1u;
        if (nd[3] == ORC_LEAF_LOD(current_lod))
            nd[3] = 0u;
        nd[7] = left;
        for (int w = 0; w < 3; w++) {
            nd[w] = parent[w];
            nd[4 + w] = parent[4 + w];
        }
        for (uint32_t c = 0; c < 2; c++) {
            const uint32_t *src = classic_nodes + 8u * (cl + c);
            uint32_t *dst = nodes + 8u * (left + c);
            for (int w = 0; w < 3; w++) {
                dst[w] = src[w];
                dst[4 + w] = src[4 + w];
            }
            dst[3] = src[3] > 0u ? ORC_LEAF_FINAL : ORC_LEAF_LOD(current_lod);
            dst[7] = ORC_NO_NEURAL_CHILD;
            uint32_t *cs = stats + 4u * (left + c);
            const float zero = 0.0f;
            memcpy(cs, &zero, 4);
            cs[1] = 1u;
            cs[2] = stats[4u * i + 2u] + 1u;
            cs[3] = 0u;
        }
        splits++;
    }
    free(chosen);
    *n_nodes = n;
    return splits;
}

void orc_tree_cut_assign_lod(uint32_t *nodes, uint32_t n_nodes, uint32_t lod)
{
    /* assign_lod_to_current_neural_leaf_nodes */
    if (lod == ORC_NUM_BVH_LODS - 1u)
        return;
    for (uint32_t i = 0; i < n_nodes; i++) {
        uint32_t *nd = nodes + 8u * i;
        if (!node_has_child(nd))
            nd[3] = nd[3] == ORC_LEAF_FINAL ? ORC_LEAF_FINAL : ORC_LEAF_LOD(lod);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Hybrid path tracer: camera paths, Lambertian bounces on the neural hits (the network's normal */
/* and albedo), an analytic ground plane and an analytic sky as the only light (the library's   */
/* k_path.cu; the reference's scatter is path_inference_kernels.cu:224-429 with a Disney BSDF,  */
/* of which this is the Lambertian case, cosine sampling as material.cuh:101-200). Every FP32   */
/* operation in the same order as the kernels, which are compiled without FMA contraction.      */
/* ------------------------------------------------------------------------------------------ */

/* Duff et al., "Building an Orthonormal Basis, Revisited", JCGT 6(1), 2017 */
static void path_onb(v3 n, v3 *t, v3 *b)
{
    const float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sign + n.z);
    const float c = n.x * n.y * a;
    *t = mk(1.0f + sign * n.x * n.x * a, sign * c, -sign * n.x);
    *b = mk(c, sign + n.y * n.y * a, -n.y);
}

/* cosine-weighted direction about n: a uniform disk point lifted to the hemisphere */
static v3 path_cosine_sample(v3 n, uint32_t *rng)
{
    const float u1 = orc_lcg_randomf(rng), u2 = orc_lcg_randomf(rng);
    float sp, cp;
    orc_sincos_turns(u2, &sp, &cp);
    const float r = sqrtf(u1), z = sqrtf(fmaxf(0.0f, 1.0f - u1));
    v3 t, b;
    path_onb(n, &t, &b);
    return mk(r * cp * t.x + r * sp * b.x + z * n.x, r * cp * t.y + r * sp * b.y + z * n.y,
              r * cp * t.z + r * sp * b.z + z * n.z);
}

uint64_t orc_path_trace(const orc_neural_scene *scene, const orc_network *net, const orc_neural_consts *c,
                        const orc_path_params *p, float *image, int n_threads)
{
    const uint32_t n = p->width * p->height * p->spp;
    float *thr = (float *)malloc(sizeof(float) * 4u * n), *rad = (float *)calloc(4u * (size_t)n, sizeof(float));
    float *rays = (float *)malloc(sizeof(float) * 8u * n), *next = (float *)malloc(sizeof(float) * 8u * n);
    uint32_t *ids = (uint32_t *)malloc(sizeof(uint32_t) * n), *next_ids = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint32_t *hits = (uint32_t *)malloc(sizeof(uint32_t) * 12u * n);
    const v3 du = load3(p->du), dv = load3(p->dv), tl = load3(p->tl);
    for (uint32_t i = 0; i < n; i++) { /* raygen: the camera jitter of sample sample_base + s */
        const uint32_t px_ = i / p->spp, smp = i - px_ * p->spp;
        const uint32_t x = px_ % p->width, y = px_ / p->width;
        uint32_t rng = orc_lcg_seed(p->sample_base + smp, p->sample_offset, px_);
        const float jx = orc_lcg_randomf(&rng), jy = orc_lcg_randomf(&rng);
        const float xf = ((float)x + jx) / (float)p->width;
        const float yf = ((float)y + jy) / (float)p->height;
        const v3 d = vnormalize(vadd(vadd(vscale(du, xf), vscale(dv, yf)), tl));
        float *r = rays + 8u * (size_t)i;
        r[0] = p->origin[0], r[1] = p->origin[1], r[2] = p->origin[2], r[3] = 1e-4f;
        r[4] = d.x, r[5] = d.y, r[6] = d.z, r[7] = FLT_MAX;
        ids[i] = i;
        thr[4u * i] = thr[4u * i + 1u] = thr[4u * i + 2u] = 1.0f;
        const uint32_t bits = rng ^ (p->seed * 0x9E3779B9u);
        memcpy(&thr[4u * i + 3u], &bits, 4);
    }
    uint32_t count = n;
    uint64_t traced = 0;
    for (uint32_t bounce = 0; count > 0 && bounce <= p->max_bounces; bounce++) {
        orc_neural_query(scene, net, c, NULL, 0.0f, rays, count, bounce == 0 ? 1u : 2u, 0, hits, n_threads);
        traced += count;
        uint32_t out = 0;
        for (uint32_t j = 0; j < count; j++) {
            const uint32_t id = ids[j];
            const float *r = rays + 8u * (size_t)j;
            const v3 ro = mk(r[0], r[1], r[2]), d = mk(r[4], r[5], r[6]);
            const uint32_t *h = hits + 12u * (size_t)j;
            float hf[8];
            memcpy(hf, h, sizeof(hf));
            const int nhit = (h[8] & 1u) != 0u;
            float t = nhit ? hf[0] : FLT_MAX;
            v3 nrm = mk(hf[1], hf[2], hf[3]), alb = mk(hf[4], hf[5], hf[6]);
            if (p->has_ground && d.y != 0.0f) {
                const float tp = (p->ground_y - ro.y) / d.y;
                if (tp > 1e-4f && tp < t) {
                    t = tp;
                    nrm = mk(0.0f, 1.0f, 0.0f);
                    alb = load3(p->ground_albedo);
                }
            }
            float *th = thr + 4u * (size_t)id;
            if (t == FLT_MAX) {
                const float w = fmaxf(d.y, 0.0f);
                float *ra = rad + 4u * (size_t)id;
                for (int k = 0; k < 3; k++)
                    ra[k] += th[k] * (p->sky_horizon[k] + (p->sky_zenith[k] - p->sky_horizon[k]) * w);
            } else if (bounce < p->max_bounces) {
                const float len = sqrtf(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
                nrm = len > 0.0f ? mk(nrm.x / len, nrm.y / len, nrm.z / len) : mk(-d.x, -d.y, -d.z);
                if (nrm.x * d.x + nrm.y * d.y + nrm.z * d.z > 0.0f)
                    nrm = mk(-nrm.x, -nrm.y, -nrm.z);
                uint32_t rng;
                memcpy(&rng, &th[3], 4);
                const v3 nd = path_cosine_sample(nrm, &rng);
                th[0] = th[0] * alb.x;
                th[1] = th[1] * alb.y;
                th[2] = th[2] * alb.z;
                memcpy(&th[3], &rng, 4);
                const v3 o = mk(ro.x + t * d.x + 1e-3f * nrm.x, ro.y + t * d.y + 1e-3f * nrm.y,
                                ro.z + t * d.z + 1e-3f * nrm.z);
                if (th[0] + th[1] + th[2] > 0.0f) {
                    float *q = next + 8u * (size_t)out;
                    q[0] = o.x, q[1] = o.y, q[2] = o.z, q[3] = 1e-4f;
                    q[4] = nd.x, q[5] = nd.y, q[6] = nd.z, q[7] = FLT_MAX;
                    next_ids[out++] = id;
                }
            }
        }
        float *tr = rays;
        rays = next;
        next = tr;
        uint32_t *ti = ids;
        ids = next_ids;
        next_ids = ti;
        count = out;
    }
    const float inv = 1.0f / (float)p->spp;
    for (uint32_t px_ = 0; px_ < p->width * p->height; px_++) {
        float r = 0.f, g = 0.f, b = 0.f;
        for (uint32_t s = 0; s < p->spp; s++) {
            const float *v = rad + 4u * ((size_t)px_ * p->spp + s);
            r += v[0];
            g += v[1];
            b += v[2];
        }
        image[4u * px_] = r * inv;
        image[4u * px_ + 1u] = g * inv;
        image[4u * px_ + 2u] = b * inv;
        image[4u * px_ + 3u] = 1.0f;
    }
    free(thr), free(rad), free(rays), free(next), free(ids), free(next_ids), free(hits);
    return traced;
}
