// device_math.cuh -- FP32 vector arithmetic with glm's evaluation order and no FMA contraction,
// the reference RNG, and the ray/box and ray/triangle tests, for the bit-exact parts of the
// kernels (classic and neural traversal, training-ray sampling).
//
// Every operation is an explicitly rounded intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn) so that nvcc cannot fuse it, and the order follows glm: dot = (x*x' + y*y') + z*z',
// cross = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y), min(a, b) = b < a ? b : a,
// max(a, b) = a < b ? b : a, normalize(v) = v * (1 / sqrt(dot(v, v))).
#pragma once

#include <cstring>
#include <cfloat>
#include <cstdint>

namespace nbvh {

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 mk3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return mk3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return mk3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ V3 mul3(V3 a, V3 b) { return mk3(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)); }
__device__ __forceinline__ V3 div3(V3 a, V3 b) { return mk3(__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y), __fdiv_rn(a.z, b.z)); }
__device__ __forceinline__ V3 scale3(V3 a, float s) { return mk3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ V3 adds3(V3 a, float s) { return mk3(__fadd_rn(a.x, s), __fadd_rn(a.y, s), __fadd_rn(a.z, s)); }
__device__ __forceinline__ float dot3(V3 a, V3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 cross3(V3 a, V3 b)
{
    return mk3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
               __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y)));
}
__device__ __forceinline__ float gmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float gmax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ V3 min3(V3 a, V3 b) { return mk3(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
__device__ __forceinline__ V3 max3(V3 a, V3 b) { return mk3(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
__device__ __forceinline__ float cmax3(V3 v) { return gmax(gmax(v.x, v.y), v.z); }
__device__ __forceinline__ float cmin3(V3 v) { return gmin(gmin(v.x, v.y), v.z); }
__device__ __forceinline__ V3 normalize3(V3 v) { return scale3(v, __fdiv_rn(1.0f, __fsqrt_rn(dot3(v, v)))); }
__device__ __forceinline__ float length3(V3 v) { return __fsqrt_rn(dot3(v, v)); }
__device__ __forceinline__ V3 ray_at(V3 o, V3 d, float t) { return add3(o, scale3(d, t)); }
__device__ __forceinline__ float gclamp01(float x) { return gmin(gmax(x, 0.0f), 1.0f); }

// ---- RNG: include/cuda/utils/lcg_rng.cuh:12-79 ----
__device__ __forceinline__ uint32_t murmur_mix(uint32_t hash, uint32_t k)
{
    k *= 0xcc9e2d51u;
    k = (k << 15) | (k >> 17);
    k *= 0x1b873593u;
    hash ^= k;
    hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
    return hash;
}
__device__ __forceinline__ uint32_t murmur_finalize(uint32_t hash)
{
    hash ^= hash >> 16;
    hash *= 0x85ebca6bu;
    hash ^= hash >> 13;
    hash *= 0xc2b2ae35u;
    hash ^= hash >> 16;
    return hash;
}
__device__ __forceinline__ uint32_t lcg_seed(uint32_t index, uint32_t frame, uint32_t linear)
{
    uint32_t s = murmur_mix(0u, linear);
    s = murmur_mix(s, 512u * frame + index);
    return murmur_finalize(s);
}
__device__ __forceinline__ float lcg_randomf(uint32_t &state)
{
    state = state * 1664525u + 1013904223u;
    return __fmul_rn(__uint2float_rn(state), 0x1p-32f);
}

// sin(2 pi u), cos(2 pi u): octant reduction of u, Taylor series of degree 11 / 12 on [0, pi/4]
// evaluated with fused multiply-adds (identical to the host restatement).
__device__ __forceinline__ void sincos_turns(float u, float &s, float &c)
{
    float y = __fmul_rn(u, 8.0f);
    float o = floorf(y);
    float f = __fsub_rn(y, o);
    int oct = ((int)o) & 7;
    float g = (oct & 1) ? __fsub_rn(1.0f, f) : f;
    float x = __fmul_rn(g, 0.785398163397448310f);
    float x2 = __fmul_rn(x, x);
    float ps = __fmaf_rn(x2, -2.50521084e-08f, 2.75573192e-06f);
    ps = __fmaf_rn(x2, ps, -1.98412698e-04f);
    ps = __fmaf_rn(x2, ps, 8.33333333e-03f);
    ps = __fmaf_rn(x2, ps, -1.66666667e-01f);
    ps = __fmaf_rn(x2, ps, 1.0f);
    float sn = __fmul_rn(x, ps);
    float pc = __fmaf_rn(x2, 2.08767570e-09f, -2.75573192e-07f);
    pc = __fmaf_rn(x2, pc, 2.48015873e-05f);
    pc = __fmaf_rn(x2, pc, -1.38888889e-03f);
    pc = __fmaf_rn(x2, pc, 4.16666667e-02f);
    pc = __fmaf_rn(x2, pc, -0.5f);
    float cs = __fmaf_rn(x2, pc, 1.0f);
    switch (oct) {
    case 0: s = sn; c = cs; break;
    case 1: s = cs; c = sn; break;
    case 2: s = cs; c = -sn; break;
    case 3: s = sn; c = -cs; break;
    case 4: s = -sn; c = -cs; break;
    case 5: s = -cs; c = -sn; break;
    case 6: s = -cs; c = sn; break;
    default: s = -sn; c = cs; break;
    }
}

// square_to_uniform_sphere, include/cuda/utils/sampling.cuh:8-14
__device__ __forceinline__ V3 uniform_sphere(float sx, float sy)
{
    float sp, cp;
    sincos_turns(sx, sp, cp);
    float cos_theta = __fsub_rn(__fmul_rn(sy, 2.0f), 1.0f);
    float sin_theta = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(cos_theta, cos_theta)));
    return mk3(__fmul_rn(sin_theta, cp), __fmul_rn(sin_theta, sp), cos_theta);
}

// ---- BVH node access (32-byte nodes as two float4) ----
struct NodeBox {
    V3 mn;
    uint32_t count;
    V3 mx;
    uint32_t offset;
};
__device__ __forceinline__ NodeBox load_node(const float4 *nodes, uint32_t idx)
{
    float4 a = __ldg(nodes + 2u * idx);
    float4 b = __ldg(nodes + 2u * idx + 1u);
    NodeBox n;
    n.mn = mk3(a.x, a.y, a.z);
    n.count = __float_as_uint(a.w);
    n.mx = mk3(b.x, b.y, b.z);
    n.offset = __float_as_uint(b.w);
    return n;
}

// Ray prepared for slab tests: the direction, its correctly rounded reciprocal and whether the
// divisions (b - o) / d may use Markstein's correctly rounded division from a correctly rounded
// reciprocal (P. Markstein, "IA-64 and Elementary Functions", 2000: with y = RN(1/d),
// q0 = RN(a*y), r = a - d*q0 (exact by FMA), RN(q0 + r*y) = RN(a/d) when nothing overflows or
// underflows). It holds here when |d_i| is in [2^-60, 2^4], o_i is 0 or |o_i| in [2^-60, 2^11]
// and every box coordinate is +0 or has magnitude in [2^-60, 2^11] (checked on the host for
// the scene): then a = b - o is +0 or |a| in [2^-83, 2^12], and the quotient is normal. Outside
// that domain the IEEE division is used. Both give the bits of the IEEE quotient.
struct RayDiv {
    V3 d, inv;
    bool fast;
};

__device__ __forceinline__ bool coord_ok(float x)
{
    const float ax = fabsf(x);
    return x == 0.0f || (ax >= 0x1p-60f && ax <= 0x1p11f);
}

__device__ __forceinline__ RayDiv make_raydiv(V3 o, V3 d, bool scene_ok)
{
    RayDiv r;
    r.d = d;
    auto dir_ok = [](float x) {
        const float ax = fabsf(x);
        return ax >= 0x1p-60f && ax <= 0x1p4f;
    };
    r.fast = scene_ok && dir_ok(d.x) && dir_ok(d.y) && dir_ok(d.z) && coord_ok(o.x) && coord_ok(o.y) && coord_ok(o.z);
    r.inv = r.fast ? mk3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)) : mk3(0.f, 0.f, 0.f);
    return r;
}

__device__ __forceinline__ float markstein_div(float a, float b, float y)
{
    const float q0 = __fmul_rn(a, y);
    const float r = __fmaf_rn(-q0, b, a);
    return __fmaf_rn(r, y, q0);
}

__device__ __forceinline__ V3 div3r(V3 a, const RayDiv &r)
{
    if (r.fast)
        return mk3(markstein_div(a.x, r.d.x, r.inv.x), markstein_div(a.y, r.d.y, r.inv.y),
                   markstein_div(a.z, r.d.z, r.inv.z));
    return div3(a, r.d);
}

// BVH2Node::intersect, include/base/accel/bvh.h:121-133
__device__ __forceinline__ float box_entry(V3 bmin, V3 bmax, V3 o, V3 d, float rmint, float rmaxt)
{
    V3 t0 = div3(sub3(bmin, o), d);
    V3 t1 = div3(sub3(bmax, o), d);
    float mint = gmax(rmint, cmax3(min3(t0, t1)));
    float maxt = gmin(rmaxt, cmin3(max3(t0, t1)));
    return (mint <= maxt) ? mint : FLT_MAX;
}

// BVH2Node::intersect with the prepared-ray division (bit-identical quotients)
__device__ __forceinline__ float box_entry(V3 bmin, V3 bmax, V3 o, const RayDiv &rd, float rmint, float rmaxt)
{
    V3 t0 = div3r(sub3(bmin, o), rd);
    V3 t1 = div3r(sub3(bmax, o), rd);
    float mint = gmax(rmint, cmax3(min3(t0, t1)));
    float maxt = gmin(rmaxt, cmin3(max3(t0, t1)));
    return (mint <= maxt) ? mint : FLT_MAX;
}

// Ray3f::intersect_bbox_min_max without ray bounds, include/cuda/base/ray.cuh:111-132
__device__ __forceinline__ bool slab_min_max(V3 bmin, V3 bmax, V3 o, V3 d, float &mint, float &maxt)
{
    V3 t0 = div3(sub3(bmin, o), d);
    V3 t1 = div3(sub3(bmax, o), d);
    mint = cmax3(min3(t0, t1));
    maxt = cmin3(max3(t0, t1));
    return mint <= maxt;
}

// dilated neural node box: BVH2Node::bbox_center (min + extent * 0.5) and
// include/cuda/neural/accel/neural_bvh2.cuh:80-86
__device__ __forceinline__ void dilated_box(const NodeBox &n, float dil, V3 &bmin, V3 &bmax)
{
    if (dil != 0.0f) {
        V3 ext = sub3(n.mx, n.mn);
        V3 center = add3(n.mn, scale3(ext, 0.5f));
        V3 next = scale3(ext, __fadd_rn(1.0f, dil));
        bmin = sub3(center, scale3(next, 0.5f));
        bmax = add3(center, scale3(next, 0.5f));
    } else {
        bmin = n.mn;
        bmax = n.mx;
    }
}

// BaseCudaBLAS::intersect_triangle (Moller-Trumbore), include/cuda/accel/bvh.cuh:98-136, on a
// pre-gathered record {v0 | prim, e1 = v1 - v0, e2 = v2 - v0}.
__device__ __forceinline__ bool tri_intersect(V3 v0, V3 e1, V3 e2, V3 o, V3 d, float rmint, float rmaxt, float &t_out,
                                              float &u_out, float &v_out)
{
    V3 pvec = cross3(d, e2);
    float det = dot3(e1, pvec);
    if (det > -1e-8f && det < 1e-8f)
        return false;
    float inv_det = __fdiv_rn(1.0f, det);
    V3 tvec = sub3(o, v0);
    float u = __fmul_rn(dot3(tvec, pvec), inv_det);
    if (u < 0.0f || u > 1.0f)
        return false;
    V3 qvec = cross3(tvec, e1);
    float v = __fmul_rn(dot3(d, qvec), inv_det);
    if (v < 0.0f || __fadd_rn(u, v) > 1.0f)
        return false;
    float t = __fmul_rn(dot3(e2, qvec), inv_det);
    if (t < rmint || t >= rmaxt)
        return false;
    t_out = t;
    u_out = u;
    v_out = v;
    return true;
}

// CudaBVH2::intersect<ShadowRay>, include/cuda/accel/bvh2.cuh:12-88: root-first DFS, nearer child
// first (swap when child1_mint > child2_mint), ray.maxt shrinks on every accepted hit.
template <bool ANY_HIT>
__device__ __forceinline__ void classic_traverse(const float4 *__restrict__ nodes, const float4 *__restrict__ tris, V3 o,
                                                 V3 d, float rmint, float rmaxt, float &best_t, float &best_u,
                                                 float &best_v, uint32_t &best_prim, uint32_t *best_rec = nullptr,
                                                 bool scene_fast_div = false)
{
    best_t = FLT_MAX;
    best_u = 0.f;
    best_v = 0.f;
    best_prim = 0xFFFFFFFFu;
    const RayDiv rd = make_raydiv(o, d, scene_fast_div);
    uint32_t stack[32];
    int sp = 0;
    NodeBox node = load_node(nodes, 0);
    for (;;) {
        if (node.count > 0u) {
            bool done = false;
            for (uint32_t pid = node.offset; pid < node.offset + node.count; pid++) {
                float4 r0 = __ldg(tris + 3u * pid);
                float4 r1 = __ldg(tris + 3u * pid + 1u);
                float4 r2 = __ldg(tris + 3u * pid + 2u);
                float t, u, v;
                if (tri_intersect(mk3(r0.x, r0.y, r0.z), mk3(r1.x, r1.y, r1.z), mk3(r2.x, r2.y, r2.z), o, d, rmint,
                                  rmaxt, t, u, v) &&
                    t < rmaxt) {
                    best_t = t;
                    best_u = u;
                    best_v = v;
                    best_prim = __float_as_uint(r0.w);
                    if (best_rec)
                        *best_rec = pid;
                    if (ANY_HIT) {
                        done = true;
                        break;
                    }
                    rmaxt = t;
                }
            }
            if (done || sp == 0)
                return;
            node = load_node(nodes, stack[--sp]);
            continue;
        }
        uint32_t c1 = node.offset, c2 = node.offset + 1u;
        // both children are adjacent: four 128-bit loads
        NodeBox n1 = load_node(nodes, c1);
        NodeBox n2 = load_node(nodes, c2);
        float d1 = box_entry(n1.mn, n1.mx, o, rd, rmint, rmaxt);
        float d2 = box_entry(n2.mn, n2.mx, o, rd, rmint, rmaxt);
        if (d1 > d2) {
            float td = d1;
            d1 = d2;
            d2 = td;
            uint32_t tc = c1;
            c1 = c2;
            c2 = tc;
            NodeBox tn = n1;
            n1 = n2;
            n2 = tn;
        }
        if (d1 == FLT_MAX) {
            if (sp == 0)
                return;
            node = load_node(nodes, stack[--sp]);
        } else {
            node = n1;
            if (d2 != FLT_MAX && sp < 32)
                stack[sp++] = c2;
        }
    }
}

// NeuralBVH2::intersect, include/cuda/neural/accel/neural_bvh2.cuh:170-292. Pops the next node
// from `stack` and returns 1 with the next entered leaf segment, 0 when the stack runs empty,
// -1 on a stack overflow (the reference prints and returns false), 2 when `budget` node visits
// ran out first (call again to continue).
template <typename Stack>
__device__ __forceinline__ int neural_intersect(const float4 *__restrict__ nodes, uint32_t lod, V3 o, V3 d, Stack &stack,
                                                int &sp, bool inference, float mint_eps_inf, float maxt_eps_inf,
                                                float mint_eps_learn, float maxt_eps_learn, float current_maxt,
                                                float dil, float &seg_mint, float &seg_maxt, uint32_t &seg_node,
                                                int budget = 0x7FFFFFFF)
{
    const float rmint = -FLT_MAX, rmaxt = current_maxt;
    uint32_t node_idx = stack[--sp];
    for (;; budget--) {
        if (budget <= 0) {
            // out of node visits: the current node goes back on the stack and the call reports "not
            // finished" (2); the next call resumes exactly here (sp <= 23: a push to 24 returned -1)
            stack[sp++] = node_idx;
            return 2;
        }
        NodeBox node = load_node(nodes, node_idx);
        if ((node.count > 0u && node.count <= 2u + lod) || node.offset == 0xFFFFFFFFu) {
            V3 bmin, bmax;
            float mint, maxt;
            dilated_box(node, dil, bmin, bmax);
            if (slab_min_max(bmin, bmax, o, d, mint, maxt)) {
                float maxt_eps = inference ? maxt_eps_inf : maxt_eps_learn;
                float mint_eps = inference ? mint_eps_inf : mint_eps_learn;
                bool valid = mint < rmaxt;
                if (mint < 0.0f)
                    valid &= maxt > maxt_eps;
                else
                    valid &= mint > mint_eps;
                if (valid) {
                    seg_mint = mint;
                    seg_maxt = maxt;
                    seg_node = node_idx;
                    return 1;
                }
            }
            if (sp == 0)
                return 0;
            node_idx = stack[--sp];
            continue;
        }
        uint32_t c1 = node.offset, c2 = node.offset + 1u;
        NodeBox n1 = load_node(nodes, c1);
        NodeBox n2 = load_node(nodes, c2);
        V3 b1min, b1max, b2min, b2max;
        dilated_box(n1, dil, b1min, b1max);
        dilated_box(n2, dil, b2min, b2max);
        float d1 = box_entry(b1min, b1max, o, d, rmint, rmaxt);
        float d2 = box_entry(b2min, b2max, o, d, rmint, rmaxt);
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
                return 0;
            node_idx = stack[--sp];
        } else {
            node_idx = c1;
            if (d2 != FLT_MAX) {
                stack[sp++] = c2;
                if (sp >= 24)
                    return -1;
            }
        }
    }
}

// Raw slab of a box: entry = max_i min(t0_i, t1_i), exit = min_i max(t0_i, t1_i) with the
// glm operation order of Ray3f::intersect_bbox_min_max (include/cuda/base/ray.cuh:111-132).
__device__ __forceinline__ void slab_raw(V3 bmin, V3 bmax, V3 o, V3 d, float &entry, float &exit_)
{
    V3 t0 = div3(sub3(bmin, o), d);
    V3 t1 = div3(sub3(bmax, o), d);
    entry = cmax3(min3(t0, t1));
    exit_ = cmin3(max3(t0, t1));
}

__device__ __forceinline__ void slab_raw(V3 bmin, V3 bmax, V3 o, const RayDiv &rd, float &entry, float &exit_)
{
    V3 t0 = div3r(sub3(bmin, o), rd);
    V3 t1 = div3r(sub3(bmax, o), rd);
    entry = cmax3(min3(t0, t1));
    exit_ = cmin3(max3(t0, t1));
}

// Leaf acceptance of NeuralBVH2::intersect (neural_bvh2.cuh:199-215) from the raw slab.
__device__ __forceinline__ bool leaf_accepts(float entry, float exit_, float rmaxt, float mint_eps, float maxt_eps)
{
    if (!(entry <= exit_))
        return false;
    bool valid = entry < rmaxt;
    if (entry < 0.0f)
        valid &= exit_ > maxt_eps;
    else
        valid &= entry > mint_eps;
    return valid;
}

// NeuralBVH2::intersect for inference on a pre-dilated copy of the cut (`nodes` boxes already
// dilated by fixed_node_dilation with the reference's operations). Returns the same accepted leaf
// segments in the same order as the reference; it differs only in work skipped:
//  * the slab of the child it descends into is carried over instead of recomputed;
//  * a child is not pushed / entered when nothing below it can be accepted: a leaf that fails the
//    acceptance test now (the bound rmaxt only shrinks later), or an interior node whose union of
//    dilated leaf boxes (`bounds`) lies entirely at t <= min(mint_eps, maxt_eps), beyond rmaxt, or
//    is missed. The slab is monotone in the box bounds for non-zero direction components, so a leaf
//    inside the union exits no later and enters no earlier than the union (`cull_ok` is false for
//    rays with a zero direction component).
// Returns 1 with the next accepted leaf, 0 when the stack runs empty, -1 on stack overflow, and 2
// when `budget` node visits are used up before either (the traversal then resumes on the next
// call with the same stack).
// Node sources of the inference traversal: the pre-dilated cut and its subtree bounds, read from
// global memory (read-only cache) or from a shared-memory copy staged at kernel start.
struct GlobalCut {
    const float4 *nodes;  // 2 float4 per node
    const float4 *bounds; // 2 float4 per node: {min, 0}, {max, 0}
    __device__ __forceinline__ NodeBox node(uint32_t i) const { return load_node(nodes, i); }
    __device__ __forceinline__ void bound(uint32_t i, V3 &mn, V3 &mx) const
    {
        const float4 a = __ldg(bounds + 2u * i), b = __ldg(bounds + 2u * i + 1u);
        mn = mk3(a.x, a.y, a.z);
        mx = mk3(b.x, b.y, b.z);
    }
};

struct SharedCut {
    const float4 *nodes;  // shared memory, 2 float4 per node
    const float2 *bounds; // shared memory, 3 float2 per node: min.xy, min.z max.x, max.yz
    __device__ __forceinline__ NodeBox node(uint32_t i) const
    {
        const float4 a = nodes[2u * i], b = nodes[2u * i + 1u];
        NodeBox n;
        n.mn = mk3(a.x, a.y, a.z);
        n.count = __float_as_uint(a.w);
        n.mx = mk3(b.x, b.y, b.z);
        n.offset = __float_as_uint(b.w);
        return n;
    }
    __device__ __forceinline__ void bound(uint32_t i, V3 &mn, V3 &mx) const
    {
        const float2 a = bounds[3u * i], b = bounds[3u * i + 1u], c = bounds[3u * i + 2u];
        mn = mk3(a.x, a.y, b.x);
        mx = mk3(b.y, c.x, c.y);
    }
};

template <typename Src, typename Stack>
__device__ __forceinline__ int neural_intersect_inference(const Src &src, uint32_t lod, V3 o, const RayDiv &d,
                                                          bool cull_ok, Stack &stack, int &sp, float mint_eps,
                                                          float maxt_eps, float current_maxt, float &seg_mint,
                                                          float &seg_maxt, uint32_t &seg_node,
                                                          int budget = 0x7FFFFFFF)
{
    const float rmint = -FLT_MAX, rmaxt = current_maxt;
    const float cull_eps = gmin(mint_eps, maxt_eps);
    uint32_t node_idx = stack[--sp];
    NodeBox node = src.node(node_idx);
    bool have_slab = false;
    float cur_e = 0.f, cur_x = 0.f;
    for (;; budget--) {
        if (budget <= 0) {
            // out of node visits: put the current node back and report "not finished" (2); the next
            // call pops it and recomputes its slab, so the traversal resumes exactly where it
            // stopped. sp <= 23 here (a push that reached 24 returned -1), so the push fits.
            stack[sp++] = node_idx;
            return 2;
        }
        const bool leaf = (node.count > 0u && node.count <= 2u + lod) || node.offset == 0xFFFFFFFFu;
        if (leaf) {
            if (!have_slab)
                slab_raw(node.mn, node.mx, o, d, cur_e, cur_x);
            if (leaf_accepts(cur_e, cur_x, rmaxt, mint_eps, maxt_eps)) {
                seg_mint = cur_e;
                seg_maxt = cur_x;
                seg_node = node_idx;
                return 1;
            }
            if (sp == 0)
                return 0;
            node_idx = stack[--sp];
            node = src.node(node_idx);
            have_slab = false;
            continue;
        }
        uint32_t c1 = node.offset, c2 = node.offset + 1u;
        NodeBox n1 = src.node(c1);
        NodeBox n2 = src.node(c2);
        float e1, x1, e2, x2;
        slab_raw(n1.mn, n1.mx, o, d, e1, x1);
        slab_raw(n2.mn, n2.mx, o, d, e2, x2);
        // intersect_traversal_bbox with check_ray_bounds (neural_bvh2.cuh:94-115)
        float m1 = gmax(rmint, e1), m2 = gmax(rmint, e2);
        float d1 = (m1 <= gmin(rmaxt, x1)) ? m1 : FLT_MAX;
        float d2 = (m2 <= gmin(rmaxt, x2)) ? m2 : FLT_MAX;
        if (d1 > d2) {
            float t = d1;
            d1 = d2;
            d2 = t;
            uint32_t tc = c1;
            c1 = c2;
            c2 = tc;
            NodeBox tn = n1;
            n1 = n2;
            n2 = tn;
            t = e1;
            e1 = e2;
            e2 = t;
            t = x1;
            x1 = x2;
            x2 = t;
        }
        auto alive = [&](const NodeBox &nb, uint32_t ci, float e, float x, float dd) -> bool {
            if (dd == FLT_MAX)
                return false;
            const bool cleaf = (nb.count > 0u && nb.count <= 2u + lod) || nb.offset == 0xFFFFFFFFu;
            if (cleaf)
                return leaf_accepts(e, x, rmaxt, mint_eps, maxt_eps);
            if (cull_ok && x <= cull_eps) {
                V3 umn, umx;
                src.bound(ci, umn, umx);
                float ue, ux;
                slab_raw(umn, umx, o, d, ue, ux);
                if (!(ue <= ux) || ux <= cull_eps || ue >= rmaxt)
                    return false;
            }
            return true;
        };
        const bool a1 = alive(n1, c1, e1, x1, d1);
        const bool a2 = alive(n2, c2, e2, x2, d2);
        if (a1) {
            node_idx = c1;
            node = n1;
            cur_e = e1;
            cur_x = x1;
            have_slab = true;
            if (a2) {
                stack[sp++] = c2;
                if (sp >= 24)
                    return -1;
            }
        } else if (a2) {
            node_idx = c2;
            node = n2;
            cur_e = e2;
            cur_x = x2;
            have_slab = true;
        } else {
            if (sp == 0)
                return 0;
            node_idx = stack[--sp];
            node = src.node(node_idx);
            have_slab = false;
        }
    }
}

// Segment encoding into the hash-grid unit cube, src/cuda/neural/neural_bvh_module_kernels.cu:48-55
__device__ __forceinline__ V3 encode_world(V3 p, V3 center, V3 ext) { return adds3(div3(sub3(p, center), ext), 0.5f); }

// decode_depth_estimate, LocalT, include/cuda/neural/neural_bvh_module_common.cuh:23-58 (the 1e-3
// literal is a double in the reference, so those expressions are evaluated in double)
__device__ __forceinline__ float decode_local_t(float out_depth, float mint, float maxt, bool inside, float depth_epsilon,
                                                float fixed_depth_epsilon)
{
    float seg_len = __fsub_rn(maxt, mint);
    float u = gclamp01(out_depth);
    float depth = FLT_MAX;
    if (inside) {
        if (depth_epsilon != 1.0f) {
            float inward = __double2float_rn(__dmul_rn((double)u, __dadd_rn((double)seg_len, 1e-3)));
            if (inward < __fsub_rn(__fsub_rn(maxt, __fmul_rn(seg_len, depth_epsilon)), fixed_depth_epsilon))
                depth = __fsub_rn(maxt, inward);
        }
    } else {
        depth = __double2float_rn(__dadd_rn(__dmul_rn((double)u, __dadd_rn((double)seg_len, 1e-3)), (double)mint));
    }
    return depth;
}

// NeuralTreeCutData::compute_loss_heuristic (include/cuda/neural/neural_bvh_renderer.h:36-47):
// loss / (iter_alive * sqrt(samples / iter_alive)), -FLT_MAX for a node without samples.
__device__ __forceinline__ float tree_cut_heuristic(float loss, uint32_t iter_alive, uint32_t samples)
{
    if (samples == 0u)
        return -FLT_MAX;
    const float alive = __uint2float_rn(iter_alive);
    return __fdiv_rn(loss, __fmul_rn(alive, __fsqrt_rn(__fdiv_rn(__uint2float_rn(samples), alive))));
}

// Round to the nearest FP8 E4M3 value (ties to even), saturating at +-448 (the "satfinite"
// convention: E4M3 has no infinity). 4 exponent bits (bias 7), 3 mantissa bits, subnormals on the
// 2^-9 grid below 2^-6. The same integer/float steps run on the host in the CPU restatement.
__host__ __device__ inline float e4m3_round(float x)
{
    uint32_t b;
    memcpy(&b, &x, 4);
    const uint32_t sign = b & 0x80000000u;
    uint32_t a = b & 0x7FFFFFFFu;
    if (a > 0x7F800000u)
        return x; // NaN
    float r;
    if (a >= 0x43E00000u) { // |x| >= 448
        a = 0x43E00000u;
        memcpy(&r, &a, 4);
    } else if (a < 0x3C800000u) { // |x| < 2^-6: the subnormal grid
        float m;
        memcpy(&m, &a, 4);
        r = rintf(m * 512.0f) * (1.0f / 512.0f);
    } else {
        const uint32_t lsb = (a >> 20) & 1u;
        a = (a + 0x7FFFFu + lsb) & 0xFFF00000u;
        if (a > 0x43E00000u)
            a = 0x43E00000u;
        memcpy(&r, &a, 4);
    }
    uint32_t rb;
    memcpy(&rb, &r, 4);
    rb |= sign;
    memcpy(&r, &rb, 4);
    return r;
}

// Scale of the hidden weight matrices in FP8 mode: w8 = e4m3(w * 2^6) / 2^6 (|w| up to 7 kept,
// normal values from 2^-12); every such value is exact in FP16.
constexpr float kFp8WeightScale = 64.0f;
// Scale of the activations entering the hidden matrices in FP8 mode: a8 = e4m3(a * 2^7) / 2^7
// (values up to 3.5, normal from 2^-13; without it the small activations of an untrained network
// round to zero and their ReLU gradients vanish).
constexpr float kFp8ActScale = 128.0f;

} // namespace nbvh
