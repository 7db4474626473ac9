// device_math.cuh -- FP32 vector arithmetic with glm's evaluation order and no FMA contraction,
// the reference RNG, and the ray/box and ray/triangle tests, for the bit-exact parts of the
// kernels (classic and neural traversal, training-ray sampling).
//
// Every operation is an explicitly rounded intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn) so that nvcc cannot fuse it, and the order follows glm: dot = (x*x' + y*y') + z*z',
// cross = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y), min(a, b) = b < a ? b : a,
// max(a, b) = a < b ? b : a, normalize(v) = v * (1 / sqrt(dot(v, v))).
#pragma once

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

// BVH2Node::intersect, include/base/accel/bvh.h:121-133
__device__ __forceinline__ float box_entry(V3 bmin, V3 bmax, V3 o, V3 d, float rmint, float rmaxt)
{
    V3 t0 = div3(sub3(bmin, o), d);
    V3 t1 = div3(sub3(bmax, o), d);
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
                                                 float &best_v, uint32_t &best_prim, uint32_t *best_rec = nullptr)
{
    best_t = FLT_MAX;
    best_u = 0.f;
    best_v = 0.f;
    best_prim = 0xFFFFFFFFu;
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
        float d1 = box_entry(n1.mn, n1.mx, o, d, rmint, rmaxt);
        float d2 = box_entry(n2.mn, n2.mx, o, d, rmint, rmaxt);
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
// -1 on a stack overflow (the reference prints and returns false).
template <typename Stack>
__device__ __forceinline__ int neural_intersect(const float4 *__restrict__ nodes, uint32_t lod, V3 o, V3 d, Stack &stack,
                                                int &sp, bool inference, float mint_eps_inf, float maxt_eps_inf,
                                                float mint_eps_learn, float maxt_eps_learn, float current_maxt,
                                                float dil, float &seg_mint, float &seg_maxt, uint32_t &seg_node)
{
    const float rmint = -FLT_MAX, rmaxt = current_maxt;
    uint32_t node_idx = stack[--sp];
    for (;;) {
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

} // namespace nbvh
