// k_path.cu -- hybrid path tracing over a neural BLAS: camera paths, Lambertian bounces on the
// surfaces the neural query returns (albedo and normal from the network), a classic analytic
// ground plane, and an analytic sky as the only light.
//
// The reference's path module (src/cuda/neural/path/path_inference_kernels.cu:224-429, scatter +
// next traversal; raygen 540-567) drives a Disney BSDF over a TLAS; this restates the Lambertian
// case as a wavefront: raygen -> [neural query -> shade/scatter with compaction] per bounce ->
// resolve. Paths that leave the scene collect sky radiance weighted by their throughput.
#include "device_math.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

// Duff et al., "Building an Orthonormal Basis, Revisited", JCGT 6(1), 2017.
__device__ __forceinline__ void onb(V3 n, V3 &t, V3 &b)
{
    const float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sign + n.z);
    const float c = n.x * n.y * a;
    t = mk3(1.0f + sign * n.x * n.x * a, sign * c, -sign * n.x);
    b = mk3(c, sign + n.y * n.y * a, -n.y);
}

// Cosine-weighted direction about n (Malley's method: uniform disk point lifted to the hemisphere).
__device__ __forceinline__ V3 cosine_sample(V3 n, uint32_t &rng)
{
    const float u1 = lcg_randomf(rng), u2 = lcg_randomf(rng);
    float sp, cp;
    sincos_turns(u2, sp, cp);
    const float r = sqrtf(u1), z = sqrtf(fmaxf(0.0f, 1.0f - u1));
    V3 t, b;
    onb(n, t, b);
    return mk3(r * cp * t.x + r * sp * b.x + z * n.x, r * cp * t.y + r * sp * b.y + z * n.y,
               r * cp * t.z + r * sp * b.z + z * n.z);
}

__device__ __forceinline__ uint32_t warp_append(bool want, uint32_t *counter)
{
    const unsigned m = __ballot_sync(kFull, want);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (m != 0u) {
        const int leader = __ffs(m) - 1;
        if (lane == leader)
            base = atomicAdd(counter, (uint32_t)__popc(m));
        base = __shfl_sync(kFull, base, leader);
    }
    return base + __popc(m & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(256) k_pt_raygen(const __grid_constant__ PathArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; // path = pixel * spp + sample
    if (i >= a.n_paths)
        return;
    const uint32_t p = i / a.spp, smp = i - p * a.spp;
    const uint32_t px = p % a.width, py = p / a.width;
    // camera_raygen jitter (include/cuda/neural/neural_bvh_module_common.cuh:222-228) with the
    // sample index running over the frame's samples from sample_base
    uint32_t rng = lcg_seed(a.sample_base + smp, a.sample_offset, p);
    const float jx = lcg_randomf(rng), jy = lcg_randomf(rng);
    const float xf = __fdiv_rn(__fadd_rn((float)px, jx), (float)a.width);
    const float yf = __fdiv_rn(__fadd_rn((float)py, jy), (float)a.height);
    const V3 du = mk3(a.du[0], a.du[1], a.du[2]), dv = mk3(a.dv[0], a.dv[1], a.dv[2]),
             tl = mk3(a.tl[0], a.tl[1], a.tl[2]);
    const V3 d = normalize3(add3(add3(scale3(du, xf), scale3(dv, yf)), tl));
    float4 *r = reinterpret_cast<float4 *>(a.rays_out + i);
    r[0] = make_float4(a.origin[0], a.origin[1], a.origin[2], 1e-4f);
    r[1] = make_float4(d.x, d.y, d.z, FLT_MAX);
    a.ids_out[i] = i;
    a.thr[i] = make_float4(1.f, 1.f, 1.f, __uint_as_float(rng ^ (a.seed * 0x9E3779B9u)));
    a.rad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// One bounce: the nearer of the neural hit and the ground plane is shaded; misses collect sky
// radiance; surviving paths (bounce < max_bounces) are appended to the next list with a
// cosine-sampled direction about the surface normal facing the incoming ray.
__global__ void __launch_bounds__(256) k_pt_shade(const __grid_constant__ PathArgs a, uint32_t count_in, uint32_t bounce)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = j < count_in;
    bool keep = false;
    uint32_t id = 0;
    V3 o = mk3(0.f, 0.f, 0.f), nd = mk3(0.f, 0.f, 1.f);
    float4 th = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in) {
        id = a.ids_in[j];
        const float4 *r = reinterpret_cast<const float4 *>(a.rays_in + j);
        const float4 ra = r[0], rb = r[1];
        const V3 ro = mk3(ra.x, ra.y, ra.z), d = mk3(rb.x, rb.y, rb.z);
        const float4 *hp = reinterpret_cast<const float4 *>(a.hits + j);
        const float4 h0 = hp[0], h1 = hp[1], h2 = hp[2];
        const bool nhit = (__float_as_uint(h2.x) & NBVH_HIT_VALID) != 0u;
        float t = nhit ? h0.x : FLT_MAX;
        V3 n = mk3(h0.y, h0.z, h0.w), alb = mk3(h1.x, h1.y, h1.z);
        if (a.has_ground && d.y != 0.0f) {
            const float tp = (a.ground_y - ro.y) / d.y;
            if (tp > 1e-4f && tp < t) {
                t = tp;
                n = mk3(0.f, 1.f, 0.f);
                alb = mk3(a.ground_albedo[0], a.ground_albedo[1], a.ground_albedo[2]);
            }
        }
        th = a.thr[id];
        if (t == FLT_MAX) {
            const float w = fmaxf(d.y, 0.0f);
            float4 rad = a.rad[id];
            rad.x += th.x * (a.sky_horizon[0] + (a.sky_zenith[0] - a.sky_horizon[0]) * w);
            rad.y += th.y * (a.sky_horizon[1] + (a.sky_zenith[1] - a.sky_horizon[1]) * w);
            rad.z += th.z * (a.sky_horizon[2] + (a.sky_zenith[2] - a.sky_horizon[2]) * w);
            a.rad[id] = rad;
        } else if (bounce < a.max_bounces) {
            const float len = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
            n = len > 0.f ? mk3(n.x / len, n.y / len, n.z / len) : mk3(-d.x, -d.y, -d.z);
            if (n.x * d.x + n.y * d.y + n.z * d.z > 0.0f)
                n = mk3(-n.x, -n.y, -n.z);
            uint32_t rng = __float_as_uint(th.w);
            nd = cosine_sample(n, rng);
            th = make_float4(th.x * alb.x, th.y * alb.y, th.z * alb.z, __uint_as_float(rng));
            a.thr[id] = th;
            o = mk3(ro.x + t * d.x + 1e-3f * n.x, ro.y + t * d.y + 1e-3f * n.y, ro.z + t * d.z + 1e-3f * n.z);
            keep = th.x + th.y + th.z > 0.0f;
        }
    }
    const uint32_t pos = warp_append(keep, a.count_out);
    if (keep) {
        float4 *r = reinterpret_cast<float4 *>(a.rays_out + pos);
        r[0] = make_float4(o.x, o.y, o.z, 1e-4f);
        r[1] = make_float4(nd.x, nd.y, nd.z, FLT_MAX);
        a.ids_out[pos] = id;
    }
}

__global__ void __launch_bounds__(256) k_pt_resolve(const __grid_constant__ PathArgs a, float4 *__restrict__ image)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.width * a.height)
        return;
    float r = 0.f, g = 0.f, b = 0.f;
    for (uint32_t s = 0; s < a.spp; s++) {
        const float4 v = a.rad[p * a.spp + s];
        r += v.x;
        g += v.y;
        b += v.z;
    }
    const float inv = 1.0f / (float)a.spp;
    image[p] = make_float4(r * inv, g * inv, b * inv, 1.0f);
}

// ---------------------------------------------------------------------------------------------
// Instanced scenes: the rays of a bounce are tested against each instance's world box, the ones
// that enter it are moved into the instance's object space (o' = A^-1 (o - b), d' = A^-1 d
// normalised, t' = t * |A^-1 d|) and answered by its model's neural query, and the closest hit
// over the instances is kept in world space.
// ---------------------------------------------------------------------------------------------

// Batched by model: all (ray, instance) pairs of one model's instances in one list, answered by
// one query of that model; the closest entry per world ray is chosen with a 64-bit atomic min of
// (distance bits, entry index) and written by k_inst_finalize.
__global__ void __launch_bounds__(256) k_inst_prepare_group(const InstanceArgs *__restrict__ group, uint32_t n_group,
                                                            const nbvh_ray *rays, uint32_t n, nbvh_ray *obj_rays,
                                                            uint32_t *obj_ids, float *obj_scale, uint32_t *obj_inst,
                                                            uint32_t *count, uint32_t capacity)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float4 ra = make_float4(0.f, 0.f, 0.f, 0.f), rb = ra;
    if (i < n) {
        const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
        ra = rp[0];
        rb = rp[1];
    }
    const float o[3] = {ra.x, ra.y, ra.z}, d[3] = {rb.x, rb.y, rb.z};
    for (uint32_t gi = 0; gi < n_group; gi++) {
        const InstanceArgs &a = group[gi];
        bool want = false;
        nbvh_ray r{};
        float sc = 1.0f;
        if (i < n) {
            float t0 = ra.w, t1 = rb.w;
            bool hit = t0 < t1;
            for (int k = 0; k < 3 && hit; k++) {
                if (d[k] == 0.0f) {
                    hit = o[k] >= a.box_min[k] && o[k] <= a.box_max[k];
                } else {
                    const float inv = 1.0f / d[k];
                    float ta = (a.box_min[k] - o[k]) * inv, tb = (a.box_max[k] - o[k]) * inv;
                    if (ta > tb) {
                        const float t = ta;
                        ta = tb;
                        tb = t;
                    }
                    t0 = fmaxf(t0, ta);
                    t1 = fminf(t1, tb);
                    hit = t0 <= t1;
                }
            }
            if (hit) {
                want = true;
                if (a.identity) {
                    for (int k = 0; k < 3; k++) {
                        r.o[k] = o[k];
                        r.d[k] = d[k];
                    }
                } else {
                    const float q[3] = {o[0] - a.xform[3], o[1] - a.xform[7], o[2] - a.xform[11]};
                    float dd[3];
                    for (int row = 0; row < 3; row++) {
                        r.o[row] = a.inv[3 * row] * q[0] + a.inv[3 * row + 1] * q[1] + a.inv[3 * row + 2] * q[2];
                        dd[row] = a.inv[3 * row] * d[0] + a.inv[3 * row + 1] * d[1] + a.inv[3 * row + 2] * d[2];
                    }
                    sc = sqrtf(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                    for (int k = 0; k < 3; k++)
                        r.d[k] = dd[k] / sc;
                }
                r.tmin = ra.w * sc;
                r.tmax = FLT_MAX;
            }
        }
        const uint32_t pos = warp_append(want, count);
        if (want && pos < capacity) {
            obj_rays[pos] = r;
            obj_ids[pos] = i;
            obj_scale[pos] = sc;
            obj_inst[pos] = a.instance;
        }
    }
}

__global__ void __launch_bounds__(256) k_inst_reset(unsigned long long *keys, nbvh_neural_hit *hits, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    keys[i] = ~0ull;
    float4 *o = reinterpret_cast<float4 *>(hits + i);
    o[0] = make_float4(FLT_MAX, 0.f, 0.f, 0.f);
    o[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    o[2] = make_float4(0.f, 0.f, __uint_as_float(0xFFFFFFFFu), __uint_as_float(0xFFFFFFFFu));
}

__global__ void __launch_bounds__(256) k_inst_vote(const nbvh_neural_hit *obj_hits, const uint32_t *obj_ids,
                                                   const float *obj_scale, uint32_t total, unsigned long long *keys,
                                                   nbvh_neural_hit *hits)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= total)
        return;
    const nbvh_neural_hit oh = obj_hits[k];
    const uint32_t i = obj_ids[k];
    atomicAdd(&hits[i].segments, oh.segments);
    const uint32_t trav = oh.flags & (NBVH_HIT_STEP_CAP | 0x8u); // step cap, stack overflow: from any entry
    if (trav)
        atomicOr(&hits[i].flags, trav);
    if (!(oh.flags & NBVH_HIT_VALID))
        return;
    const float t = oh.t / obj_scale[k];
    const uint32_t b = __float_as_uint(t);
    const uint32_t ord = (b & 0x80000000u) ? ~b : (b | 0x80000000u); // orders as the float
    atomicMin(keys + i, ((unsigned long long)ord << 32) | k);
}

__global__ void __launch_bounds__(256) k_inst_finalize(const InstanceArgs *__restrict__ all, const nbvh_neural_hit *obj_hits,
                                                       const float *obj_scale, const uint32_t *obj_inst,
                                                       const unsigned long long *keys, uint32_t n, nbvh_neural_hit *hits)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const unsigned long long key = keys[i];
    if (key == ~0ull)
        return;
    const uint32_t k = (uint32_t)(key & 0xFFFFFFFFull);
    const nbvh_neural_hit oh = obj_hits[k];
    const InstanceArgs &a = all[obj_inst[k]];
    float nrm[3] = {oh.normal[0], oh.normal[1], oh.normal[2]};
    if (!a.identity) {
        float m[3];
        for (int row = 0; row < 3; row++) // inverse transpose: column `row` of A^-1
            m[row] = a.inv[row] * nrm[0] + a.inv[3 + row] * nrm[1] + a.inv[6 + row] * nrm[2];
        const float len = sqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        for (int c = 0; c < 3; c++)
            nrm[c] = len > 0.f ? m[c] / len : m[c];
    }
    nbvh_neural_hit &w = hits[i];
    const uint32_t ord = (uint32_t)(key >> 32);
    w.t = __uint_as_float((ord & 0x80000000u) ? (ord & 0x7FFFFFFFu) : ~ord);
    w.normal[0] = nrm[0];
    w.normal[1] = nrm[1];
    w.normal[2] = nrm[2];
    w.albedo[0] = oh.albedo[0];
    w.albedo[1] = oh.albedo[1];
    w.albedo[2] = oh.albedo[2];
    w.visibility = oh.visibility;
    w.flags = (w.flags & (NBVH_HIT_STEP_CAP | 0x8u)) | oh.flags;
    w.prim = oh.prim;
    w.reserved = a.instance;
}

} // namespace

cudaError_t launch_inst_group(const InstanceArgs *group, uint32_t n_group, const nbvh_ray *rays, uint32_t n,
                              nbvh_ray *obj_rays, uint32_t *obj_ids, float *obj_scale, uint32_t *obj_inst,
                              uint32_t *count, uint32_t capacity, cudaStream_t s)
{
    if (n == 0 || n_group == 0)
        return cudaSuccess;
    k_inst_prepare_group<<<(n + 255u) / 256u, 256, 0, s>>>(group, n_group, rays, n, obj_rays, obj_ids, obj_scale,
                                                           obj_inst, count, capacity);
    return cudaGetLastError();
}

cudaError_t launch_inst_reset(unsigned long long *keys, nbvh_neural_hit *hits, uint32_t n, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    k_inst_reset<<<(n + 255u) / 256u, 256, 0, s>>>(keys, hits, n);
    return cudaGetLastError();
}

cudaError_t launch_inst_vote_finalize(const InstanceArgs *all, const nbvh_neural_hit *obj_hits, const uint32_t *obj_ids,
                                      const float *obj_scale, const uint32_t *obj_inst, uint32_t total,
                                      unsigned long long *keys, nbvh_neural_hit *hits, uint32_t n, cudaStream_t s)
{
    if (total > 0)
        k_inst_vote<<<(total + 255u) / 256u, 256, 0, s>>>(obj_hits, obj_ids, obj_scale, total, keys, hits);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || n == 0)
        return e;
    k_inst_finalize<<<(n + 255u) / 256u, 256, 0, s>>>(all, obj_hits, obj_scale, obj_inst, keys, n, hits);
    return cudaGetLastError();
}

cudaError_t launch_path_raygen(const PathArgs &a, cudaStream_t s)
{
    if (a.n_paths == 0)
        return cudaSuccess;
    k_pt_raygen<<<(a.n_paths + 255u) / 256u, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_path_shade(const PathArgs &a, uint32_t count_in, uint32_t bounce, cudaStream_t s)
{
    if (count_in == 0)
        return cudaSuccess;
    k_pt_shade<<<(count_in + 255u) / 256u, 256, 0, s>>>(a, count_in, bounce);
    return cudaGetLastError();
}

cudaError_t launch_path_resolve(const PathArgs &a, float *image, cudaStream_t s)
{
    const uint32_t n = a.width * a.height;
    if (n == 0)
        return cudaSuccess;
    k_pt_resolve<<<(n + 255u) / 256u, 256, 0, s>>>(a, reinterpret_cast<float4 *>(image));
    return cudaGetLastError();
}

} // namespace nbvh
