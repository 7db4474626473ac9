// k_classic.cu -- K1: classic BVH2 closest-hit / any-hit queries (the plain method and the judge).
//
// One thread per ray. Ray records are read with two 128-bit loads, a node pair (both children of
// an interior node are adjacent) with four, a pre-gathered triangle record {v0|prim, e1, e2} with
// three; hits are written with one 128-bit store. The traversal order and every FP32 operation
// follow CudaBVH2::intersect (include/cuda/accel/bvh2.cuh:12-88) and
// BaseCudaBLAS::intersect_triangle (include/cuda/accel/bvh.cuh:98-136), so prim, t, u and v are
// bit-identical to the CPU restatement of the same code on the same BVH. The slab divisions use
// the prepared-ray form (a correctly rounded reciprocal per ray and Markstein's FMA correction)
// when the ray and the scene lie in its exact domain.
#include "device_math.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

__device__ __forceinline__ void load_ray(const nbvh_ray *rays, uint32_t i, V3 &o, float &tmin, V3 &d, float &tmax)
{
    const float4 *r = reinterpret_cast<const float4 *>(rays + i);
    float4 a = __ldg(r);
    float4 b = __ldg(r + 1);
    o = mk3(a.x, a.y, a.z);
    tmin = a.w;
    d = mk3(b.x, b.y, b.z);
    tmax = b.w;
}

template <bool ANY_HIT>
__global__ void __launch_bounds__(128) k_classic(const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                 const nbvh_ray *__restrict__ rays, uint32_t n,
                                                 nbvh_hit *__restrict__ hits, const uint32_t *__restrict__ ray_list,
                                                 bool fast_div)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t ray_id = ray_list ? ray_list[i] : i;
    V3 o, d;
    float tmin, tmax;
    load_ray(rays, ray_id, o, tmin, d, tmax);
    float t, u, v;
    uint32_t prim;
    classic_traverse<ANY_HIT>(nodes, tris, o, d, tmin, tmax, t, u, v, prim, nullptr, fast_div);
    reinterpret_cast<float4 *>(hits)[ray_id] = make_float4(t, u, v, __uint_as_float(prim));
}

// Classic answers written into neural hit records: for ignore_neural_blas (every ray) and for the
// fallback list of the neural query (rays whose leaf is non-neural or whose visibility is within
// the confidence margin of the threshold).
template <bool ANY_HIT>
__global__ void __launch_bounds__(128) k_classic_to_neural(const float4 *__restrict__ nodes,
                                                           const float4 *__restrict__ tris,
                                                           const nbvh_ray *__restrict__ rays, uint32_t n,
                                                           const uint32_t *__restrict__ list,
                                                           const QueryCounters *__restrict__ counters,
                                                           nbvh_neural_hit *__restrict__ hits, bool fast_div)
{
    uint32_t count = list ? min(counters->fallback_count, n) : n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        uint32_t ray_id = list ? list[i] : i;
        V3 o, d;
        float tmin, tmax;
        load_ray(rays, ray_id, o, tmin, d, tmax);
        float t, u, v;
        uint32_t prim;
        classic_traverse<ANY_HIT>(nodes, tris, o, d, tmin, tmax, t, u, v, prim, nullptr, fast_div);
        float4 *out = reinterpret_cast<float4 *>(hits + ray_id);
        uint32_t prev_segments = list ? hits[ray_id].segments : 0u;
        uint32_t prev_flags = list ? (hits[ray_id].flags & ~NBVH_HIT_VALID) : 0u;
        uint32_t flags = (prim != 0xFFFFFFFFu ? NBVH_HIT_VALID : 0u) | NBVH_HIT_CLASSIC_FALLBACK | prev_flags;
        out[0] = make_float4(t, 0.f, 0.f, 0.f);
        out[1] = make_float4(0.f, 0.f, 0.f, 0.f);
        out[2] = make_float4(__uint_as_float(flags), __uint_as_float(prev_segments), __uint_as_float(prim), 0.f);
    }
}

} // namespace

cudaError_t launch_classic(const float4 *nodes, const float4 *tris, const nbvh_ray *rays, uint32_t n, nbvh_hit *hits,
                           bool any_hit, const uint32_t *ray_list, bool fast_div, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    dim3 block(128), grid((n + 127u) / 128u);
    if (any_hit)
        k_classic<true><<<grid, block, 0, s>>>(nodes, tris, rays, n, hits, ray_list, fast_div);
    else
        k_classic<false><<<grid, block, 0, s>>>(nodes, tris, rays, n, hits, ray_list, fast_div);
    return cudaGetLastError();
}

cudaError_t launch_classic_fallback(const float4 *nodes, const float4 *tris, const nbvh_ray *rays, const uint32_t *list,
                                    const QueryCounters *counters, uint32_t max_list, nbvh_neural_hit *hits,
                                    bool any_hit, bool fast_div, int num_sms, cudaStream_t s)
{
    if (max_list == 0)
        return cudaSuccess;
    uint32_t blocks = (uint32_t)num_sms * 8u;
    uint32_t need = (max_list + 127u) / 128u;
    if (need < blocks)
        blocks = need;
    if (any_hit)
        k_classic_to_neural<true><<<blocks, 128, 0, s>>>(nodes, tris, rays, max_list, list, counters, hits, fast_div);
    else
        k_classic_to_neural<false><<<blocks, 128, 0, s>>>(nodes, tris, rays, max_list, list, counters, hits, fast_div);
    return cudaGetLastError();
}

cudaError_t launch_classic_as_neural(const float4 *nodes, const float4 *tris, const nbvh_ray *rays, uint32_t n,
                                     nbvh_neural_hit *hits, bool any_hit, bool fast_div, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    uint32_t blocks = (n + 127u) / 128u;
    if (any_hit)
        k_classic_to_neural<true><<<blocks, 128, 0, s>>>(nodes, tris, rays, n, nullptr, nullptr, hits, fast_div);
    else
        k_classic_to_neural<false><<<blocks, 128, 0, s>>>(nodes, tris, rays, n, nullptr, nullptr, hits, fast_div);
    return cudaGetLastError();
}

} // namespace nbvh
