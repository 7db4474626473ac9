// k_neural.cu -- stand-alone kernels of the neural path: the N-BVH segment enumeration (K2 alone)
// and the hash-grid encoding (K3 forward alone, FP32 features). Network inference on explicit
// positions is the training encoder's FP16 rows followed by the tcgen05 MLP (k_train.cu,
// k_mlp_tc.cu); the neural closest-hit query itself is the wavefront in k_query.cu.
#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

// Every leaf segment a ray enters with current_maxt = FLT_MAX (NeuralBVH2::intersect alone, on the
// same pre-dilated, culling traversal the query kernel uses).
__global__ void __launch_bounds__(128) k_segments(const float4 *__restrict__ nodes, const float4 *__restrict__ bounds,
                                                  NeuralConsts nc, const nbvh_ray *__restrict__ rays, uint32_t n,
                                                  uint32_t max_segments, nbvh_segment *__restrict__ segs,
                                                  uint32_t *__restrict__ counts)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float4 *r = reinterpret_cast<const float4 *>(rays + i);
    float4 ra = __ldg(r), rb = __ldg(r + 1);
    V3 o = mk3(ra.x, ra.y, ra.z), d = mk3(rb.x, rb.y, rb.z);
    const bool cull_ok = d.x != 0.0f && d.y != 0.0f && d.z != 0.0f;
    const RayDiv rdiv = make_raydiv(o, d, nc.fast_div_ok != 0u);
    uint32_t stack[kNeuralStackSize];
    int sp = 1;
    stack[0] = 0;
    uint32_t cnt = 0;
    while (sp > 0) {
        float mint, maxt;
        uint32_t nd;
        const GlobalCut cut{nodes, bounds};
        int res = neural_intersect_inference(cut, nc.bvh_lod, o, rdiv, cull_ok, stack, sp,
                                             nc.inference_mint_epsilon, nc.inference_maxt_epsilon, FLT_MAX, mint,
                                             maxt, nd);
        if (res != 1)
            break;
        if (cnt < max_segments) {
            nbvh_segment s;
            s.mint = mint;
            s.maxt = maxt;
            s.node = nd;
            s.reserved = 0;
            segs[(size_t)i * max_segments + cnt] = s;
        }
        cnt++;
    }
    counts[i] = cnt;
}

// Hash-grid features (FP32 before the FP16 rounding), one thread per (row, point, level); level l
// of a point's block holds its F features at l * F.
__global__ void __launch_bounds__(128) k_encode(const __grid_constant__ GridParams grid, const uint32_t *__restrict__ table,
                                                const float *__restrict__ positions, uint32_t n,
                                                float *__restrict__ features)
{
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t total = (uint64_t)n * grid.n_points * grid.n_levels;
    if (i >= total)
        return;
    const uint32_t F = grid.n_features;
    uint32_t l = (uint32_t)(i % grid.n_levels);
    uint64_t rp = i / grid.n_levels; // row * points + point
    const float *src = positions + rp * 3u;
    const V3 p = mk3(src[0], src[1], src[2]);
    float *dst = features + (rp * grid.n_levels + l) * F;
    if (F == 4u) {
        float f[4];
        encode_level_wide<4>(table, grid, l, p, f);
        for (uint32_t k = 0; k < 4u; k++)
            dst[k] = f[k];
    } else if (F == 8u) {
        float f[8];
        encode_level_wide<8>(table, grid, l, p, f);
        for (uint32_t k = 0; k < 8u; k++)
            dst[k] = f[k];
    } else {
        const float2 f = encode_level<true>(table, grid, l, p);
        dst[0] = f.x;
        dst[1] = f.y;
    }
}


} // namespace

cudaError_t launch_segments(const float4 *dilated_nodes, const float4 *bounds, const NeuralConsts &nc,
                            const nbvh_ray *rays, uint32_t n, uint32_t max_segments, nbvh_segment *segs,
                            uint32_t *counts, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    k_segments<<<(n + 127u) / 128u, 128, 0, s>>>(dilated_nodes, bounds, nc, rays, n, max_segments, segs, counts);
    return cudaGetLastError();
}

cudaError_t launch_encode(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                          const float *positions, uint32_t n, float *features, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    uint32_t n_network_params = kNeurons * grid.n_inputs + (n_hidden_layers - 1u) * kNeurons * kNeurons +
                                kOutputsPadded * kNeurons;
    const uint32_t *table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    uint64_t total = (uint64_t)n * grid.n_points * grid.n_levels;
    k_encode<<<(unsigned)((total + 127u) / 128u), 128, 0, s>>>(grid, table, positions, n, features);
    return cudaGetLastError();
}

} // namespace nbvh
