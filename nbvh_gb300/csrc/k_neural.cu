// k_neural.cu -- stand-alone kernels of the neural path: the N-BVH segment enumeration (K2 alone),
// hash-grid encoding (K3 forward alone) and network inference on explicit positions (K3 + K4
// forward). The neural closest-hit query itself is the wavefront in k_query.cu.
#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

__device__ __forceinline__ void copy_grid_params(GridParams &dst, const GridParams &src)
{
    const uint32_t *s = reinterpret_cast<const uint32_t *>(&src);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (uint32_t i = threadIdx.x; i < sizeof(GridParams) / 4u; i += blockDim.x)
        d[i] = s[i];
}

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

struct InferArgs {
    GridParams grid;
    const uint32_t *table;
    const __half *weights;
    const float *positions;
    float *outputs;
    uint32_t n_hidden_layers;
    uint32_t n;
    uint32_t fp8;
};

// Network inference on explicit encoded positions: one warp per 16-row tile, grid-stride.
template <bool BF16, bool FP8>
__global__ void __launch_bounds__(kThreads, 2) k_network_inference(const __grid_constant__ InferArgs args)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GridParams &gp = *reinterpret_cast<GridParams *>(smem_raw);
    const uint32_t n_inputs = args.grid.n_inputs, P = args.grid.n_points, L = args.grid.n_levels;
    __half *sw = reinterpret_cast<__half *>(smem_raw + kGridParamsSmem);
    const SmemNetLayout SL = smem_net_layout(n_inputs, args.n_hidden_layers);
    const uint32_t fld = n_inputs + 8u;
    __half *feat = sw + SL.total + (size_t)(threadIdx.x >> 5) * 16u * fld; // per-warp feature tile
    copy_grid_params(gp, args.grid);
    load_weights_to_smem(args.weights, sw, n_inputs, args.n_hidden_layers);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const uint32_t warps_total = gridDim.x * kWarps;
    const uint32_t n_tiles = (args.n + 15u) / 16u;
    (void)L;
    for (uint32_t tile = blockIdx.x * kWarps + (threadIdx.x >> 5); tile < n_tiles; tile += warps_total) {
        const uint32_t r0 = tile * 16u + g, r1 = r0 + 8u;
        const bool act0 = r0 < args.n, act1 = r1 < args.n;
        const uint32_t rows = args.n - tile * 16u;
        const uint32_t mask = rows >= 16u ? 0xFFFFu : ((1u << rows) - 1u);
        auto pos = [&](uint32_t r, uint32_t p) -> V3 {
            const float *src = args.positions + ((size_t)(tile * 16u + r) * P + p) * 3u;
            return mk3(__ldg(src), __ldg(src + 1), __ldg(src + 2));
        };
        encode_tile_any<BF16>(args.table, gp, pos, mask, feat, fld);
        float o4[4];
        mlp_tile_from_smem<BF16, FP8>(sw, feat, fld, n_inputs, args.n_hidden_layers, o4);
        __syncwarp();
        if (act0) {
            args.outputs[(size_t)r0 * 8u + tig * 2] = o4[0];
            args.outputs[(size_t)r0 * 8u + tig * 2 + 1] = o4[1];
        }
        if (act1) {
            args.outputs[(size_t)r1 * 8u + tig * 2] = o4[2];
            args.outputs[(size_t)r1 * 8u + tig * 2 + 1] = o4[3];
        }
    }
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
        const float2 f = encode_level(table, grid, l, p);
        dst[0] = f.x;
        dst[1] = f.y;
    }
}

template <typename K>
cudaError_t prepare_smem(K kernel, size_t bytes)
{
    (void)bytes; // every launch stays below the common limit
    return allow_max_dynamic_smem(kernel);
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

cudaError_t launch_network_inference(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                                     const float *positions, uint32_t n, float *outputs, uint32_t prec, int num_sms,
                                     cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    const bool bf16 = prec == NBVH_PRECISION_BF16;
    InferArgs a;
    a.fp8 = prec == NBVH_PRECISION_FP8 ? 1u : 0u;
    a.grid = grid;
    uint32_t n_network_params = kNeurons * grid.n_inputs + (n_hidden_layers - 1u) * kNeurons * kNeurons +
                                kOutputsPadded * kNeurons;
    a.table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    a.weights = params_h;
    a.positions = positions;
    a.outputs = outputs;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    size_t smem = kGridParamsSmem + smem_net_layout(grid.n_inputs, n_hidden_layers).total * sizeof(__half) +
                  (size_t)kWarps * 16u * (grid.n_inputs + 8u) * sizeof(__half);
    const bool fp8 = a.fp8 != 0u;
    cudaError_t e = bf16  ? prepare_smem(k_network_inference<true, false>, smem)
                    : fp8 ? prepare_smem(k_network_inference<false, true>, smem)
                          : prepare_smem(k_network_inference<false, false>, smem);
    if (e != cudaSuccess)
        return e;
    uint32_t tiles = (n + 15u) / 16u;
    uint32_t blocks = (tiles + kWarps - 1u) / kWarps;
    uint32_t cap = (uint32_t)num_sms * 2u;
    if (blocks > cap)
        blocks = cap;
    if (bf16)
        k_network_inference<true, false><<<blocks, kThreads, smem, s>>>(a);
    else if (fp8)
        k_network_inference<false, true><<<blocks, kThreads, smem, s>>>(a);
    else
        k_network_inference<false, false><<<blocks, kThreads, smem, s>>>(a);
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
