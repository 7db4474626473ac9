// k_neural.cu -- K2 (N-BVH traversal + compaction), K3 (hash-grid encoding, forward) and K4
// (fused MLP, forward) fused into one persistent inference kernel, plus the stand-alone
// segment, encoding and network-inference kernels used by the tests and the C API.
//
// The reference runs this path as a host loop of three launches and a device-to-host sync per
// traversal step (NeuralPathModule::neural_bvh_traversal, src/cuda/neural/path/path_module.cu:
// 54-137), materialising FP32 network inputs/outputs and each ray's stack in global memory. Here
// every warp owns 32 ray slots for the whole kernel: lane i traverses slot i's ray (its stack
// lives in thread-local memory), the warp evaluates the 32 entered leaf segments as two 16-row
// MLP tiles on the tensor cores (the hash-grid features are gathered straight into the A-operand
// fragments), and finished rays are replaced from a global queue (one atomicAdd per warp refill,
// lanes ranked by ballot/popc), so tiles stay full without any host round trip.
#include <type_traits>

#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr unsigned kFull = 0xFFFFFFFFu;

struct QueryArgs {
    GridParams grid;
    NeuralConsts nc;
    const float4 *nodes;  // pre-dilated inference copy of the cut
    const float4 *bounds; // union of dilated leaf boxes per node
    const uint8_t *non_neural;
    const uint32_t *table;
    const __half *weights;
    const nbvh_ray *rays;
    nbvh_neural_hit *hits;
    QueryCounters *counters;
    uint32_t *fallback_list;
    uint32_t n_hidden_layers;
    uint32_t n;
    uint32_t n_cut_nodes;
};

__device__ __forceinline__ void write_hit(nbvh_neural_hit *hits, uint32_t id, float t, V3 nrm, V3 alb, float vis,
                                          uint32_t flags, uint32_t segments)
{
    float4 *out = reinterpret_cast<float4 *>(hits + id);
    out[0] = make_float4(t, nrm.x, nrm.y, nrm.z);
    out[1] = make_float4(alb.x, alb.y, alb.z, vis);
    out[2] = make_float4(__uint_as_float(flags), __uint_as_float(segments), __uint_as_float(kInvalid), 0.f);
}

__device__ __forceinline__ void copy_grid_params(GridParams &dst, const GridParams &src)
{
    const uint32_t *s = reinterpret_cast<const uint32_t *>(&src);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (uint32_t i = threadIdx.x; i < sizeof(GridParams) / 4u; i += blockDim.x)
        d[i] = s[i];
}

// One CTA of 16 warps per SM; each warp owns 32 ray slots. Shared memory: grid geometry, the padded
// FP16 network, optionally the pre-dilated cut (2 float4 per node) and its subtree bounds (3 float2
// per node), then 32 x (points * 3 + 8) floats of per-warp scratch.
constexpr int kQWarps = 16;
constexpr int kQThreads = kQWarps * 32;

template <bool SMEM_CUT>
__global__ void __launch_bounds__(kQThreads, 1) k_neural_query(const __grid_constant__ QueryArgs args)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GridParams &gp = *reinterpret_cast<GridParams *>(smem_raw);
    const uint32_t n_inputs = args.grid.n_inputs, P = args.grid.n_points, L = args.grid.n_levels;
    const SmemNetLayout SL = smem_net_layout(n_inputs, args.n_hidden_layers);
    __half *sw = reinterpret_cast<__half *>(smem_raw + sizeof(GridParams));
    unsigned char *after_net = reinterpret_cast<unsigned char *>(sw + SL.total);
    const uint32_t cut_bytes = SMEM_CUT ? args.n_cut_nodes * 56u : 0u;
    float *warp_area = reinterpret_cast<float *>(after_net + cut_bytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *pts = warp_area + (size_t)warp * 32u * (P * 3u + 8u); // [32][P*3]
    float *outs = pts + 32u * P * 3u;                            // [32][8]

    copy_grid_params(gp, args.grid);
    load_weights_to_smem(args.weights, sw, n_inputs, args.n_hidden_layers);
    float4 *s_nodes = reinterpret_cast<float4 *>(after_net);
    float2 *s_bounds = reinterpret_cast<float2 *>(after_net + args.n_cut_nodes * 32u);
    if (SMEM_CUT) {
        for (uint32_t i = threadIdx.x; i < 2u * args.n_cut_nodes; i += blockDim.x)
            s_nodes[i] = __ldg(args.nodes + i);
        for (uint32_t i = threadIdx.x; i < args.n_cut_nodes; i += blockDim.x) {
            const float4 a = __ldg(args.bounds + 2u * i), b = __ldg(args.bounds + 2u * i + 1u);
            s_bounds[3u * i] = make_float2(a.x, a.y);
            s_bounds[3u * i + 1u] = make_float2(a.z, b.x);
            s_bounds[3u * i + 2u] = make_float2(b.y, b.z);
        }
    }
    __syncthreads();
    using Cut = typename std::conditional<SMEM_CUT, SharedCut, GlobalCut>::type;
    Cut cut;
    if constexpr (SMEM_CUT) {
        cut.nodes = s_nodes;
        cut.bounds = s_bounds;
    } else {
        cut.nodes = args.nodes;
        cut.bounds = args.bounds;
    }

    const NeuralConsts &nc = args.nc;
    const V3 smin = mk3(nc.scene_min[0], nc.scene_min[1], nc.scene_min[2]);
    const V3 smax = mk3(nc.scene_max[0], nc.scene_max[1], nc.scene_max[2]);
    const float dilation = __fadd_rn(__fadd_rn(1.0f, nc.node_extent_dilation), nc.fixed_node_dilation);
    const V3 ext = scale3(sub3(smax, smin), dilation);
    const V3 center = scale3(add3(smax, smin), 0.5f);
    const float thr = nc.visibility_threshold;

    // slot state (lane = slot)
    enum : int { kEmpty = 0, kNeed = 1, kReady = 2 };
    int state = kEmpty;
    uint32_t ray_id = kInvalid;
    V3 o = mk3(0, 0, 0), d = mk3(0, 0, 0), nrm = mk3(0, 0, 0), alb = mk3(0, 0, 0);
    float best_t = FLT_MAX, vis = 0.f, seg_mint = 0.f, seg_maxt = 0.f, cur_maxt = FLT_MAX;
    bool valid = false, cull_ok = false;
    RayDiv rdiv = make_raydiv(o, mk3(1.f, 1.f, 1.f), false);
    uint32_t flags = 0, segments = 0, seg_node = 0, rng = 0;
    uint32_t stack[kNeuralStackSize];
    int sp = 0;
    bool exhausted = false;
    uint32_t st_segments = 0, st_capped = 0, st_overflow = 0, st_fallback = 0;

    auto finalize = [&]() {
        write_hit(args.hits, ray_id, valid ? best_t : FLT_MAX, nrm, alb, valid ? vis : 0.f,
                  flags | (valid ? NBVH_HIT_VALID : 0u), segments);
        state = kEmpty;
    };
    auto to_fallback = [&]() {
        write_hit(args.hits, ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, flags, segments);
        uint32_t slot = atomicAdd(&args.counters->fallback_count, 1u);
        args.fallback_list[slot] = ray_id;
        st_fallback++;
        state = kEmpty;
    };

    for (;;) {
        // ---- fill: empty slots take rays from the global queue; every slot that needs its next
        //      leaf segment (first one of a new ray, or the next one after an inference step)
        //      traverses the cut at the same call site, so lanes diverge as little as possible ----
        for (;;) {
            if (!exhausted) {
                const unsigned need = __ballot_sync(kFull, state == kEmpty);
                if (need != 0u) {
                    const uint32_t cnt = __popc(need);
                    uint32_t base = 0;
                    if (lane == 0)
                        base = atomicAdd(&args.counters->queue_head, cnt);
                    base = __shfl_sync(kFull, base, 0);
                    if ((uint64_t)base + cnt >= (uint64_t)args.n)
                        exhausted = true;
                    if (state == kEmpty) {
                        const uint32_t id = base + __popc(need & ((1u << lane) - 1u));
                        if (base < args.n && id < args.n) {
                            const float4 *r = reinterpret_cast<const float4 *>(args.rays + id);
                            const float4 ra = __ldg(r), rb = __ldg(r + 1);
                            ray_id = id;
                            o = mk3(ra.x, ra.y, ra.z);
                            d = mk3(rb.x, rb.y, rb.z);
                            cull_ok = d.x != 0.0f && d.y != 0.0f && d.z != 0.0f;
                            rdiv = make_raydiv(o, d, nc.fast_div_ok != 0u);
                            best_t = rb.w; // the ray's tmax plays the role of the current closest hit
                            cur_maxt = FLT_MAX; // the first leaf is searched unbounded (common.cuh:332-343)
                            valid = false;
                            vis = 0.f;
                            nrm = mk3(0, 0, 0);
                            alb = mk3(0, 0, 0);
                            flags = 0;
                            segments = 0;
                            rng = lcg_seed(0u, 0u, id);
                            stack[0] = 0;
                            sp = 1;
                            state = kNeed;
                        }
                    }
                }
            }
            if (state == kNeed) {
                const int res = neural_intersect_inference(cut, nc.bvh_lod, o, rdiv, cull_ok, stack, sp,
                                                           nc.inference_mint_epsilon, nc.inference_maxt_epsilon,
                                                           cur_maxt, seg_mint, seg_maxt, seg_node);
                if (res == 1) {
                    if (args.non_neural && args.non_neural[seg_node])
                        to_fallback();
                    else
                        state = kReady;
                } else {
                    if (res < 0) {
                        flags |= 0x8u;
                        st_overflow++;
                    }
                    finalize();
                }
            }
            const bool refill = !exhausted && __any_sync(kFull, state == kEmpty);
            if (!refill && !__any_sync(kFull, state == kNeed))
                break;
        }
        if (!__any_sync(kFull, state == kReady))
            break;

        // ---- step cap, then the segment's encoded points ----
        if (state == kReady && segments > nc.max_traversal_steps) {
            flags |= NBVH_HIT_STEP_CAP;
            st_capped++;
            finalize();
        }
        if (state == kReady) {
            float a = seg_mint, b = seg_maxt;
            if (a < 0.0f) { // encode_bvh_network_input_data swaps for a negative mint (kernels.cu:281-286)
                const float t = a;
                a = b;
                b = t;
            }
            const V3 epo = encode_world(ray_at(o, d, a), center, ext);
            const V3 epi = encode_world(ray_at(o, d, b), center, ext);
            for (uint32_t k = 0; k < P; k++) {
                const V3 p = segment_point(epo, epi, segment_t(k, P, args.grid.segment_distribution, rng));
                float *dst = pts + (lane * P + k) * 3u;
                dst[0] = p.x;
                dst[1] = p.y;
                dst[2] = p.z;
            }
        }
        const unsigned act_mask = __ballot_sync(kFull, state == kReady);
        __syncwarp();

        // ---- K3 + K4: hash-grid features into A fragments, fused MLP on two 16-row tiles ----
#pragma unroll 1
        for (int tile = 0; tile < 2; tile++) {
            if (((act_mask >> (tile * 16)) & 0xFFFFu) == 0u)
                continue;
            const int g = lane >> 2, tig = lane & 3;
            const int r0 = tile * 16 + g, r1 = r0 + 8;
            const bool act0 = (act_mask >> r0) & 1u, act1 = (act_mask >> r1) & 1u;
            auto feat = [&](int row, uint32_t j) -> uint32_t {
                const uint32_t p = j / L, l = j - p * L;
                const float *src = pts + (row * P + p) * 3u;
                const float2 f = encode_level(args.table, gp, l, mk3(src[0], src[1], src[2]));
                return pack_half2(f.x, f.y);
            };
            auto make_a = [&](uint32_t kb, uint32_t(&a)[4]) {
                const uint32_t j0 = kb * 8u + (uint32_t)tig, j1 = j0 + 4u;
                a[0] = act0 ? feat(r0, j0) : 0u;
                a[1] = act1 ? feat(r1, j0) : 0u;
                a[2] = act0 ? feat(r0, j1) : 0u;
                a[3] = act1 ? feat(r1, j1) : 0u;
            };
            float o4[4];
            mlp_forward_tile(sw, n_inputs, args.n_hidden_layers, make_a, o4);
            outs[r0 * 8 + tig * 2] = o4[0];
            outs[r0 * 8 + tig * 2 + 1] = o4[1];
            outs[r1 * 8 + tig * 2] = o4[2];
            outs[r1 * 8 + tig * 2 + 1] = o4[3];
        }
        __syncwarp();

        // ---- decode, keep the closest hit, then ask for the next leaf (K2) ----
        if (state == kReady) {
            float out[8];
#pragma unroll
            for (int k = 0; k < 8; k++)
                out[k] = outs[lane * 8 + k];
            segments++;
            st_segments++;
            if (nc.fallback_margin > 0.0f && fabsf(__fsub_rn(out[0], thr)) < nc.fallback_margin) {
                to_fallback();
            } else {
                // process_neural_bvh_traversal_step, src/cuda/neural/path/path_inference_kernels.cu:61-131
                float new_depth = best_t;
                bool stop = false;
                if (out[0] > thr) {
                    const bool inside = seg_mint < 0.0f;
                    if (nc.visibility_only && !inside) {
                        valid = true;
                        vis = out[0];
                        stop = true;
                    } else {
                        const float de = decode_local_t(out[1], seg_mint, seg_maxt, inside, nc.depth_epsilon,
                                                        nc.fixed_depth_epsilon);
                        if (de != FLT_MAX) {
                            if (nc.visibility_only) {
                                valid = true;
                                vis = out[0];
                                stop = true;
                            } else if (de < best_t) {
                                valid = true;
                                best_t = de;
                                new_depth = de;
                                vis = out[0];
                                nrm = normalize3(mk3(__fsub_rn(__fmul_rn(out[2], 2.0f), 1.0f),
                                                     __fsub_rn(__fmul_rn(out[3], 2.0f), 1.0f),
                                                     __fsub_rn(__fmul_rn(out[4], 2.0f), 1.0f)));
                                alb = mk3(out[5], out[6], out[7]);
                            }
                        }
                    }
                }
                // process_bvh_network_output_and_intersect_neural_bvh, common.cuh:496-550
                if (stop || sp == 0) {
                    finalize();
                } else {
                    cur_maxt = new_depth;
                    state = kNeed;
                }
            }
        }
    }

    // per-warp statistics
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        st_segments += __shfl_xor_sync(kFull, st_segments, off);
        st_capped += __shfl_xor_sync(kFull, st_capped, off);
        st_overflow += __shfl_xor_sync(kFull, st_overflow, off);
        st_fallback += __shfl_xor_sync(kFull, st_fallback, off);
    }
    if (lane == 0) {
        if (st_segments)
            atomicAdd(&args.counters->segments, st_segments);
        if (st_capped)
            atomicAdd(&args.counters->step_capped, st_capped);
        if (st_overflow)
            atomicAdd(&args.counters->stack_overflow, st_overflow);
        if (st_fallback)
            atomicAdd(&args.counters->fallback, st_fallback);
    }
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
};

// Network inference on explicit encoded positions: one warp per 32-row tile, grid-stride.
__global__ void __launch_bounds__(kThreads, 2) k_network_inference(const __grid_constant__ InferArgs args)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GridParams &gp = *reinterpret_cast<GridParams *>(smem_raw);
    const uint32_t n_inputs = args.grid.n_inputs, P = args.grid.n_points, L = args.grid.n_levels;
    __half *sw = reinterpret_cast<__half *>(smem_raw + sizeof(GridParams));
    copy_grid_params(gp, args.grid);
    load_weights_to_smem(args.weights, sw, n_inputs, args.n_hidden_layers);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const uint32_t warps_total = gridDim.x * kWarps;
    const uint32_t n_tiles = (args.n + 15u) / 16u;
    for (uint32_t tile = blockIdx.x * kWarps + (threadIdx.x >> 5); tile < n_tiles; tile += warps_total) {
        const uint32_t r0 = tile * 16u + g, r1 = r0 + 8u;
        const bool act0 = r0 < args.n, act1 = r1 < args.n;
        auto feat = [&](uint32_t row, uint32_t j) -> uint32_t {
            uint32_t p = j / L, l = j - p * L;
            const float *src = args.positions + ((size_t)row * P + p) * 3u;
            float2 f = encode_level(args.table, gp, l, mk3(__ldg(src), __ldg(src + 1), __ldg(src + 2)));
            return pack_half2(f.x, f.y);
        };
        auto make_a = [&](uint32_t kb, uint32_t(&a)[4]) {
            uint32_t j0 = kb * 8u + (uint32_t)tig, j1 = j0 + 4u;
            a[0] = act0 ? feat(r0, j0) : 0u;
            a[1] = act1 ? feat(r1, j0) : 0u;
            a[2] = act0 ? feat(r0, j1) : 0u;
            a[3] = act1 ? feat(r1, j1) : 0u;
        };
        float o4[4];
        mlp_forward_tile(sw, n_inputs, args.n_hidden_layers, make_a, o4);
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

// Hash-grid features (FP32 before the FP16 rounding), one thread per (row, point, level).
__global__ void __launch_bounds__(128) k_encode(const __grid_constant__ GridParams grid, const uint32_t *__restrict__ table,
                                                const float *__restrict__ positions, uint32_t n,
                                                float *__restrict__ features)
{
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t total = (uint64_t)n * grid.n_points * grid.n_levels;
    if (i >= total)
        return;
    uint32_t l = (uint32_t)(i % grid.n_levels);
    uint64_t rp = i / grid.n_levels; // row * points + point
    const float *src = positions + rp * 3u;
    float2 f = encode_level(table, grid, l, mk3(src[0], src[1], src[2]));
    features[rp * grid.n_levels * 2u + 2u * l] = f.x;
    features[rp * grid.n_levels * 2u + 2u * l + 1u] = f.y;
}

template <typename K>
cudaError_t prepare_smem(K kernel, size_t bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

} // namespace

static size_t query_smem_host(uint32_t n_inputs, uint32_t n_hidden, uint32_t n_points, uint32_t cut_nodes)
{
    return sizeof(GridParams) + smem_net_layout(n_inputs, n_hidden).total * sizeof(__half) + (size_t)cut_nodes * 56u +
           (size_t)kQWarps * 32u * (n_points * 3u + 8u) * sizeof(float);
}

constexpr size_t kSmemLimit = 227u * 1024u;

template <bool SMEM_CUT>
static cudaError_t launch_query_variant(const QueryArgs &a, size_t smem, int num_sms, cudaStream_t s)
{
    cudaError_t e = prepare_smem(k_neural_query<SMEM_CUT>, smem);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_neural_query<SMEM_CUT>, kQThreads, smem);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    uint32_t blocks = (uint32_t)(num_sms * per_sm);
    const uint32_t needed = (a.n + kQThreads - 1u) / kQThreads;
    if (needed < blocks)
        blocks = needed;
    k_neural_query<SMEM_CUT><<<blocks, kQThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_neural_query(const float4 *dilated_nodes, const float4 *bounds, uint32_t n_cut_nodes,
                                const uint8_t *non_neural, const __half *params_h, const GridParams &grid,
                                const NeuralConsts &nc, uint32_t n_hidden_layers, const nbvh_ray *rays, uint32_t n,
                                nbvh_neural_hit *hits, QueryCounters *counters, uint32_t *fallback_list, int num_sms,
                                cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    QueryArgs a;
    a.grid = grid;
    a.nc = nc;
    a.nodes = dilated_nodes;
    a.bounds = bounds;
    a.non_neural = non_neural;
    const uint32_t n_network_params =
        kNeurons * grid.n_inputs + (n_hidden_layers - 1u) * kNeurons * kNeurons + kOutputsPadded * kNeurons;
    a.table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    a.weights = params_h;
    a.rays = rays;
    a.hits = hits;
    a.counters = counters;
    a.fallback_list = fallback_list;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    a.n_cut_nodes = n_cut_nodes;
    const size_t smem_cut = query_smem_host(grid.n_inputs, n_hidden_layers, grid.n_points, n_cut_nodes);
    if (smem_cut <= kSmemLimit)
        return launch_query_variant<true>(a, smem_cut, num_sms, s);
    return launch_query_variant<false>(a, query_smem_host(grid.n_inputs, n_hidden_layers, grid.n_points, 0u), num_sms,
                                       s);
}

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
                                     const float *positions, uint32_t n, float *outputs, int num_sms, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    InferArgs a;
    a.grid = grid;
    uint32_t n_network_params = kNeurons * grid.n_inputs + (n_hidden_layers - 1u) * kNeurons * kNeurons +
                                kOutputsPadded * kNeurons;
    a.table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    a.weights = params_h;
    a.positions = positions;
    a.outputs = outputs;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    size_t smem = sizeof(GridParams) + smem_net_layout(grid.n_inputs, n_hidden_layers).total * sizeof(__half);
    cudaError_t e = prepare_smem(k_network_inference, smem);
    if (e != cudaSuccess)
        return e;
    uint32_t tiles = (n + 15u) / 16u;
    uint32_t blocks = (tiles + kWarps - 1u) / kWarps;
    uint32_t cap = (uint32_t)num_sms * 2u;
    if (blocks > cap)
        blocks = cap;
    k_network_inference<<<blocks, kThreads, smem, s>>>(a);
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
