// k_query.cu -- the neural closest-hit / visibility query as a device-resident wavefront.
//
// Reference path: NeuralPathModule::neural_bvh_traversal (src/cuda/neural/path/path_module.cu:
// 54-137) runs, per traversal step, an encode kernel, tcnn inference, a process kernel and a
// compaction kernel, then copies the active count to the host and synchronises. Here:
//
//   k_wave_first  one thread per ray: the first entered leaf (K2). Rays that enter none are
//                 answered at once; the others are appended (warp-aggregated) to state list 0.
//   k_wave_step   persistent over the listed rays, 32 rows per warp: the segment's encoded points,
//                 hash-grid features gathered straight into the tensor-core A fragments (K3), the
//                 fused FP16 MLP (K4), the LocalT decode and closest-hit update, then the next
//                 entered leaf (K2) for the rays that continue, appended to the other list.
//
// Every row of a tile is a live ray, so the tensor cores and the gathers work on full tiles, and
// the two kernels stay small. Per-ray state (~120 bytes plus the live part of the stack) moves
// through HBM once per step in coalesced structure-of-arrays form. The host checks the list
// count once per batch of steps (one 4-byte copy), instead of once per step.
#include <type_traits>

#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kStepWarps = 16;
constexpr int kStepThreads = kStepWarps * 32;

struct WaveArgs {
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
    WaveList lists[2];
    uint32_t *wave_counts; // 3 rotating list counters
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

// packed meta.w: segments (bits 0-15), stack size (16-23), flags (24-31)
__device__ __forceinline__ uint32_t pack_meta(uint32_t segments, int sp, uint32_t flags)
{
    return (segments & 0xFFFFu) | ((uint32_t)sp << 16) | (flags << 24);
}

struct RayState {
    V3 o, d, nrm, alb;
    float best_t, vis, seg_mint, seg_maxt;
    uint32_t seg_node, ray_id, segments, flags, rng;
    int sp;
};

__device__ __forceinline__ void store_state(const WaveList &L, uint32_t pos, const RayState &s, const uint32_t *stack)
{
    L.od0[pos] = make_float4(s.o.x, s.o.y, s.o.z, s.best_t);
    L.od1[pos] = make_float4(s.d.x, s.d.y, s.d.z, s.seg_mint);
    L.meta[pos] = make_uint4(__float_as_uint(s.seg_maxt), s.seg_node, s.ray_id, pack_meta(s.segments, s.sp, s.flags));
    L.nv[pos] = make_float4(s.nrm.x, s.nrm.y, s.nrm.z, s.vis);
    L.ar[pos] = make_float4(s.alb.x, s.alb.y, s.alb.z, __uint_as_float(s.rng));
    for (int k = 0; k < s.sp; k++)
        L.stack[(size_t)k * L.capacity + pos] = stack[k];
}

__device__ __forceinline__ void load_state(const WaveList &L, uint32_t pos, RayState &s, uint32_t *stack)
{
    const float4 a = L.od0[pos], b = L.od1[pos], c = L.nv[pos], e = L.ar[pos];
    const uint4 m = L.meta[pos];
    s.o = mk3(a.x, a.y, a.z);
    s.best_t = a.w;
    s.d = mk3(b.x, b.y, b.z);
    s.seg_mint = b.w;
    s.seg_maxt = __uint_as_float(m.x);
    s.seg_node = m.y;
    s.ray_id = m.z;
    s.segments = m.w & 0xFFFFu;
    s.sp = (int)((m.w >> 16) & 0xFFu);
    s.flags = m.w >> 24;
    s.nrm = mk3(c.x, c.y, c.z);
    s.vis = c.w;
    s.alb = mk3(e.x, e.y, e.z);
    s.rng = __float_as_uint(e.w);
    for (int k = 0; k < s.sp; k++)
        stack[k] = L.stack[(size_t)k * L.capacity + pos];
}

// warp-aggregated append position for lanes with `want` set
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

__global__ void __launch_bounds__(256) k_wave_first(const __grid_constant__ WaveArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool listed = false;
    RayState s;
    uint32_t stack[kNeuralStackSize];
    if (i < a.n) {
        const float4 *r = reinterpret_cast<const float4 *>(a.rays + i);
        const float4 ra = __ldg(r), rb = __ldg(r + 1);
        s.o = mk3(ra.x, ra.y, ra.z);
        s.d = mk3(rb.x, rb.y, rb.z);
        const bool cull_ok = s.d.x != 0.0f && s.d.y != 0.0f && s.d.z != 0.0f;
        const RayDiv rdiv = make_raydiv(s.o, s.d, a.nc.fast_div_ok != 0u);
        s.sp = 1;
        stack[0] = 0;
        const GlobalCut cut{a.nodes, a.bounds};
        // the first leaf is searched with an unbounded current_maxt (common.cuh:332-343)
        const int res = neural_intersect_inference(cut, a.nc.bvh_lod, s.o, rdiv, cull_ok, stack, s.sp,
                                                   a.nc.inference_mint_epsilon, a.nc.inference_maxt_epsilon, FLT_MAX,
                                                   s.seg_mint, s.seg_maxt, s.seg_node);
        if (res == 1) {
            if (a.non_neural && a.non_neural[s.seg_node]) {
                write_hit(a.hits, i, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, 0u, 0u);
                const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                a.fallback_list[slot] = i;
                atomicAdd(&a.counters->fallback, 1u);
            } else {
                listed = true;
                s.best_t = rb.w; // the ray's tmax plays the role of the current closest hit
                s.vis = 0.f;
                s.nrm = mk3(0, 0, 0);
                s.alb = mk3(0, 0, 0);
                s.ray_id = i;
                s.segments = 0;
                s.flags = 0;
                s.rng = lcg_seed(0u, 0u, i);
            }
        } else {
            if (res < 0)
                atomicAdd(&a.counters->stack_overflow, 1u);
            write_hit(a.hits, i, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, res < 0 ? 0x8u : 0u, 0u);
        }
    }
    const uint32_t pos = warp_append(listed, &a.wave_counts[0]);
    if (listed)
        store_state(a.lists[0], pos, s, stack);
}

template <bool SMEM_CUT>
__global__ void __launch_bounds__(kStepThreads, 1) k_wave_step(const __grid_constant__ WaveArgs a, uint32_t it)
{
    const uint32_t count_in = *reinterpret_cast<volatile const uint32_t *>(&a.wave_counts[it % 3u]);
    uint32_t *count_out = &a.wave_counts[(it + 1u) % 3u];
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.wave_counts[(it + 2u) % 3u] = 0u; // output counter of the next step (last read a step ago)
    const uint32_t n_tiles = (count_in + 31u) / 32u;
    if (blockIdx.x * kStepWarps >= n_tiles)
        return; // nothing for this block: skip staging the network

    extern __shared__ __align__(16) unsigned char smem_raw[];
    GridParams &gp = *reinterpret_cast<GridParams *>(smem_raw);
    const uint32_t n_inputs = a.grid.n_inputs, P = a.grid.n_points, L = a.grid.n_levels;
    const SmemNetLayout SL = smem_net_layout(n_inputs, a.n_hidden_layers);
    __half *sw = reinterpret_cast<__half *>(smem_raw + sizeof(GridParams));
    unsigned char *after_net = reinterpret_cast<unsigned char *>(sw + SL.total);
    const uint32_t cut_bytes = SMEM_CUT ? a.n_cut_nodes * 56u : 0u;
    float *warp_area = reinterpret_cast<float *>(after_net + cut_bytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *pts = warp_area + (size_t)warp * 32u * (P * 3u + 8u); // [32][P*3]
    float *outs = pts + 32u * P * 3u;                            // [32][8]
    const uint32_t fld = n_inputs + 8u;
    __half *feat = reinterpret_cast<__half *>(warp_area + (size_t)kStepWarps * 32u * (P * 3u + 8u)) +
                   (size_t)warp * 16u * fld; // per-warp 16-row feature tile
    (void)L;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&a.grid);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&gp);
        for (uint32_t i = threadIdx.x; i < sizeof(GridParams) / 4u; i += blockDim.x)
            dst[i] = src[i];
    }
    load_weights_to_smem(a.weights, sw, n_inputs, a.n_hidden_layers);
    float4 *s_nodes = reinterpret_cast<float4 *>(after_net);
    float2 *s_bounds = reinterpret_cast<float2 *>(after_net + a.n_cut_nodes * 32u);
    if (SMEM_CUT) {
        for (uint32_t i = threadIdx.x; i < 2u * a.n_cut_nodes; i += blockDim.x)
            s_nodes[i] = __ldg(a.nodes + i);
        for (uint32_t i = threadIdx.x; i < a.n_cut_nodes; i += blockDim.x) {
            const float4 u = __ldg(a.bounds + 2u * i), v = __ldg(a.bounds + 2u * i + 1u);
            s_bounds[3u * i] = make_float2(u.x, u.y);
            s_bounds[3u * i + 1u] = make_float2(u.z, v.x);
            s_bounds[3u * i + 2u] = make_float2(v.y, v.z);
        }
    }
    __syncthreads();
    using Cut = typename std::conditional<SMEM_CUT, SharedCut, GlobalCut>::type;
    Cut cut;
    if constexpr (SMEM_CUT) {
        cut.nodes = s_nodes;
        cut.bounds = s_bounds;
    } else {
        cut.nodes = a.nodes;
        cut.bounds = a.bounds;
    }

    const NeuralConsts &nc = a.nc;
    const V3 smin = mk3(nc.scene_min[0], nc.scene_min[1], nc.scene_min[2]);
    const V3 smax = mk3(nc.scene_max[0], nc.scene_max[1], nc.scene_max[2]);
    const float dilation = __fadd_rn(__fadd_rn(1.0f, nc.node_extent_dilation), nc.fixed_node_dilation);
    const V3 ext = scale3(sub3(smax, smin), dilation);
    const V3 center = scale3(add3(smax, smin), 0.5f);
    const float thr = nc.visibility_threshold;
    const WaveList &in = a.lists[it & 1u];
    const WaveList &out = a.lists[(it + 1u) & 1u];
    uint32_t st_segments = 0, st_capped = 0, st_overflow = 0, st_fallback = 0;

    for (uint32_t tile = blockIdx.x * kStepWarps + warp; tile < n_tiles; tile += gridDim.x * kStepWarps) {
        const uint32_t row = tile * 32u + (uint32_t)lane;
        bool active = row < count_in;
        RayState s;
        uint32_t stack[kNeuralStackSize];
        if (active) {
            load_state(in, row, s, stack);
            if (s.segments > nc.max_traversal_steps) { // step cap (path_module.cu:68, last_inference)
                s.flags |= NBVH_HIT_STEP_CAP;
                st_capped++;
                const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                write_hit(a.hits, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                          s.segments);
                active = false;
            }
        }
        if (active) {
            float ta = s.seg_mint, tb = s.seg_maxt;
            if (ta < 0.0f) { // encode_bvh_network_input_data swaps for a negative mint (kernels.cu:281-286)
                const float t = ta;
                ta = tb;
                tb = t;
            }
            const V3 epo = encode_world(ray_at(s.o, s.d, ta), center, ext);
            const V3 epi = encode_world(ray_at(s.o, s.d, tb), center, ext);
            for (uint32_t k = 0; k < P; k++) {
                const V3 p = segment_point(epo, epi, segment_t(k, P, a.grid.segment_distribution, s.rng));
                float *dst = pts + (lane * P + k) * 3u;
                dst[0] = p.x;
                dst[1] = p.y;
                dst[2] = p.z;
            }
        }
        const unsigned act_mask = __ballot_sync(kFull, active);
        __syncwarp();
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            const uint32_t mask = (act_mask >> (half * 16)) & 0xFFFFu;
            if (mask == 0u)
                continue;
            const int g = lane >> 2, tig = lane & 3;
            const int r0 = half * 16 + g, r1 = r0 + 8;
            auto pos = [&](uint32_t r, uint32_t p) -> V3 {
                const float *src = pts + ((half * 16u + r) * P + p) * 3u;
                return mk3(src[0], src[1], src[2]);
            };
            encode_tile_to_smem(a.table, gp, pos, mask, feat, fld);
            float o4[4];
            mlp_tile_from_smem(sw, feat, fld, n_inputs, a.n_hidden_layers, o4);
            outs[r0 * 8 + tig * 2] = o4[0];
            outs[r0 * 8 + tig * 2 + 1] = o4[1];
            outs[r1 * 8 + tig * 2] = o4[2];
            outs[r1 * 8 + tig * 2 + 1] = o4[3];
            __syncwarp();
        }
        __syncwarp();

        bool keep = false;
        if (active) {
            float o8[8];
#pragma unroll
            for (int k = 0; k < 8; k++)
                o8[k] = outs[lane * 8 + k];
            s.segments++;
            st_segments++;
            bool done = false;
            if (nc.fallback_margin > 0.0f && fabsf(__fsub_rn(o8[0], thr)) < nc.fallback_margin) {
                write_hit(a.hits, s.ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, s.flags & ~NBVH_HIT_VALID,
                          s.segments);
                const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                a.fallback_list[slot] = s.ray_id;
                st_fallback++;
                done = true;
            } else {
                // process_neural_bvh_traversal_step, src/cuda/neural/path/path_inference_kernels.cu:61-131
                float new_depth = s.best_t;
                bool stop = false;
                if (o8[0] > thr) {
                    const bool inside = s.seg_mint < 0.0f;
                    if (nc.visibility_only && !inside) {
                        s.flags |= NBVH_HIT_VALID;
                        s.vis = o8[0];
                        stop = true;
                    } else {
                        const float de = decode_local_t(o8[1], s.seg_mint, s.seg_maxt, inside, nc.depth_epsilon,
                                                        nc.fixed_depth_epsilon);
                        if (de != FLT_MAX) {
                            if (nc.visibility_only) {
                                s.flags |= NBVH_HIT_VALID;
                                s.vis = o8[0];
                                stop = true;
                            } else if (de < s.best_t) {
                                s.flags |= NBVH_HIT_VALID;
                                s.best_t = de;
                                new_depth = de;
                                s.vis = o8[0];
                                s.nrm = normalize3(mk3(__fsub_rn(__fmul_rn(o8[2], 2.0f), 1.0f),
                                                       __fsub_rn(__fmul_rn(o8[3], 2.0f), 1.0f),
                                                       __fsub_rn(__fmul_rn(o8[4], 2.0f), 1.0f)));
                                s.alb = mk3(o8[5], o8[6], o8[7]);
                            }
                        }
                    }
                }
                // process_bvh_network_output_and_intersect_neural_bvh, common.cuh:496-550
                if (!stop && s.sp > 0) {
                    const bool cull_ok = s.d.x != 0.0f && s.d.y != 0.0f && s.d.z != 0.0f;
                    const RayDiv rdiv = make_raydiv(s.o, s.d, nc.fast_div_ok != 0u);
                    const int res = neural_intersect_inference(cut, nc.bvh_lod, s.o, rdiv, cull_ok, stack, s.sp,
                                                               nc.inference_mint_epsilon, nc.inference_maxt_epsilon,
                                                               new_depth, s.seg_mint, s.seg_maxt, s.seg_node);
                    if (res == 1) {
                        if (a.non_neural && a.non_neural[s.seg_node]) {
                            write_hit(a.hits, s.ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f,
                                      s.flags & ~NBVH_HIT_VALID, s.segments);
                            const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                            a.fallback_list[slot] = s.ray_id;
                            st_fallback++;
                            done = true;
                        } else {
                            keep = true;
                        }
                    } else if (res < 0) {
                        s.flags |= 0x8u;
                        st_overflow++;
                    }
                }
            }
            if (!keep && !done) {
                const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                write_hit(a.hits, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                          s.segments);
            }
        }
        const uint32_t pos = warp_append(keep, count_out);
        if (keep)
            store_state(out, pos, s, stack);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        st_segments += __shfl_xor_sync(kFull, st_segments, off);
        st_capped += __shfl_xor_sync(kFull, st_capped, off);
        st_overflow += __shfl_xor_sync(kFull, st_overflow, off);
        st_fallback += __shfl_xor_sync(kFull, st_fallback, off);
    }
    if (lane == 0) {
        if (st_segments)
            atomicAdd(&a.counters->segments, st_segments);
        if (st_capped)
            atomicAdd(&a.counters->step_capped, st_capped);
        if (st_overflow)
            atomicAdd(&a.counters->stack_overflow, st_overflow);
        if (st_fallback)
            atomicAdd(&a.counters->fallback, st_fallback);
    }
}

size_t step_smem(uint32_t n_inputs, uint32_t n_hidden, uint32_t n_points, uint32_t cut_nodes)
{
    return sizeof(GridParams) + smem_net_layout(n_inputs, n_hidden).total * sizeof(__half) + (size_t)cut_nodes * 56u +
           (size_t)kStepWarps * 32u * (n_points * 3u + 8u) * sizeof(float) +
           (size_t)kStepWarps * 16u * (n_inputs + 8u) * sizeof(__half);
}

constexpr size_t kSmemLimit = 227u * 1024u;
constexpr uint32_t kStepsPerCheck = 4;

template <bool SMEM_CUT>
cudaError_t run_steps(const WaveArgs &a, size_t smem, int num_sms, uint32_t max_steps, uint32_t *h_count,
                      cudaEvent_t ev, cudaStream_t s, uint32_t &launches)
{
    cudaError_t e = cudaFuncSetAttribute(k_wave_step<SMEM_CUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    // every listed ray advances one leaf per step; the loop ends when a list comes out empty or the
    // step cap (each ray at most max_traversal_steps + 1 segments) plus the final capping step is reached
    const uint32_t limit = max_steps + 2u;
    for (uint32_t it = 0; it < limit;) {
        const uint32_t batch = (limit - it) < kStepsPerCheck ? (limit - it) : kStepsPerCheck;
        for (uint32_t b = 0; b < batch; b++, it++) {
            k_wave_step<SMEM_CUT><<<num_sms, kStepThreads, smem, s>>>(a, it);
            e = cudaGetLastError();
            if (e != cudaSuccess)
                return e;
            launches++;
        }
        e = cudaMemcpyAsync(h_count, &a.wave_counts[it % 3u], sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess)
            return e;
        if (ev) {
            e = cudaEventRecord(ev, s);
            if (e != cudaSuccess)
                return e;
            e = cudaEventSynchronize(ev);
        } else {
            e = cudaStreamSynchronize(s);
        }
        if (e != cudaSuccess)
            return e;
        if (*h_count == 0u)
            break;
    }
    return cudaSuccess;
}

} // namespace

cudaError_t launch_wave_query(const float4 *dilated_nodes, const float4 *bounds, uint32_t n_cut_nodes,
                              const uint8_t *non_neural, const __half *params_h, const GridParams &grid,
                              const NeuralConsts &nc, uint32_t n_hidden_layers, const nbvh_ray *rays, uint32_t n,
                              nbvh_neural_hit *hits, QueryCounters *counters, uint32_t *fallback_list,
                              const WaveList lists[2], uint32_t *wave_counts, uint32_t *h_count, cudaEvent_t ev,
                              int num_sms, cudaStream_t s, uint32_t *launches)
{
    *launches = 0;
    if (n == 0)
        return cudaSuccess;
    WaveArgs a;
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
    a.lists[0] = lists[0];
    a.lists[1] = lists[1];
    a.wave_counts = wave_counts;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    a.n_cut_nodes = n_cut_nodes;
    cudaError_t e = cudaMemsetAsync(wave_counts, 0, 3u * sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return e;
    k_wave_first<<<(n + 255u) / 256u, 256, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    *launches = 1;
    const size_t smem_cut = step_smem(grid.n_inputs, n_hidden_layers, grid.n_points, n_cut_nodes);
    if (smem_cut <= kSmemLimit)
        return run_steps<true>(a, smem_cut, num_sms, nc.max_traversal_steps, h_count, ev, s, *launches);
    return run_steps<false>(a, step_smem(grid.n_inputs, n_hidden_layers, grid.n_points, 0u), num_sms,
                            nc.max_traversal_steps, h_count, ev, s, *launches);
}

// ---------------------------------------------------------------------------------------------
// Fixed scratch of the allocation-free query: a file-scope device array, so the CUDA runtime
// creates one copy per device when it loads this module and no call allocates it.
// ---------------------------------------------------------------------------------------------

namespace {
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];
constexpr int kNoallocMaxDevices = 64;
} // namespace

cudaError_t noalloc_scratch(int device, NoallocScratch *out)
{
    static std::mutex mu;
    static unsigned char *base[kNoallocMaxDevices] = {};
    if (device < 0 || device >= kNoallocMaxDevices)
        return cudaErrorInvalidDevice;
    unsigned char *p;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!base[device]) {
            void *addr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
            if (e != cudaSuccess)
                return e;
            base[device] = static_cast<unsigned char *>(addr);
        }
        p = base[device];
    }
    const size_t n = kNoallocRays;
    for (int k = 0; k < 2; k++) {
        WaveList &L = out->lists[k];
        L.od0 = reinterpret_cast<float4 *>(p);
        L.od1 = L.od0 + n;
        L.nv = L.od1 + n;
        L.ar = L.nv + n;
        L.meta = reinterpret_cast<uint4 *>(L.ar + n);
        L.stack = reinterpret_cast<uint32_t *>(L.meta + n);
        L.capacity = (uint32_t)n;
        p += kNoallocListBytes;
    }
    out->fallback_list = reinterpret_cast<uint32_t *>(p);
    p += n * 4u;
    out->counters = reinterpret_cast<QueryCounters *>(p);
    p += 256u;
    out->wave_counts = reinterpret_cast<uint32_t *>(p);
    return cudaSuccess;
}

} // namespace nbvh
