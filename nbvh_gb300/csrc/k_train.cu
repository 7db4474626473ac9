// k_train.cu -- run-optimisation kernels: training-ray generation and labelling on the device,
// the hash-grid encoding of the training rows, forward + composite loss + backward with the weight
// gradients on the tcgen05 tensor cores (K4 backward), the hash-grid gradient scatter (K3
// backward) and the fused Adam step (K5).
//
// Reference path: NeuralBVHRenderer::render, m_run_optimisation branch
// (src/cuda/neural/neural_bvh_renderer.cu:141-288): granular_sample_bvh_network_input_data
// (src/cuda/neural/neural_bvh_module_kernels.cu:119-264), then tcnn's trainer->training_step
// (encoding + FullyFusedMLP forward, PathTracingCompositeLoss, backward, Adam wrapped in
// ExponentialDecay; configured at src/cuda/neural/neural_bvh_module.cu:118-263).
#include <cuda.h>

#include <cstring>
#include <vector>

#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"
#include "tc_device.cuh"

namespace nbvh {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------------------------
// Training rays (n_sub_batch = 1): stack_based_sample_uniform_bvh_density
// (include/cuda/neural/neural_bvh_module_common.cuh:703-781), sample_bbox_position (635-660),
// generate_single_bvh_network_output_reference (783-861), LocalT depth target (586-629).
// ---------------------------------------------------------------------------------------------

struct SampleArgs {
    GridParams grid;
    NeuralConsts nc;
    const float4 *neural_nodes;
    const float4 *nodes;
    const float4 *tris;
    const float *albedo;
    float *positions;
    float *targets;
    uint32_t *sample_nodes;
    uint32_t training_step;
    uint32_t batch_size;
    uint32_t n;
    uint32_t learned_lod;
    uint32_t classic_fast_div; // classic BVH coordinates in the fast-division domain
    NodeSurvival survival;
};

__device__ __forceinline__ V3 cube_pos_on_face(int face, float u, float v) // sampling.cuh:85-94
{
    switch (face) {
    case 0: return mk3(1.0f, u, v);
    case 1: return mk3(0.0f, u, v);
    case 2: return mk3(u, 1.0f, v);
    case 3: return mk3(u, 0.0f, v);
    case 4: return mk3(u, v, 1.0f);
    default: return mk3(u, v, 0.0f);
    }
}

// A sample's state after its leaf segment was found: origin | mint, direction | maxt, node | rng |
// dilation.
struct SampleFound {
    float4 o_mint, d_maxt;
    uint4 node_rng;
};

constexpr uint32_t kFindThreads = 256;
constexpr int kFindVisits = 8; // node visits of a traversal between lane refills

// First part of the sampler: every sample's direction, LoD and dilation, then its search for an
// entered leaf segment from random origins in the scaled scene box (a fresh origin after every
// traversal that finds none). Persistent warps take samples from a counter and run the traversals
// in rounds of kFindVisits node visits, refilling the lanes whose sample is done, so that one
// sample's many retries do not hold its warp's other lanes idle. Every sample draws the same
// random numbers in the same order as a thread running it alone.
__global__ void __launch_bounds__(kFindThreads, 4) k_training_find(const __grid_constant__ SampleArgs a,
                                                                  SampleFound *__restrict__ found,
                                                                  uint32_t *__restrict__ counter)
{
    const NeuralConsts &c = a.nc;
    const V3 smin = mk3(c.scene_min[0], c.scene_min[1], c.scene_min[2]);
    const V3 smax = mk3(c.scene_max[0], c.scene_max[1], c.scene_max[2]);
    const float h = __fmul_rn(__fsub_rn(c.sampling_bbox_scaling, 1.0f), 0.5f);
    const int lane = threadIdx.x & 31;
    uint32_t i = 0, rng = 0, sampled_lod = 0, node = 0, guard = 0;
    float dil = 0.f, mint = 0.f, maxt = 0.f;
    V3 o = mk3(0, 0, 0), dir = mk3(0, 0, 0);
    uint32_t stack[kNeuralStackSize];
    int sp = 0;
    bool active = false, need_origin = false, exhausted = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !active);
        if (idle != 0u && !exhausted) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(counter, (uint32_t)__popc(idle));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            exhausted = base + (uint32_t)__popc(idle) >= a.n;
            const uint32_t k = base + __popc(idle & ((1u << lane) - 1u));
            if (!active && k < a.n) {
                i = k;
                rng = lcg_seed(a.training_step * a.batch_size, 0u, i);
                const float sx = lcg_randomf(rng);
                const float sy = lcg_randomf(rng);
                dir = uniform_sphere(sx, sy);
                // sampled LoD among the ones learned so far (common.cuh:719-721)
                const uint32_t n_lods = kNumBvhLods - a.learned_lod;
                const uint32_t lod_pick = __float2uint_rz(__fmul_rn(lcg_randomf(rng), __uint2float_rn(n_lods)));
                sampled_lod = a.learned_lod + min(lod_pick, n_lods - 1u);
                dil = __fadd_rn(c.fixed_node_dilation, __fmul_rn(lcg_randomf(rng), c.node_extent_dilation));
                mint = maxt = 0.f;
                node = 0;
                guard = 0;
                need_origin = true;
                active = true;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, active)) {
            if (exhausted)
                break;
            continue;
        }
        if (active) {
            if (need_origin) {
                stack[0] = 0;
                sp = 1;
                const float px = lcg_randomf(rng);
                const float py = lcg_randomf(rng);
                const float pz = lcg_randomf(rng);
                V3 ps = sub3(scale3(mk3(px, py, pz), c.sampling_bbox_scaling), mk3(h, h, h));
                o = add3(mul3(ps, sub3(smax, smin)), smin);
                need_origin = false;
            }
            const int res = neural_intersect(a.neural_nodes, sampled_lod, o, dir, stack, sp, false,
                                             c.inference_mint_epsilon, c.inference_maxt_epsilon,
                                             c.learning_mint_epsilon, c.learning_maxt_epsilon, FLT_MAX, dil, mint,
                                             maxt, node, kFindVisits);
            if (res != 2) {
                if (res < 0)
                    sp = 0;
                if (res != 1 && ++guard < 100000u) {
                    need_origin = true; // no leaf from this origin: the next attempt draws another
                } else {
                    SampleFound f;
                    f.o_mint = make_float4(o.x, o.y, o.z, mint);
                    f.d_maxt = make_float4(dir.x, dir.y, dir.z, maxt);
                    f.node_rng = make_uint4(node, rng, __float_as_uint(dil), 0u);
                    found[i] = f;
                    active = false;
                }
            }
        }
    }
}

// Second part of the sampler, one thread per sample: leaf-boundary origins, node survival, the
// encoded segment points and the classic-BVH labels.
__global__ void __launch_bounds__(128) k_training_samples(const __grid_constant__ SampleArgs a,
                                                          const SampleFound *__restrict__ found)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const NeuralConsts &c = a.nc;
    const V3 smin = mk3(c.scene_min[0], c.scene_min[1], c.scene_min[2]);
    const V3 smax = mk3(c.scene_max[0], c.scene_max[1], c.scene_max[2]);
    const SampleFound f = found[i];
    V3 o = mk3(f.o_mint.x, f.o_mint.y, f.o_mint.z), d = mk3(f.d_maxt.x, f.d_maxt.y, f.d_maxt.z);
    float mint = f.o_mint.w, maxt = f.d_maxt.w;
    const uint32_t node = f.node_rng.x;
    uint32_t rng = f.node_rng.y;
    const float dil = __uint_as_float(f.node_rng.z);
    if (c.leaf_boundary_sampling_ratio != 0.0f && lcg_randomf(rng) <= c.leaf_boundary_sampling_ratio) {
        int f1 = __float2int_rz(__fmul_rn(lcg_randomf(rng), 6.0f));
        f1 = f1 < 5 ? f1 : 5;
        int f2;
        do {
            f2 = __float2int_rz(__fmul_rn(lcg_randomf(rng), 6.0f));
            f2 = f2 < 5 ? f2 : 5;
        } while (f1 == f2);
        const float u1 = lcg_randomf(rng), v1 = lcg_randomf(rng);
        const V3 lp1 = cube_pos_on_face(f1, u1, v1);
        const float u2 = lcg_randomf(rng), v2 = lcg_randomf(rng);
        const V3 lp2 = cube_pos_on_face(f2, u2, v2);
        NodeBox nb = load_node(a.neural_nodes, node);
        V3 ext = sub3(nb.mx, nb.mn);
        V3 center = add3(nb.mn, scale3(ext, 0.5f));
        V3 next = scale3(ext, __fadd_rn(1.0f, dil));
        V3 nmin = sub3(center, scale3(next, 0.5f));
        V3 entry = add3(nmin, mul3(lp1, next));
        V3 exitp = add3(nmin, mul3(lp2, next));
        o = entry;
        d = normalize3(sub3(exitp, entry));
        mint = 0.0f;
        maxt = length3(sub3(exitp, entry));
    }
    if (a.sample_nodes)
        a.sample_nodes[i] = node;
    if (a.survival.enabled) {
        // node survival (neural_bvh_module_kernels.cu:184-199): a rejected sample leaves its slot's
        // previous input and target in place; its node index is already written
        const uint4 st = reinterpret_cast<const uint4 *>(a.survival.stats)[node];
        const float estimate = tree_cut_heuristic(__uint_as_float(st.x), st.y, st.w);
        const float cur_max = a.survival.max_word ? __uint_as_float(*a.survival.max_word) : 0.0f;
        float kept = fmaxf(a.survival.min_prob, __fdiv_rn(estimate, cur_max));
        if (!(estimate <= cur_max))
            kept = 1.0f;
        if (__fmul_rn(a.survival.scale, kept) < lcg_randomf(rng))
            return;
    }

    // encoded segment points (neural_bvh_module_kernels.cu:10-97)
    const float dilation = __fadd_rn(__fadd_rn(1.0f, c.node_extent_dilation), c.fixed_node_dilation);
    const V3 sext = scale3(sub3(smax, smin), dilation);
    const V3 scenter = scale3(add3(smax, smin), 0.5f);
    const V3 epo = encode_world(ray_at(o, d, mint), scenter, sext);
    const V3 epi = encode_world(ray_at(o, d, maxt), scenter, sext);
    const uint32_t P = a.grid.n_points;
    for (uint32_t k = 0; k < P; k++) {
        V3 p = segment_point(epo, epi, segment_t(k, P, a.grid.segment_distribution, rng));
        float *dst = a.positions + ((size_t)i * P + k) * 3u;
        dst[0] = p.x;
        dst[1] = p.y;
        dst[2] = p.z;
    }

    // labels from the classic BLAS on [mint, maxt]
    float t, u, v;
    uint32_t prim, rec = 0;
    classic_traverse<false>(a.nodes, a.tris, o, d, mint, maxt, t, u, v, prim, &rec, a.classic_fast_div != 0u);
    float4 *tg = reinterpret_cast<float4 *>(a.targets + 8u * (size_t)i);
    if (t != FLT_MAX) {
        const float depth =
            __double2float_rn(__ddiv_rn((double)__fsub_rn(t, mint), __dadd_rn((double)__fsub_rn(maxt, mint), 1e-3)));
        float4 r1 = __ldg(a.tris + 3u * rec + 1u), r2 = __ldg(a.tris + 3u * rec + 2u);
        V3 gn = normalize3(cross3(mk3(r1.x, r1.y, r1.z), mk3(r2.x, r2.y, r2.z)));
        V3 nn = scale3(adds3(gn, 1.0f), 0.5f);
        float ax = 0.9f, ay = 0.9f, az = 0.9f;
        if (a.albedo) {
            ax = a.albedo[3u * prim];
            ay = a.albedo[3u * prim + 1u];
            az = a.albedo[3u * prim + 2u];
        }
        tg[0] = make_float4(1.0f, depth, nn.x, nn.y);
        tg[1] = make_float4(nn.z, ax, ay, az);
    } else {
        tg[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        tg[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// ---------------------------------------------------------------------------------------------
// Composite loss: include/cuda/neural/utils/loss_gradient.cuh:25-94,
// include/cuda/neural/utils/pt_composite_loss.cuh:18-123
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ void loss_and_gradient(int type, float target, float pred, float &loss, float &grad)
{
    switch (type) {
    case NBVH_LOSS_RELATIVE_L2: {
        float diff = pred - target;
        float denom = pred * pred + 1e-2f;
        loss = diff * diff / denom;
        grad = 2.0f * diff / denom;
        break;
    }
    case NBVH_LOSS_RELATIVE_L1: {
        float scale = 1.0f / (fabsf(pred) + 1e-2f);
        float diff = pred - target;
        loss = fabsf(diff) * scale;
        grad = copysignf(scale, diff);
        break;
    }
    case NBVH_LOSS_L1: {
        float diff = pred - target;
        loss = fabsf(diff);
        grad = copysignf(1.0f, diff);
        break;
    }
    case NBVH_LOSS_BCE: {
        const float eps = 1e-5f;
        float p = fminf(fmaxf(pred, eps), 1.0f - eps);
        loss = -(target * logf(p) + (1.0f - target) * logf(1.0f - p));
        grad = -(target - p) / (p - (p * p));
        break;
    }
    case NBVH_LOSS_LOG_L2: {
        float diff = logf(1.0f + pred) - logf(1.0f + target);
        loss = diff * diff;
        grad = 2.0f * diff / (pred + 1.0f);
        break;
    }
    case NBVH_LOSS_L_HALF: {
        float sd = sqrtf(fabsf(pred - target));
        loss = sd;
        grad = 1.0f / (2.0f * sd + 1e-5f);
        break;
    }
    default: {
        float diff = pred - target;
        loss = diff * diff;
        grad = 2.0f * diff;
        break;
    }
    }
}

// loss value (normalised by n_total) and d loss / d output (loss scale applied) of one element
__device__ __forceinline__ void composite_loss(const LossConsts &lc, uint32_t ch, float pred, float target,
                                               float target_vis, float &value, float &grad)
{
    float loss = 0.f, g = 0.f;
    const bool ignore = lc.masking ? (target_vis < 0.5f) : false;
    if (ch == 0) {
        loss_and_gradient(lc.visibility_loss, target, pred, loss, g);
        loss *= lc.visibility_loss_scale;
        g *= lc.visibility_loss_scale;
    } else if (ch == 1 && !ignore) {
        loss_and_gradient(lc.depth_loss, target, pred, loss, g);
        loss *= lc.depth_loss_scale;
        g *= lc.depth_loss_scale;
    } else if (ch >= 2 && ch < 5 && !ignore && lc.learn_normal) {
        if (lc.normal_linear) {
            const float n_length = 0.1f;
            float n_axis = (pred * 2.0f - 1.0f) / n_length;
            float lin = n_axis * 0.5f + 0.5f;
            loss_and_gradient(lc.normal_loss, target, lin, loss, g);
            g *= 1.0f / n_length;
        } else {
            loss_and_gradient(lc.normal_loss, target, pred, loss, g);
        }
        loss *= lc.normal_loss_scale;
        g *= lc.normal_loss_scale;
    } else if (ch >= 5 && ch < 8 && !ignore && lc.learn_albedo) {
        if (lc.albedo_linear) {
            const float n_length = 0.1f;
            float lin = pred / n_length;
            loss_and_gradient(lc.albedo_loss, target, lin, loss, g);
            g *= 1.0f / n_length;
        } else {
            loss_and_gradient(lc.albedo_loss, target, pred, loss, g);
        }
        loss *= lc.albedo_loss_scale;
        g *= lc.albedo_loss_scale;
    }
    value = loss * lc.inv_n_total;
    grad = lc.loss_scale * g * lc.inv_n_total;
}

// ---------------------------------------------------------------------------------------------
// The hash-grid features of the training rows, in the MLP precision, into rows of row_stride
// halves (n_inputs: the tensor-core kernel's feature rows): one thread per (row, point), the
// levels in order, F features per level stored together (K3 forward).
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_train_encode(const __grid_constant__ GridParams grid,
                                                      const uint32_t *__restrict__ table,
                                                      const float *__restrict__ positions, uint32_t n,
                                                      __half *__restrict__ feat, uint32_t row_stride, uint32_t bf16)
{
    const uint32_t P = grid.n_points, L = grid.n_levels, F = grid.n_features;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * P)
        return;
    const uint32_t row = (uint32_t)(i / P), p = (uint32_t)(i - (uint64_t)row * P);
    const float *src = positions + i * 3u;
    const V3 pos = mk3(__ldg(src), __ldg(src + 1), __ldg(src + 2));
    auto pack16 = [bf16](float lo, float hi) { return bf16 ? pack_bf162(lo, hi) : pack_half2(lo, hi); };
    __half *dst = feat + (size_t)row * row_stride + (size_t)p * L * F;
    for (uint32_t l = 0; l < L; l++) {
        if (F == 4u) {
            float f[4];
            encode_level_wide<4>(table, grid, l, pos, f);
            *reinterpret_cast<uint2 *>(dst + 4u * l) = make_uint2(pack16(f[0], f[1]), pack16(f[2], f[3]));
        } else if (F == 8u) {
            float f[8];
            encode_level_wide<8>(table, grid, l, pos, f);
            *reinterpret_cast<uint4 *>(dst + 8u * l) =
                make_uint4(pack16(f[0], f[1]), pack16(f[2], f[3]), pack16(f[4], f[5]), pack16(f[6], f[7]));
        } else {
            const float2 f = encode_level<true>(table, grid, l, pos);
            *reinterpret_cast<uint32_t *>(dst + 2u * l) = pack16(f.x, f.y);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Training forward + composite loss + backward on the tensor cores (K3/K4 backward).
//
// k_train_encode writes each row's FP16 features; then one CTA per SM (128 threads, one tile row
// per thread and TMEM lane) runs 128-row tiles through
//   forward   Z_{j+1} = X_j W_j^T for every matrix j (tcgen05, M = 128 rows), the ReLU'd 16-bit
//             activations X_{j+1} written back to shared memory (and their ReLU masks kept in
//             registers), then the sigmoid, the composite loss and dZ_out = dL/dZ_out;
//   backward  for j = H .. 0: dX_j = dZ_{j+1} W_j (W_j read transposed, as an MN-major operand)
//             and dW_j^T += X_j^T dZ_{j+1} over the tile's 128 rows (both operands read
//             transposed from the same shared-memory tiles), then dZ_j = dX_j * (X_j > 0);
//             dX_0, rounded to the MLP precision, goes to global memory for the grid scatter.
// The weight gradients stay in tensor memory, accumulated over all the CTA's tiles, and are
// added to the FP32 gradient once per CTA at the end. Every [128 rows][C columns] tile lives in
// shared memory in the K-major core-matrix layout (8-column block c at c * 2,048 bytes, row r at
// r * 16 within it): with M = rows it is a K-major operand (LBO 2,048, SBO 128), with K = rows an
// MN-major one (LBO 128, SBO 2,048). The input tile arrives in that layout from TMA (8-value boxes).
// ---------------------------------------------------------------------------------------------

constexpr uint32_t kTcRows = 128;
constexpr uint32_t kTcThreads = 128;
constexpr uint32_t kColBlock = kTcRows * 16u; // bytes between 8-column blocks of a row tile
constexpr uint32_t kTcAccCols = 128;          // TMEM columns of the current layer's accumulator
constexpr uint32_t kTcTmemCols = 512;
constexpr uint32_t kTcWgColsMax = kTcTmemCols - kTcAccCols;
constexpr uint32_t kTcMaxMatrices = kMaxHiddenLayers + 1u;

struct TrainTcArgs {
    const __half *wpacked; // 16-bit matrices in the K-major operand layout, back to back
    uint32_t wbytes;
    uint32_t n_inputs;
    uint32_t n_hidden_layers;
    uint32_t n;
    const float *targets; // n x 8
    LossConsts lc;
    __half *dfeat;        // n x n_inputs gradients of the encoded features (emit launches)
    float *grad;          // FP32 gradient vector (network matrices first)
    float *loss_sum;
    float *sample_loss;   // per row: sum of its output channels' loss values (may be NULL)
    uint32_t *status;     // nonzero when a bounded wait gave up
    uint32_t wg_mask;     // bit j: this launch accumulates the gradient of matrix j
    uint32_t emit;        // this launch writes dfeat, the loss and the per-row losses
    uint32_t min_matrix;  // the backward runs from matrix H down to this one
    // shared-memory offsets (bytes from the 1,024-byte aligned base)
    uint32_t x0_off;                      // two input tile buffers of n_inputs * 256 bytes
    uint32_t x_off[kTcMaxMatrices];       // X_j (j = 1..H): 64-column tile (shared when not in wg_mask)
    uint32_t dz_off, dzo_off, bar_off;
    uint32_t wg_col[kTcMaxMatrices];      // TMEM column of the dW_j^T accumulator
    uint64_t wait_ns;                     // time limit of the phase waits
    uint32_t stall;                       // failure-path test: wait on an mbarrier nothing arrives at
};

__host__ __device__ constexpr uint32_t tc_w0_bytes(uint32_t n_in) { return kNeurons * n_in * 2u; }
__host__ __device__ constexpr uint32_t tc_hidden_w_bytes() { return kNeurons * kNeurons * 2u; }
// byte offset of matrix j in the packed weights; its output and input widths
__host__ __device__ inline uint32_t tc_w_off(uint32_t j, uint32_t n_in)
{
    return j == 0u ? 0u : tc_w0_bytes(n_in) + (j - 1u) * tc_hidden_w_bytes();
}
__host__ __device__ inline uint32_t tc_n_out(uint32_t j, uint32_t H) { return j < H ? kNeurons : kOutputsPadded; }
__host__ __device__ inline uint32_t tc_n_in(uint32_t j, uint32_t n_in) { return j == 0u ? n_in : kNeurons; }
// FP32 parameter offset of matrix j (row-major [out][in])
__host__ __device__ inline uint32_t tc_param_off(uint32_t j, uint32_t n_in)
{
    return j == 0u ? 0u : kNeurons * n_in + (j - 1u) * kNeurons * kNeurons;
}

// this thread's row of a [128][cols] tile: 16-byte chunk c (columns 8c .. 8c + 7)
__device__ __forceinline__ void store_row_chunks(unsigned char *tile, uint32_t row, const uint32_t *words,
                                                 uint32_t chunks)
{
    for (uint32_t c = 0; c < chunks; c++)
        *reinterpret_cast<uint4 *>(tile + c * kColBlock + row * 16u) =
            make_uint4(words[4u * c], words[4u * c + 1u], words[4u * c + 2u], words[4u * c + 3u]);
}

template <bool BF16, bool FP8>
__global__ void __launch_bounds__(kTcThreads, 1) k_train_tc(const __grid_constant__ CUtensorMap fmap,
                                                            const __grid_constant__ TrainTcArgs a)
{
    using Pr = MlpPrec<BF16>;
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t K0 = a.n_inputs, H = a.n_hidden_layers;
    const uint32_t n_tiles = (a.n + kTcRows - 1u) / kTcRows;
    if (blockIdx.x >= n_tiles)
        return;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const bool issuer = tid == 0u;
    // weights, load 0, load 1, mma, and one nothing arrives at (failure-path test)
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + a.bar_off);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 5);
    const uint32_t base = tc::smem_addr(smem);
    const uint32_t bar_w = tc::smem_addr(&bars[0]), bar_mma = tc::smem_addr(&bars[3]);
    const uint32_t x0_bytes = K0 * kTcRows * 2u;

    if (warp == 0u) {
        tc::tmem_alloc(tc::smem_addr(slot), kTcTmemCols);
        tc::tmem_relinquish();
    }
    if (issuer) {
        for (uint32_t b = 0; b < 5u; b++)
            tc::mbar_init(tc::smem_addr(&bars[b]), 1u);
        tc::mbar_init_fence();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t lane_off = (32u * warp) << 16; // this warp's TMEM lanes

    auto load_tile = [&](uint32_t t, uint32_t buf) {
        const uint32_t bar = tc::smem_addr(&bars[1u + buf]);
        const uint32_t dst = base + a.x0_off + buf * x0_bytes;
        tc::mbar_expect_tx(bar, x0_bytes);
        for (uint32_t c = 0; c < K0 / 8u; c++)
            tc::tma_load_2d(dst + c * kColBlock, &fmap, (int32_t)(8u * c), (int32_t)(t * kTcRows), bar);
    };
    uint32_t t = blockIdx.x;
    bool load_pending[2] = {false, false};
    if (issuer) {
        tc::mbar_expect_tx(bar_w, a.wbytes);
        for (uint32_t o = 0; o < a.wbytes; o += 16384u)
            tc::bulk_load(base + o, reinterpret_cast<const unsigned char *>(a.wpacked) + o,
                          a.wbytes - o < 16384u ? a.wbytes - o : 16384u, bar_w);
        load_tile(t, 0u);
    }
    load_pending[0] = true;
    bool ok = issuer ? tc::mbar_wait(bar_w, 0u, a.wait_ns) : true;
    if (a.stall && issuer) // nothing ever arrives at this barrier: the wait runs out
        ok = ok && tc::mbar_wait(tc::smem_addr(&bars[4]), 0u, a.wait_ns);
    ok = __syncthreads_and(ok);

    uint32_t ph_load[2] = {0u, 0u}, ph_mma = 0u, buf = 0u;
    bool mma_pending = false, first_tile = true;
    float loss_acc = 0.f;
    // waits for the MMAs committed so far; false (everyone) if the wait gave up
    auto mma_done = [&]() -> bool {
        bool r = issuer ? tc::mbar_wait(bar_mma, ph_mma, a.wait_ns) : true;
        r = __syncthreads_and(r);
        if (r) {
            ph_mma ^= 1u;
            mma_pending = false;
            tc::fence_after_sync();
        }
        return r;
    };
    for (; ok && t < n_tiles; t += gridDim.x, buf ^= 1u) {
        ok = issuer ? tc::mbar_wait(tc::smem_addr(&bars[1u + buf]), ph_load[buf], a.wait_ns) : true;
        ok = __syncthreads_and(ok);
        if (!ok)
            break;
        ph_load[buf] ^= 1u;
        load_pending[buf] = false;
        // the other buffer's last reader (the previous tile's MMAs) has completed
        if (t + gridDim.x < n_tiles) {
            if (issuer)
                load_tile(t + gridDim.x, buf ^ 1u);
            load_pending[buf ^ 1u] = true;
        }
        const uint32_t x0_addr = base + a.x0_off + buf * x0_bytes;
        auto x_addr = [&](uint32_t j) { return j == 0u ? x0_addr : base + a.x_off[j]; };
        const uint32_t row = t * kTcRows + tid;
        const bool valid = row < a.n;
        uint32_t relu_mask[2u * kTcMaxMatrices]; // bit c of X_j's row: words 2j, 2j + 1
        // ---------------- forward ----------------
        for (uint32_t j = 0; j <= H && ok; j++) {
            const uint32_t nout = tc_n_out(j, H), nin = tc_n_in(j, K0);
            if (issuer) {
                tc::fence_after_sync();
                const uint32_t idesc = tc::idesc_f16(kTcRows, nout, BF16);
                const uint32_t w_addr = base + tc_w_off(j, K0), a_addr = x_addr(j);
                for (uint32_t k = 0; k < nin / 16u; k++) {
                    const uint64_t ad = tc::smem_desc(a_addr + 2u * k * kColBlock, kColBlock, 128u);
                    const uint64_t bd = tc::smem_desc(w_addr + 2u * k * (nout * 16u), nout * 16u, 128u);
                    tc::mma_f16(tmem, ad, bd, idesc, k > 0u ? 1u : 0u);
                }
                tc::mma_commit(bar_mma);
            }
            mma_pending = true;
            if (!(ok = mma_done()))
                break;
            if (j < H) { // X_{j+1} = relu(Z_{j+1}) in the MLP precision (FP8 mode: E4M3 into hidden matrices)
                uint32_t v[4][16];
#pragma unroll
                for (int q = 0; q < 4; q++)
                    tc::tmem_ld16(tmem + lane_off + 16u * q, v[q]);
                tc::tmem_wait_ld();
                uint32_t packed[32];
                const bool quant = FP8 && j + 1u < H;
                uint32_t m0 = 0u, m1 = 0u;
#pragma unroll
                for (int c = 0; c < 32; c++) {
                    const float lo = __uint_as_float(v[c >> 3][(2 * c) & 15]);
                    const float hi = __uint_as_float(v[c >> 3][(2 * c + 1) & 15]);
                    const uint32_t p = quant ? fp8_act_relu_half2(lo, hi) : pack_relu<BF16>(lo, hi);
                    packed[c] = p;
                    const uint32_t bits = ((p & 0xFFFFu) != 0u ? 1u : 0u) | ((p >> 16) != 0u ? 2u : 0u);
                    if (c < 16)
                        m0 |= bits << (2 * c);
                    else
                        m1 |= bits << (2 * (c - 16));
                }
                relu_mask[2u * (j + 1u)] = m0;
                relu_mask[2u * (j + 1u) + 1u] = m1;
                store_row_chunks(smem + a.x_off[j + 1u], tid, packed, 8u);
            } else { // sigmoid, composite loss, dZ_out
                uint32_t v[8];
                tc::tmem_ld8(tmem + lane_off, v);
                tc::tmem_wait_ld();
                float tgt[8];
                if (valid) {
                    const float4 t0 = __ldg(reinterpret_cast<const float4 *>(a.targets + (size_t)row * 8u));
                    const float4 t1 = __ldg(reinterpret_cast<const float4 *>(a.targets + (size_t)row * 8u) + 1);
                    tgt[0] = t0.x, tgt[1] = t0.y, tgt[2] = t0.z, tgt[3] = t0.w;
                    tgt[4] = t1.x, tgt[5] = t1.y, tgt[6] = t1.z, tgt[7] = t1.w;
                }
                float dz[8], val[8];
#pragma unroll
                for (int ch = 0; ch < 8; ch++) {
                    const float y = 1.0f / (1.0f + expf(-__uint_as_float(v[ch])));
                    float value = 0.f, gr = 0.f;
                    if (valid) {
                        composite_loss(a.lc, (uint32_t)ch, y, tgt[ch], tgt[0], value, gr);
                        gr = Pr::round(gr); // 16-bit output gradient
                    }
                    val[ch] = value;
                    dz[ch] = gr * y * (1.0f - y); // sigmoid backward
                }
                const float rl = ((val[0] + val[1]) + (val[2] + val[3])) + ((val[4] + val[5]) + (val[6] + val[7]));
                loss_acc += rl;
                if (valid && a.emit && a.sample_loss)
                    a.sample_loss[row] = rl;
                uint32_t packed[8] = {Pr::pack(dz[0], dz[1]), Pr::pack(dz[2], dz[3]), Pr::pack(dz[4], dz[5]),
                                      Pr::pack(dz[6], dz[7]), 0u, 0u, 0u, 0u};
                store_row_chunks(smem + a.dzo_off, tid, packed, 2u);
            }
            tc::fence_async_shared(); // the tile rows written above are read by the next MMAs
            tc::fence_before_sync();
            __syncthreads();
        }
        // ---------------- backward ----------------
        for (int jj = (int)H; jj >= (int)a.min_matrix && ok; jj--) {
            const uint32_t j = (uint32_t)jj;
            const uint32_t nout = tc_n_out(j, H), nin = tc_n_in(j, K0);
            const uint32_t dz_addr = base + (j == H ? a.dzo_off : a.dz_off);
            const bool dgrad = j > a.min_matrix || (j == 0u && a.emit);
            const bool wgrad = (a.wg_mask >> j) & 1u;
            if (issuer) {
                tc::fence_after_sync();
                if (dgrad) { // dX_j (128 x nin) = dZ_{j+1} (128 x nout) . W_j (nout x nin), W_j MN-major
                    const uint32_t idesc = tc::idesc_f16_major(kTcRows, nin, BF16, false, true);
                    const uint32_t w_addr = base + tc_w_off(j, K0);
                    for (uint32_t k = 0; k < nout / 16u; k++) {
                        const uint64_t ad = tc::smem_desc(dz_addr + 2u * k * kColBlock, kColBlock, 128u);
                        const uint64_t bd = tc::smem_desc(w_addr + 256u * k, 128u, nout * 16u);
                        tc::mma_f16(tmem, ad, bd, idesc, k > 0u ? 1u : 0u);
                    }
                }
                if (wgrad) { // dW_j^T (128 x nout; rows >= nin unused) += X_j^T . dZ_{j+1}, K = the 128 rows
                    const uint32_t idesc = tc::idesc_f16_major(kTcRows, nout, BF16, true, true);
                    const uint32_t xa = x_addr(j);
                    for (uint32_t k = 0; k < kTcRows / 16u; k++) {
                        const uint64_t ad = tc::smem_desc(xa + 256u * k, 128u, kColBlock);
                        const uint64_t bd = tc::smem_desc(dz_addr + 256u * k, 128u, kColBlock);
                        tc::mma_f16(tmem + a.wg_col[j], ad, bd, idesc, (first_tile && k == 0u) ? 0u : 1u);
                    }
                }
                tc::mma_commit(bar_mma);
            }
            mma_pending = true;
            if (!(ok = mma_done()))
                break;
            if (j >= 1u && j > a.min_matrix) { // dZ_j = dX_j * (X_j > 0), 16-bit
                uint32_t v[4][16];
#pragma unroll
                for (int q = 0; q < 4; q++)
                    tc::tmem_ld16(tmem + lane_off + 16u * q, v[q]);
                tc::tmem_wait_ld();
                const uint32_t m0 = relu_mask[2u * j], m1 = relu_mask[2u * j + 1u];
                uint32_t packed[32];
#pragma unroll
                for (int c = 0; c < 32; c++) {
                    const uint32_t bits = (c < 16 ? m0 >> (2 * c) : m1 >> (2 * (c - 16))) & 3u;
                    const float lo = (bits & 1u) ? __uint_as_float(v[c >> 3][(2 * c) & 15]) : 0.f;
                    const float hi = (bits & 2u) ? __uint_as_float(v[c >> 3][(2 * c + 1) & 15]) : 0.f;
                    packed[c] = Pr::pack(lo, hi);
                }
                store_row_chunks(smem + a.dz_off, tid, packed, 8u);
            } else if (j == 0u && a.emit) { // dX_0, rounded to the MLP precision, for the grid scatter
                uint4 *dst = reinterpret_cast<uint4 *>(a.dfeat + (size_t)row * K0);
                for (uint32_t q = 0; q < K0 / 16u; q++) {
                    uint32_t v[16];
                    tc::tmem_ld16(tmem + lane_off + 16u * q, v); // warp-wide: rows past the batch too
                    tc::tmem_wait_ld();
                    if (valid) {
                        uint32_t w[8];
#pragma unroll
                        for (int c = 0; c < 8; c++)
                            w[c] = Pr::pack(__uint_as_float(v[2 * c]), __uint_as_float(v[2 * c + 1]));
                        dst[2u * q] = make_uint4(w[0], w[1], w[2], w[3]);
                        dst[2u * q + 1u] = make_uint4(w[4], w[5], w[6], w[7]);
                    }
                }
            }
            tc::fence_async_shared();
            tc::fence_before_sync();
            __syncthreads();
        }
        first_tile = false;
    }
    if (!ok) {
        // a wait ran out: record it, give copies and MMAs still in flight one more bounded wait
        if (issuer) {
            atomicOr(a.status, 1u);
            for (uint32_t b = 0; b < 2u; b++)
                if (load_pending[b])
                    tc::mbar_wait(tc::smem_addr(&bars[1u + b]), ph_load[b]);
            if (mma_pending)
                tc::mbar_wait(bar_mma, ph_mma);
        }
    } else if (!first_tile) {
        // the CTA's weight gradients: lane m of the dW_j^T accumulator holds column m of dW_j
        for (uint32_t j = 0; j <= H; j++) {
            if (!((a.wg_mask >> j) & 1u))
                continue;
            const uint32_t nout = tc_n_out(j, H), nin = tc_n_in(j, K0);
            float *g = a.grad + tc_param_off(j, K0);
            for (uint32_t q = 0; q < nout / 16u; q++) {
                uint32_t v[16];
                tc::tmem_ld16(tmem + lane_off + a.wg_col[j] + 16u * q, v);
                tc::tmem_wait_ld();
                if (tid < nin) {
#pragma unroll
                    for (int c = 0; c < 16; c++) {
                        const float x = __uint_as_float(v[c]);
                        if (x != 0.f)
                            atomicAdd(g + (size_t)(16u * q + (uint32_t)c) * nin + tid, x);
                    }
                }
            }
        }
        if (a.emit) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
                loss_acc += __shfl_xor_sync(kFull, loss_acc, off);
            if ((tid & 31u) == 0u && loss_acc != 0.f)
                atomicAdd(a.loss_sum, loss_acc);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0u) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kTcTmemCols);
    }
}

// ---------------------------------------------------------------------------------------------
// Hash-grid gradient scatter: one thread per (row, point), the levels in order; the corners and
// weights of the forward encoding, each corner's F feature gradients added with vector atomics
// (the 16-bit input-feature gradients come from k_train_tc).
// ---------------------------------------------------------------------------------------------

template <bool BF16>
__global__ void __launch_bounds__(256) k_grid_scatter(const __grid_constant__ GridParams grid,
                                                      const float *__restrict__ positions,
                                                      const __half *__restrict__ dfeat, uint32_t n,
                                                      float *__restrict__ grid_grad)
{
    const uint32_t P = grid.n_points, L = grid.n_levels, F = grid.n_features, n_in = grid.n_inputs;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * P)
        return;
    const uint32_t row = (uint32_t)(i / P), p = (uint32_t)(i - (uint64_t)row * P);
    const float *src = positions + i * 3u;
    const V3 pp = mk3(__ldg(src), __ldg(src + 1), __ldg(src + 2));
    const uint32_t *gw = reinterpret_cast<const uint32_t *>(dfeat + (size_t)row * n_in + (size_t)p * L * F);
    for (uint32_t l = 0; l < L; l++) {
        float g[8];
        bool any = false;
        for (uint32_t q = 0; q < F / 2u; q++) {
            const float2 v = MlpPrec<BF16>::unpack(__ldg(gw + l * (F / 2u) + q));
            g[2 * q] = v.x;
            g[2 * q + 1] = v.y;
            any |= v.x != 0.f || v.y != 0.f;
        }
        if (!any)
            continue;
        const float s = grid.scale[l];
        const float px = __fmaf_rn(pp.x, s, 0.5f), py = __fmaf_rn(pp.y, s, 0.5f), pz = __fmaf_rn(pp.z, s, 0.5f);
        const float flx = floorf(px), fly = floorf(py), flz = floorf(pz);
        const uint32_t gx = (uint32_t)(int32_t)flx, gy = (uint32_t)(int32_t)fly, gz = (uint32_t)(int32_t)flz;
        const float rx = __fsub_rn(px, flx), ry = __fsub_rn(py, fly), rz = __fsub_rn(pz, flz);
        const uint32_t res = grid.res[l], size = grid.size[l], off = grid.offset[l];
        const bool hashed = grid.hashed[l] != 0u;
        auto corner = [&](uint32_t c, uint32_t &idx, float &w) {
            const uint32_t x = gx + (c & 1u), y = gy + ((c >> 1) & 1u), z = gz + ((c >> 2) & 1u);
            if (hashed) {
                idx = (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (size - 1u);
            } else {
                idx = x + y * res + z * res * res;
                if (idx >= size)
                    idx %= size;
            }
            w = __fmul_rn(__fmul_rn((c & 1u) ? rx : __fsub_rn(1.0f, rx), (c & 2u) ? ry : __fsub_rn(1.0f, ry)),
                          (c & 4u) ? rz : __fsub_rn(1.0f, rz));
        };
        // corners in pairs (x, x + 1): with 2 features, a pair whose entries are the two halves of
        // one aligned 16-byte word (every even x on hashed levels, every even entry on dense
        // ones) takes one 16-byte atomic instead of two 8-byte ones
#pragma unroll
        for (uint32_t c = 0; c < 8; c += 2) {
            uint32_t i0, i1;
            float w0, w1;
            corner(c, i0, w0);
            corner(c + 1u, i1, w1);
            if (F == 2u) {
                const uint32_t e0 = off + i0, e1 = off + i1;
                if ((e0 ^ e1) == 1u) {
                    const uint32_t lo = e0 < e1 ? e0 : e1;
                    const float wl = e0 < e1 ? w0 : w1, wh = e0 < e1 ? w1 : w0;
                    atomicAdd(reinterpret_cast<float4 *>(grid_grad + (size_t)lo * 2u),
                              make_float4(wl * g[0], wl * g[1], wh * g[0], wh * g[1]));
                } else {
                    atomicAdd(reinterpret_cast<float2 *>(grid_grad + (size_t)e0 * 2u), make_float2(w0 * g[0], w0 * g[1]));
                    atomicAdd(reinterpret_cast<float2 *>(grid_grad + (size_t)e1 * 2u), make_float2(w1 * g[0], w1 * g[1]));
                }
            } else {
                float *ea = grid_grad + (size_t)(off + i0) * F, *eb = grid_grad + (size_t)(off + i1) * F;
                for (uint32_t q = 0; q < F / 4u; q++) {
                    atomicAdd(reinterpret_cast<float4 *>(ea) + q,
                              make_float4(w0 * g[4 * q], w0 * g[4 * q + 1], w0 * g[4 * q + 2], w0 * g[4 * q + 3]));
                    atomicAdd(reinterpret_cast<float4 *>(eb) + q,
                              make_float4(w1 * g[4 * q], w1 * g[4 * q + 1], w1 * g[4 * q + 2], w1 * g[4 * q + 3]));
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// K5: Adam + ExponentialDecay (step size precomputed on the host with the bias corrections),
// FP32 master weights, m and v; writes the FP16 copy the kernels read.
// ---------------------------------------------------------------------------------------------

// 16-bit copy of parameter i: the first n_bf16 parameters (the network matrices in BF16 mode) as
// BF16, those in [fp8_lo, fp8_hi) (the hidden 64x64 matrices in FP8 mode) as their FP8-E4M3 value
// at scale 2^6 (exact in FP16), the rest as FP16.
__device__ __forceinline__ __half to_param16(float x, uint32_t i, const ParamPrecision &pp)
{
    if (i < pp.n_bf16) {
        const __nv_bfloat16 b = __float2bfloat16_rn(x);
        return *reinterpret_cast<const __half *>(&b);
    }
    if (i >= pp.fp8_lo && i < pp.fp8_hi)
        return __float2half_rn(__fmul_rn(e4m3_round(__fmul_rn(x, kFp8WeightScale)), 1.0f / kFp8WeightScale));
    return __float2half_rn(x);
}

__global__ void __launch_bounds__(256) k_adam(float *__restrict__ params, __half *__restrict__ params_h,
                                              float *__restrict__ m, float *__restrict__ v,
                                              const float *__restrict__ grad, uint32_t n, float lr_t, float beta1,
                                              float beta2, float eps, float l2_reg, float grad_scale,
                                              const ParamPrecision pp)
{
    const float omb1 = __fsub_rn(1.0f, beta1), omb2 = __fsub_rn(1.0f, beta2);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float w = params[i];
        const float gr = __fadd_rn(__fmul_rn(grad[i], grad_scale), __fmul_rn(l2_reg, w));
        const float mi = __fadd_rn(__fmul_rn(beta1, m[i]), __fmul_rn(omb1, gr));
        const float vi = __fadd_rn(__fmul_rn(beta2, v[i]), __fmul_rn(omb2, __fmul_rn(gr, gr)));
        m[i] = mi;
        v[i] = vi;
        const float nw = __fsub_rn(w, __fmul_rn(lr_t, __fdiv_rn(mi, __fadd_rn(__fsqrt_rn(vi), eps))));
        params[i] = nw;
        params_h[i] = to_param16(nw, i, pp);
    }
}

__global__ void k_to_half(const float *__restrict__ p, __half *__restrict__ h, uint32_t n, const ParamPrecision pp)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        h[i] = to_param16(p[i], i, pp);
}

__global__ void k_scale(float *__restrict__ p, size_t n, float s)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] *= s;
}

// One launch of k_train_tc: the matrices whose weight gradients it accumulates (wg_mask), whether
// it also writes the loss and the feature gradients (the launch that reaches matrix 0), and its
// shared-memory layout and TMEM columns.
struct TrainTcPass {
    TrainTcArgs a;
    size_t smem;
};

constexpr size_t kTcSmemLimit = 227u * 1024u;
constexpr size_t kTcSmPerSm = 228u * 1024u;

// Lays out one pass over the matrices in `mask`; false if it does not fit shared memory or TMEM.
bool plan_train_pass(uint32_t n_in, uint32_t H, uint32_t mask, bool emit, TrainTcPass &p)
{
    TrainTcArgs &a = p.a;
    std::memset(&a, 0, sizeof(a));
    const uint32_t wbytes = packed_weight_bytes(n_in, H);
    uint32_t off = (wbytes + 1023u) & ~1023u;
    a.wbytes = wbytes;
    a.x0_off = off;
    off += 2u * n_in * kTcRows * 2u;
    bool transient = false;
    for (uint32_t j = 1; j <= H; j++) {
        if ((mask >> j) & 1u) {
            a.x_off[j] = off;
            off += kNeurons * kTcRows * 2u;
        } else {
            transient = true;
        }
    }
    if (transient) {
        for (uint32_t j = 1; j <= H; j++)
            if (!((mask >> j) & 1u))
                a.x_off[j] = off;
        off += kNeurons * kTcRows * 2u;
    }
    // the weight-gradient MMAs read 128 columns of every X tile (rows past the matrix's input width
    // are ignored): a 64-column tile is always followed by at least 16 KB (the next tile or dZ)
    a.dz_off = off;
    off += kNeurons * kTcRows * 2u;
    a.dzo_off = off;
    off += kOutputsPadded * kTcRows * 2u;
    a.bar_off = off;
    off += 64u;
    uint32_t col = kTcAccCols;
    for (uint32_t j = 0; j <= H; j++) {
        if (!((mask >> j) & 1u))
            continue;
        a.wg_col[j] = col;
        col += tc_n_out(j, H);
    }
    if (col > kTcTmemCols || off > kTcSmemLimit)
        return false;
    uint32_t lo = H;
    for (uint32_t j = 0; j <= H; j++)
        if ((mask >> j) & 1u) {
            lo = j;
            break;
        }
    a.wg_mask = mask;
    a.emit = emit ? 1u : 0u;
    a.min_matrix = emit ? 0u : lo;
    // at least half an SM of shared memory, so that one CTA (and its 512 TMEM columns) per SM
    const size_t one_per_sm = kTcSmPerSm / 2u - 1024u + 128u;
    p.smem = off < one_per_sm ? one_per_sm : off;
    return true;
}

// The passes: all matrices in one launch when they fit (up to 5 hidden layers), else groups of
// matrices from the output matrix down, the last group (with matrix 0) writing the loss.
std::vector<TrainTcPass> plan_train_passes(uint32_t n_in, uint32_t H)
{
    std::vector<TrainTcPass> passes;
    TrainTcPass p;
    const uint32_t all = (1u << (H + 1u)) - 1u;
    if (plan_train_pass(n_in, H, all, true, p)) {
        passes.push_back(p);
        return passes;
    }
    uint32_t mask = 0u;
    for (int j = (int)H; j >= 0; j--) {
        const uint32_t trial = mask | (1u << j);
        if (plan_train_pass(n_in, H, trial, j == 0, p)) {
            mask = trial;
            if (j == 0)
                passes.push_back(p);
            continue;
        }
        TrainTcPass done;
        plan_train_pass(n_in, H, mask, false, done);
        passes.push_back(done);
        mask = 1u << j;
        if (j == 0) {
            plan_train_pass(n_in, H, mask, true, p);
            passes.push_back(p);
        }
    }
    return passes;
}

} // namespace

cudaError_t launch_training_samples(const float4 *neural_nodes, const float4 *nodes, const float4 *tris,
                                    const float *albedo, const NeuralConsts &nc, const GridParams &grid,
                                    uint32_t training_step, uint32_t batch_size, uint32_t n, float *positions,
                                    float *targets, uint32_t *sample_nodes, uint32_t learned_lod,
                                    const NodeSurvival *survival, float4 *state, bool classic_fast_div, int num_sms,
                                    cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    SampleArgs a;
    a.grid = grid;
    a.nc = nc;
    a.neural_nodes = neural_nodes;
    a.nodes = nodes;
    a.tris = tris;
    a.albedo = albedo;
    a.positions = positions;
    a.targets = targets;
    a.sample_nodes = sample_nodes;
    a.training_step = training_step;
    a.batch_size = batch_size;
    a.n = n;
    a.learned_lod = learned_lod < kNumBvhLods ? learned_lod : kNumBvhLods - 1u;
    a.classic_fast_div = classic_fast_div ? 1u : 0u;
    if (survival && survival->enabled && survival->stats)
        a.survival = *survival;
    else
        a.survival = NodeSurvival{nullptr, nullptr, 1.0f, 0.0f, 0u};
    SampleFound *found = reinterpret_cast<SampleFound *>(state);
    uint32_t *counter = reinterpret_cast<uint32_t *>(found + n);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return e;
    uint32_t blocks = (n + kFindThreads - 1u) / kFindThreads;
    if (blocks > (uint32_t)num_sms * 4u)
        blocks = (uint32_t)num_sms * 4u;
    k_training_find<<<blocks, kFindThreads, 0, s>>>(a, found, counter);
    k_training_samples<<<(n + 127u) / 128u, 128, 0, s>>>(a, found);
    return cudaGetLastError();
}

cudaError_t launch_encode_rows(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                               const float *positions, uint32_t n, __half *features, bool bf16, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    const uint32_t n_network_params =
        kNeurons * grid.n_inputs + (n_hidden_layers - 1u) * kNeurons * kNeurons + kOutputsPadded * kNeurons;
    const uint32_t *table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    const uint64_t threads = (uint64_t)n * grid.n_points;
    k_train_encode<<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(grid, table, positions, n, features,
                                                                      grid.n_inputs, bf16 ? 1u : 0u);
    return cudaGetLastError();
}

cudaError_t launch_train_step(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                              const LossConsts &lc, const float *positions, const float *targets, uint32_t n,
                              __half *features, __half *dfeat, __half *wpacked, float *grad, float *loss_sum,
                              float *sample_loss, uint32_t *status, bool bf16, bool fp8, int num_sms, cudaStream_t s,
                              uint64_t wait_ns, bool stall, const cudaEvent_t *marks)
{
    if (n == 0)
        return cudaSuccess;
    cudaError_t e = marks ? cudaEventRecord(marks[0], s) : cudaSuccess;
    if (e != cudaSuccess)
        return e;
    const uint32_t H = n_hidden_layers, n_in = grid.n_inputs;
    const uint32_t n_network_params =
        kNeurons * n_in + (H - 1u) * kNeurons * kNeurons + kOutputsPadded * kNeurons;
    const uint32_t *table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    {
        const uint64_t threads = (uint64_t)n * grid.n_points;
        k_train_encode<<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(grid, table, positions, n, features, n_in,
                                                                          bf16 ? 1u : 0u);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = launch_pack_weights(params_h, n_in, H, wpacked, s);
    if (e == cudaSuccess && marks)
        e = cudaEventRecord(marks[1], s);
    if (e != cudaSuccess)
        return e;
    TensorMapBytes mb;
    if ((e = make_feature_map(features, n_in, n, &mb, false)) != cudaSuccess)
        return e;
    CUtensorMap fmap;
    std::memcpy(&fmap, mb.bytes, sizeof(fmap));
    auto kernel = bf16 ? k_train_tc<true, false> : (fp8 ? k_train_tc<false, true> : k_train_tc<false, false>);
    if ((e = allow_max_dynamic_smem(kernel)) != cudaSuccess)
        return e;
    const uint32_t tiles = (n + kTcRows - 1u) / kTcRows;
    const uint32_t blocks = tiles < (uint32_t)num_sms ? tiles : (uint32_t)num_sms;
    for (TrainTcPass &p : plan_train_passes(n_in, H)) {
        TrainTcArgs &a = p.a;
        a.wpacked = wpacked;
        a.n_inputs = n_in;
        a.n_hidden_layers = H;
        a.n = n;
        a.targets = targets;
        a.lc = lc;
        a.dfeat = dfeat;
        a.grad = grad;
        a.loss_sum = loss_sum;
        a.sample_loss = sample_loss;
        a.status = status;
        a.wait_ns = wait_ns ? wait_ns : tc::kWaitLimitNs;
        a.stall = stall ? 1u : 0u;
        kernel<<<blocks, kTcThreads, p.smem, s>>>(fmap, a);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
    }
    if (marks && (e = cudaEventRecord(marks[2], s)) != cudaSuccess)
        return e;
    const uint64_t threads = (uint64_t)n * grid.n_points;
    if (bf16)
        k_grid_scatter<true><<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(grid, positions, dfeat, n,
                                                                                 grad + n_network_params);
    else
        k_grid_scatter<false><<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(grid, positions, dfeat, n,
                                                                                  grad + n_network_params);
    e = cudaGetLastError();
    if (e == cudaSuccess && marks)
        e = cudaEventRecord(marks[3], s);
    return e;
}

cudaError_t launch_scale(float *data, size_t n, float scale, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    k_scale<<<1024, 256, 0, s>>>(data, n, scale);
    return cudaGetLastError();
}

cudaError_t launch_adam(float *params, __half *params_h, float *m, float *v, const float *grad, uint32_t n, float lr_t,
                        float beta1, float beta2, float eps, float l2_reg, float grad_scale, const ParamPrecision &pp,
                        cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    uint32_t blocks = (n + 255u) / 256u;
    if (blocks > 8192u)
        blocks = 8192u;
    k_adam<<<blocks, 256, 0, s>>>(params, params_h, m, v, grad, n, lr_t, beta1, beta2, eps, l2_reg, grad_scale, pp);
    return cudaGetLastError();
}

cudaError_t launch_params_to_half(const float *params, __half *params_h, uint32_t n, const ParamPrecision &pp,
                                  cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    uint32_t blocks = (n + 255u) / 256u;
    if (blocks > 8192u)
        blocks = 8192u;
    k_to_half<<<blocks, 256, 0, s>>>(params, params_h, n, pp);
    return cudaGetLastError();
}

} // namespace nbvh
