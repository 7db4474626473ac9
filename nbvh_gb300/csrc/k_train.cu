// k_train.cu -- run-optimisation kernels: training-ray generation and labelling on the device,
// fused forward + composite loss + backward (K3/K4 backward, hash-grid gradient scatter), the
// weight-gradient pass on the tensor cores, and the fused Adam step (K5).
//
// Reference path: NeuralBVHRenderer::render, m_run_optimisation branch
// (src/cuda/neural/neural_bvh_renderer.cu:141-288): granular_sample_bvh_network_input_data
// (src/cuda/neural/neural_bvh_module_kernels.cu:119-264), then tcnn's trainer->training_step
// (encoding + FullyFusedMLP forward, PathTracingCompositeLoss, backward, Adam wrapped in
// ExponentialDecay; configured at src/cuda/neural/neural_bvh_module.cu:118-263).
#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"

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

__global__ void __launch_bounds__(128) k_training_samples(const __grid_constant__ SampleArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const NeuralConsts &c = a.nc;
    const V3 smin = mk3(c.scene_min[0], c.scene_min[1], c.scene_min[2]);
    const V3 smax = mk3(c.scene_max[0], c.scene_max[1], c.scene_max[2]);
    uint32_t rng = lcg_seed(a.training_step * a.batch_size, 0u, i);
    const float sx = lcg_randomf(rng);
    const float sy = lcg_randomf(rng);
    const V3 dir = uniform_sphere(sx, sy);
    // sampled LoD among the ones learned so far (common.cuh:719-721)
    const uint32_t n_lods = kNumBvhLods - a.learned_lod;
    const uint32_t lod_pick = __float2uint_rz(__fmul_rn(lcg_randomf(rng), __uint2float_rn(n_lods)));
    const uint32_t sampled_lod = a.learned_lod + min(lod_pick, n_lods - 1u);
    const float dil = __fadd_rn(c.fixed_node_dilation, __fmul_rn(lcg_randomf(rng), c.node_extent_dilation));
    uint32_t stack[kNeuralStackSize];
    int sp = 0;
    bool valid = false;
    V3 o = mk3(0, 0, 0), d = dir;
    float mint = 0.f, maxt = 0.f;
    uint32_t node = 0;
    uint32_t guard = 0;
    const float h = __fmul_rn(__fsub_rn(c.sampling_bbox_scaling, 1.0f), 0.5f);
    do {
        if (!valid) {
            stack[0] = 0;
            sp = 1;
            const float px = lcg_randomf(rng);
            const float py = lcg_randomf(rng);
            const float pz = lcg_randomf(rng);
            V3 ps = sub3(scale3(mk3(px, py, pz), c.sampling_bbox_scaling), mk3(h, h, h));
            o = add3(mul3(ps, sub3(smax, smin)), smin);
            d = dir;
        }
        int res = neural_intersect(a.neural_nodes, sampled_lod, o, d, stack, sp, false, c.inference_mint_epsilon,
                                   c.inference_maxt_epsilon, c.learning_mint_epsilon, c.learning_maxt_epsilon, FLT_MAX,
                                   dil, mint, maxt, node);
        valid = (res == 1);
        if (res < 0)
            sp = 0;
    } while (!valid && ++guard < 100000u);

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
    classic_traverse<false>(a.nodes, a.tris, o, d, mint, maxt, t, u, v, prim, &rec);
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
// Fused forward + loss + backward (data gradients). One warp per 16-row tile. Per row it writes
// the FP16 input activation of every layer (acts) and the pre-activation gradient of every layer
// (dz) for the weight-gradient pass, and scatters the input-feature gradient into the hash-grid
// gradient with 64-bit vector atomics.
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const void *p)
{
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// The hash-grid features of the training rows, in the MLP precision, into the first n_inputs
// activations of each row (acts row stride acts_stride halves): one thread per (row, point), the
// levels in order, F features per level stored together.
__global__ void __launch_bounds__(256) k_train_encode(const __grid_constant__ GridParams grid,
                                                      const uint32_t *__restrict__ table,
                                                      const float *__restrict__ positions, uint32_t n,
                                                      __half *__restrict__ acts, uint32_t acts_stride, uint32_t bf16)
{
    const uint32_t P = grid.n_points, L = grid.n_levels, F = grid.n_features;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * P)
        return;
    const uint32_t row = (uint32_t)(i / P), p = (uint32_t)(i - (uint64_t)row * P);
    const float *src = positions + i * 3u;
    const V3 pos = mk3(__ldg(src), __ldg(src + 1), __ldg(src + 2));
    auto pack16 = [bf16](float lo, float hi) { return bf16 ? pack_bf162(lo, hi) : pack_half2(lo, hi); };
    __half *dst = acts + (size_t)row * acts_stride + (size_t)p * L * F;
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
            const float2 f = encode_level(table, grid, l, pos);
            *reinterpret_cast<uint32_t *>(dst + 2u * l) = pack16(f.x, f.y);
        }
    }
}

struct TrainArgs {
    GridParams grid;
    LossConsts lc;
    const uint32_t *table;
    const __half *weights;
    const float *positions;
    const float *targets;
    __half *acts;      // n x acts_stride
    __half *dz;        // n x dz_stride
    float2 *grid_grad; // n_grid_entries x (n_features / 2) feature pairs
    float *loss_sum;
    float *sample_loss; // per row: sum of its output channels' loss values (may be NULL)
    uint32_t fp8;       // hidden-matrix inputs rounded to FP8-E4M3 (straight-through in the backward)
    uint32_t n_hidden_layers;
    uint32_t n;
};

constexpr int kTrainWarps = 8;
constexpr int kTrainThreads = kTrainWarps * 32;

template <bool BF16, bool FP8>
__global__ void __launch_bounds__(kTrainThreads, 1) k_train_fwd_bwd(const __grid_constant__ TrainArgs a)
{
    using Pr = MlpPrec<BF16>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GridParams &gp = *reinterpret_cast<GridParams *>(smem_raw);
    const uint32_t n_in = a.grid.n_inputs, P = a.grid.n_points, L = a.grid.n_levels, H = a.n_hidden_layers;
    const SmemNetLayout SL = smem_net_layout(n_in, H);
    __half *sw = reinterpret_cast<__half *>(smem_raw + kGridParamsSmem);
    {
        const uint32_t *s = reinterpret_cast<const uint32_t *>(&a.grid);
        uint32_t *dd = reinterpret_cast<uint32_t *>(&gp);
        for (uint32_t i = threadIdx.x; i < sizeof(GridParams) / 4u; i += blockDim.x)
            dd[i] = s[i];
    }
    load_weights_to_smem(a.weights, sw, n_in, H);
    __syncthreads();

    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const uint32_t acts_stride = n_in + H * kNeurons, dz_stride = H * kNeurons + kOutputsPadded;
    const uint32_t n_tiles = (a.n + 15u) / 16u;
    const uint32_t warps_total = gridDim.x * kTrainWarps;
    float loss_acc = 0.f;

    for (uint32_t tile = blockIdx.x * kTrainWarps + (threadIdx.x >> 5); tile < n_tiles; tile += warps_total) {
        const uint32_t r0 = tile * 16u + g, r1 = r0 + 8u;
        const bool act0 = r0 < a.n, act1 = r1 < a.n;
        auto pos_of = [&](uint32_t row, uint32_t p) -> V3 {
            const float *src = a.positions + ((size_t)row * P + p) * 3u;
            return mk3(__ldg(src), __ldg(src + 1), __ldg(src + 2));
        };
        // ---------------- forward ----------------
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
            acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
        for (uint32_t kb = 0; kb < n_in / 16u; kb++) {
            // the encoded features (k_train_encode wrote them to the rows' first n_in activations)
            uint32_t af[4];
            auto feat = [&](bool act, uint32_t row, uint32_t col) -> uint32_t {
                return act ? *reinterpret_cast<const uint32_t *>(a.acts + (size_t)row * acts_stride + col) : 0u;
            };
            af[0] = feat(act0, r0, kb * 16u + tig * 2u);
            af[1] = feat(act1, r1, kb * 16u + tig * 2u);
            af[2] = feat(act0, r0, kb * 16u + tig * 2u + 8u);
            af[3] = feat(act1, r1, kb * 16u + tig * 2u + 8u);
            const __half *wrow = sw + g * SL.ld0 + kb * 16u + tig * 2;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                uint32_t b0 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * SL.ld0);
                uint32_t b1 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * SL.ld0 + 8);
                Pr::mma(acc[nt], af, b0, b1);
            }
        }
        uint32_t ah[4][4];
        for (uint32_t layer = 1; layer <= H; layer++) {
            relu_pack<BF16, FP8>(acc, ah, layer < H); // FP8 mode: inputs of the hidden matrices
            // store x_layer (input of matrix `layer`)
            __half *dst0 = a.acts + (size_t)r0 * acts_stride + n_in + (layer - 1u) * kNeurons;
            __half *dst1 = a.acts + (size_t)r1 * acts_stride + n_in + (layer - 1u) * kNeurons;
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
                if (act0) {
                    *reinterpret_cast<uint32_t *>(dst0 + kb * 16 + tig * 2) = ah[kb][0];
                    *reinterpret_cast<uint32_t *>(dst0 + kb * 16 + tig * 2 + 8) = ah[kb][2];
                }
                if (act1) {
                    *reinterpret_cast<uint32_t *>(dst1 + kb * 16 + tig * 2) = ah[kb][1];
                    *reinterpret_cast<uint32_t *>(dst1 + kb * 16 + tig * 2 + 8) = ah[kb][3];
                }
            }
            if (layer == H)
                break;
            const __half *wl = sw + SL.hidden_off + (layer - 1u) * kNeurons * kHiddenLd;
#pragma unroll
            for (int nt = 0; nt < 8; nt++)
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
                const __half *wrow = wl + g * kHiddenLd + kb * 16 + tig * 2;
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    uint32_t b0 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * kHiddenLd);
                    uint32_t b1 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * kHiddenLd + 8);
                    Pr::mma(acc[nt], ah[kb], b0, b1);
                }
            }
        }
        // output layer: only columns 0..7 carry outputs
        float oc[4] = {0.f, 0.f, 0.f, 0.f};
        {
            const __half *wo = sw + SL.out_off + g * kHiddenLd + tig * 2;
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
                uint32_t b0 = *reinterpret_cast<const uint32_t *>(wo + kb * 16);
                uint32_t b1 = *reinterpret_cast<const uint32_t *>(wo + kb * 16 + 8);
                Pr::mma(oc, ah[kb], b0, b1);
            }
        }
        // ---------------- loss ----------------
        float dzo[4], row_vals[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const uint32_t row = (e < 2) ? r0 : r1;
            const bool act = (e < 2) ? act0 : act1;
            const uint32_t ch = (uint32_t)tig * 2u + (uint32_t)(e & 1);
            float y = 1.0f / (1.0f + expf(-oc[e]));
            float value = 0.f, gr = 0.f;
            if (act) {
                const float tgt = __ldg(a.targets + (size_t)row * 8u + ch);
                const float tvis = __ldg(a.targets + (size_t)row * 8u);
                composite_loss(a.lc, ch, y, tgt, tvis, value, gr);
                gr = Pr::round(gr); // 16-bit output gradient
            }
            loss_acc += value;
            row_vals[e] = value;
            dzo[e] = gr * y * (1.0f - y); // sigmoid backward
        }
        if (a.sample_loss) { // the four lanes of a quad hold the eight channels of rows r0 and r1
            float l0 = row_vals[0] + row_vals[1], l1 = row_vals[2] + row_vals[3];
            l0 += __shfl_xor_sync(kFull, l0, 1);
            l1 += __shfl_xor_sync(kFull, l1, 1);
            l0 += __shfl_xor_sync(kFull, l0, 2);
            l1 += __shfl_xor_sync(kFull, l1, 2);
            if (tig == 0) {
                if (act0)
                    a.sample_loss[r0] = l0;
                if (act1)
                    a.sample_loss[r1] = l1;
            }
        }
        // dz_out (cols 0..7; 8..15 stay zero)
        {
            uint32_t lo = Pr::pack(dzo[0], dzo[1]), hi = Pr::pack(dzo[2], dzo[3]);
            if (act0) {
                __half *dst = a.dz + (size_t)r0 * dz_stride + H * kNeurons;
                *reinterpret_cast<uint32_t *>(dst + tig * 2) = lo;
                *reinterpret_cast<uint32_t *>(dst + 8 + tig * 2) = 0u;
            }
            if (act1) {
                __half *dst = a.dz + (size_t)r1 * dz_stride + H * kNeurons;
                *reinterpret_cast<uint32_t *>(dst + tig * 2) = hi;
                *reinterpret_cast<uint32_t *>(dst + 8 + tig * 2) = 0u;
            }
        }
        // ---------------- backward ----------------
        // dx_H = dz_out . W_out (K = 16 outputs, only 0..7 non-zero)
        uint32_t adz[4][4]; // A fragments of the current dz (k = out channel)
        adz[0][0] = Pr::pack(dzo[0], dzo[1]);
        adz[0][1] = Pr::pack(dzo[2], dzo[3]);
        adz[0][2] = 0u;
        adz[0][3] = 0u;
        uint32_t n_kb = 1;
        const __half *wmat = sw + SL.out_off; // matrix whose transpose maps dz to dx
        uint32_t wld = kHiddenLd;
        for (int layer = (int)H; layer >= 1; layer--) {
            // dx_layer (16 x 64) = dz . W  (B from W rows = k, contiguous in = n: ldmatrix.trans)
#pragma unroll
            for (int nt = 0; nt < 8; nt++)
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
            for (uint32_t kb = 0; kb < n_kb; kb++) {
#pragma unroll
                for (int np = 0; np < 4; np++) {
                    uint32_t b[4];
                    const __half *addr = wmat + (kb * 16u + (lane & 15)) * wld + np * 16 + (lane >> 4) * 8;
                    ldsm_x4_trans(b, addr);
                    Pr::mma(acc[2 * np], adz[kb], b[0], b[1]);
                    Pr::mma(acc[2 * np + 1], adz[kb], b[2], b[3]);
                }
            }
            // dz_layer = dx_layer * (x_layer > 0), x_layer = input activation of matrix `layer`
            const __half *x0 = a.acts + (size_t)r0 * acts_stride + n_in + (uint32_t)(layer - 1) * kNeurons;
            const __half *x1 = a.acts + (size_t)r1 * acts_stride + n_in + (uint32_t)(layer - 1) * kNeurons;
            __half *dzw0 = a.dz + (size_t)r0 * dz_stride + (uint32_t)(layer - 1) * kNeurons;
            __half *dzw1 = a.dz + (size_t)r1 * dz_stride + (uint32_t)(layer - 1) * kNeurons;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                float2 m0 = act0 ? Pr::unpack(*reinterpret_cast<const uint32_t *>(x0 + nt * 8 + tig * 2))
                                 : make_float2(0.f, 0.f);
                float2 m1 = act1 ? Pr::unpack(*reinterpret_cast<const uint32_t *>(x1 + nt * 8 + tig * 2))
                                 : make_float2(0.f, 0.f);
                acc[nt][0] = m0.x > 0.f ? acc[nt][0] : 0.f;
                acc[nt][1] = m0.y > 0.f ? acc[nt][1] : 0.f;
                acc[nt][2] = m1.x > 0.f ? acc[nt][2] : 0.f;
                acc[nt][3] = m1.y > 0.f ? acc[nt][3] : 0.f;
            }
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
                adz[kb][0] = Pr::pack(acc[2 * kb][0], acc[2 * kb][1]);
                adz[kb][1] = Pr::pack(acc[2 * kb][2], acc[2 * kb][3]);
                adz[kb][2] = Pr::pack(acc[2 * kb + 1][0], acc[2 * kb + 1][1]);
                adz[kb][3] = Pr::pack(acc[2 * kb + 1][2], acc[2 * kb + 1][3]);
                if (act0) {
                    *reinterpret_cast<uint32_t *>(dzw0 + kb * 16 + tig * 2) = adz[kb][0];
                    *reinterpret_cast<uint32_t *>(dzw0 + kb * 16 + tig * 2 + 8) = adz[kb][2];
                }
                if (act1) {
                    *reinterpret_cast<uint32_t *>(dzw1 + kb * 16 + tig * 2) = adz[kb][1];
                    *reinterpret_cast<uint32_t *>(dzw1 + kb * 16 + tig * 2 + 8) = adz[kb][3];
                }
            }
            n_kb = 4;
            wmat = (layer >= 2) ? sw + SL.hidden_off + (uint32_t)(layer - 2) * kNeurons * kHiddenLd : sw;
            wld = (layer >= 2) ? kHiddenLd : SL.ld0;
        }
        // dx_0 (16 x n_in) = dz_1 . W_0, n-tile by n-tile, scattered into the grid gradient
        for (uint32_t nt = 0; nt < n_in / 8u; nt++) {
            float dx[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
                uint32_t b[4];
                // x2 is enough here; reuse the x4 form with the upper half pointing at the same tile
                const __half *addr = sw + (kb * 16u + (lane & 15)) * SL.ld0 + nt * 8u;
                ldsm_x4_trans(b, addr);
                Pr::mma(dx, adz[kb], b[0], b[1]);
            }
            // feature pair j = nt * 4 + tig (features 2 sub, 2 sub + 1 of level l of point p) for
            // rows r0, r1
            const uint32_t j = nt * 4u + (uint32_t)tig;
            const uint32_t pairs = gp.n_features / 2u;
            const uint32_t pl = j / pairs, sub = j - pl * pairs;
            const uint32_t p = pl / L, l = pl - p * L;
#pragma unroll
            for (int rr = 0; rr < 2; rr++) {
                const bool act = rr ? act1 : act0;
                if (!act)
                    continue;
                const uint32_t row = rr ? r1 : r0;
                const float g0 = Pr::round(dx[2 * rr]);
                const float g1 = Pr::round(dx[2 * rr + 1]);
                if (g0 == 0.f && g1 == 0.f)
                    continue;
                // corner indices / weights of this (row, point, level), as encode_level
                V3 pp = pos_of(row, p);
                const float s = gp.scale[l];
                const float px = __fmaf_rn(pp.x, s, 0.5f), py = __fmaf_rn(pp.y, s, 0.5f), pz = __fmaf_rn(pp.z, s, 0.5f);
                const float flx = floorf(px), fly = floorf(py), flz = floorf(pz);
                const uint32_t gx = (uint32_t)(int32_t)flx, gy = (uint32_t)(int32_t)fly, gz = (uint32_t)(int32_t)flz;
                const float rx = __fsub_rn(px, flx), ry = __fsub_rn(py, fly), rz = __fsub_rn(pz, flz);
                const uint32_t res = gp.res[l], size = gp.size[l], off = gp.offset[l];
                const bool hashed = gp.hashed[l] != 0u;
#pragma unroll
                for (uint32_t c = 0; c < 8; c++) {
                    uint32_t x = gx + (c & 1u), y = gy + ((c >> 1) & 1u), z = gz + ((c >> 2) & 1u);
                    uint32_t idx;
                    if (hashed) {
                        idx = (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (size - 1u);
                    } else {
                        idx = x + y * res + z * res * res;
                        if (idx >= size)
                            idx %= size;
                    }
                    float w = __fmul_rn(__fmul_rn((c & 1u) ? rx : __fsub_rn(1.0f, rx), (c & 2u) ? ry : __fsub_rn(1.0f, ry)),
                                        (c & 4u) ? rz : __fsub_rn(1.0f, rz));
                    atomicAdd(a.grid_grad + (size_t)(off + idx) * pairs + sub, make_float2(w * g0, w * g1));
                }
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        loss_acc += __shfl_xor_sync(kFull, loss_acc, off);
    if (lane == 0 && loss_acc != 0.f)
        atomicAdd(a.loss_sum, loss_acc);
}

// ---------------------------------------------------------------------------------------------
// Weight gradients dW_m = sum_rows dz_m^T x_m, split over row chunks: every block stages 64 rows of
// activations and gradients in shared memory and accumulates all (m16, n8) output tiles of every
// matrix in registers (tiles dealt round-robin to the warps), then adds them to the global FP32
// gradient once.
// ---------------------------------------------------------------------------------------------

constexpr int kWgWarps = 8;
constexpr int kWgThreads = kWgWarps * 32;
constexpr uint32_t kWgRows = 64;
constexpr int kMaxTilesPerWarp = 32;

struct WgArgs {
    const __half *acts;
    const __half *dz;
    float *grad;
    uint32_t n_inputs;
    uint32_t n_hidden_layers;
    uint32_t n;
    uint32_t rows_per_block;
};

__device__ __forceinline__ void tile_info(uint32_t t, uint32_t n_in, uint32_t H, uint32_t &mat, uint32_t &mt,
                                          uint32_t &nt)
{
    const uint32_t t0 = 4u * (n_in / 8u); // tiles of matrix 0
    if (t < t0) {
        mat = 0;
        mt = t / (n_in / 8u);
        nt = t % (n_in / 8u);
        return;
    }
    t -= t0;
    const uint32_t th = 32u * (H - 1u);
    if (t < th) {
        mat = 1u + t / 32u;
        mt = (t % 32u) / 8u;
        nt = t % 8u;
        return;
    }
    t -= th;
    mat = H; // output matrix: one m-tile (16 rows), 8 n-tiles
    mt = 0;
    nt = t;
}

template <int TPW, bool BF16>
__global__ void __launch_bounds__(kWgThreads, 1) k_weight_grads(const __grid_constant__ WgArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t n_in = a.n_inputs, H = a.n_hidden_layers;
    const uint32_t acts_stride = n_in + H * kNeurons, dz_stride = H * kNeurons + kOutputsPadded;
    const uint32_t sa_ld = acts_stride + 8u, sz_ld = dz_stride + 8u;
    __half *sa = reinterpret_cast<__half *>(smem_raw);
    __half *sz = sa + kWgRows * sa_ld;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const uint32_t n_tiles = 4u * (n_in / 8u) + 32u * (H - 1u) + 8u;

    float acc[TPW][4];
#pragma unroll
    for (int i = 0; i < TPW; i++)
        acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;

    const uint32_t row_begin = blockIdx.x * a.rows_per_block;
    uint32_t row_end = row_begin + a.rows_per_block;
    if (row_end > a.n)
        row_end = a.n;
    for (uint32_t c0 = row_begin; c0 < row_end; c0 += kWgRows) {
        __syncthreads();
        // stage 64 rows (zero-filled past the end)
        const uint32_t wa = acts_stride / 2u, wz = dz_stride / 2u;
        for (uint32_t i = threadIdx.x; i < kWgRows * wa; i += blockDim.x) {
            uint32_t r = i / wa, c = i % wa;
            uint32_t v = (c0 + r < row_end) ? __ldg(reinterpret_cast<const uint32_t *>(a.acts + (size_t)(c0 + r) * acts_stride) + c) : 0u;
            *reinterpret_cast<uint32_t *>(sa + r * sa_ld + 2u * c) = v;
        }
        for (uint32_t i = threadIdx.x; i < kWgRows * wz; i += blockDim.x) {
            uint32_t r = i / wz, c = i % wz;
            uint32_t v = (c0 + r < row_end) ? __ldg(reinterpret_cast<const uint32_t *>(a.dz + (size_t)(c0 + r) * dz_stride) + c) : 0u;
            *reinterpret_cast<uint32_t *>(sz + r * sz_ld + 2u * c) = v;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < TPW; i++) {
            const uint32_t t = (uint32_t)warp + (uint32_t)i * kWgWarps;
            if (t >= n_tiles)
                break;
            uint32_t mat, mt, nt;
            tile_info(t, n_in, H, mat, mt, nt);
            const uint32_t zoff = mat * kNeurons + mt * 16u; // dz column of this tile's first out row
            const uint32_t xoff = (mat == 0) ? nt * 8u : n_in + (mat - 1u) * kNeurons + nt * 8u;
#pragma unroll
            for (uint32_t kb = 0; kb < kWgRows / 16u; kb++) {
                uint32_t af[4], bf[4];
                // A = dz^T (m = out channel, k = row): ldmatrix.trans of the [row][out] tile
                const __half *pa = sz + (kb * 16u + (lane & 7) + ((lane >> 4) << 3)) * sz_ld + zoff + ((lane >> 3) & 1) * 8;
                ldsm_x4_trans(af, pa);
                // B = x (k = row, n = in channel): ldmatrix.trans of the [row][in] tile
                const __half *pb = sa + (kb * 16u + (lane & 15)) * sa_ld + xoff;
                ldsm_x4_trans(bf, pb);
                MlpPrec<BF16>::mma(acc[i], af, bf[0], bf[1]);
            }
        }
    }
    // one global accumulation per block
#pragma unroll
    for (int i = 0; i < TPW; i++) {
        const uint32_t t = (uint32_t)warp + (uint32_t)i * kWgWarps;
        if (t >= n_tiles)
            break;
        uint32_t mat, mt, nt;
        tile_info(t, n_in, H, mat, mt, nt);
        const uint32_t cols = (mat == 0) ? n_in : kNeurons;
        const uint32_t moff = (mat == 0) ? 0u : kNeurons * n_in + (mat - 1u) * kNeurons * kNeurons;
        const uint32_t row_a = mt * 16u + g, row_b = row_a + 8u, col = nt * 8u + tig * 2u;
        float *gw = a.grad + moff;
        if (mat == H && row_a >= kOutputs) {
        } else {
            atomicAdd(gw + row_a * cols + col, acc[i][0]);
            atomicAdd(gw + row_a * cols + col + 1, acc[i][1]);
        }
        if (!(mat == H && row_b >= kOutputs)) {
            atomicAdd(gw + row_b * cols + col, acc[i][2]);
            atomicAdd(gw + row_b * cols + col + 1, acc[i][3]);
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

} // namespace

cudaError_t launch_training_samples(const float4 *neural_nodes, const float4 *nodes, const float4 *tris,
                                    const float *albedo, const NeuralConsts &nc, const GridParams &grid,
                                    uint32_t training_step, uint32_t batch_size, uint32_t n, float *positions,
                                    float *targets, uint32_t *sample_nodes, uint32_t learned_lod,
                                    const NodeSurvival *survival, cudaStream_t s)
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
    if (survival && survival->enabled && survival->stats)
        a.survival = *survival;
    else
        a.survival = NodeSurvival{nullptr, nullptr, 1.0f, 0.0f, 0u};
    k_training_samples<<<(n + 127u) / 128u, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_train_forward_backward(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                                          const LossConsts &lc, const float *positions, const float *targets,
                                          uint32_t n, __half *acts, __half *dz, float *grad, float *loss_sum,
                                          float *sample_loss, bool bf16, bool fp8, int num_sms, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    TrainArgs a;
    a.grid = grid;
    a.lc = lc;
    const uint32_t n_network_params =
        kNeurons * grid.n_inputs + (n_hidden_layers - 1u) * kNeurons * kNeurons + kOutputsPadded * kNeurons;
    a.table = reinterpret_cast<const uint32_t *>(params_h + n_network_params);
    a.weights = params_h;
    a.positions = positions;
    a.targets = targets;
    a.acts = acts;
    a.dz = dz;
    a.grid_grad = reinterpret_cast<float2 *>(grad + n_network_params);
    a.loss_sum = loss_sum;
    a.sample_loss = sample_loss;
    a.fp8 = fp8 ? 1u : 0u;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    const size_t smem = kGridParamsSmem + smem_net_layout(grid.n_inputs, n_hidden_layers).total * sizeof(__half);
    {
        const uint64_t threads = (uint64_t)n * grid.n_points;
        k_train_encode<<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(
            grid, a.table, positions, n, acts, grid.n_inputs + n_hidden_layers * kNeurons, bf16 ? 1u : 0u);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    cudaError_t e = bf16  ? allow_max_dynamic_smem(k_train_fwd_bwd<true, false>)
                    : fp8 ? allow_max_dynamic_smem(k_train_fwd_bwd<false, true>)
                          : allow_max_dynamic_smem(k_train_fwd_bwd<false, false>);
    if (e != cudaSuccess)
        return e;
    const uint32_t tiles = (n + 15u) / 16u;
    uint32_t blocks = (tiles + kTrainWarps - 1u) / kTrainWarps;
    const uint32_t cap = (uint32_t)num_sms * 2u;
    if (blocks > cap)
        blocks = cap;
    if (bf16)
        k_train_fwd_bwd<true, false><<<blocks, kTrainThreads, smem, s>>>(a);
    else if (fp8)
        k_train_fwd_bwd<false, true><<<blocks, kTrainThreads, smem, s>>>(a);
    else
        k_train_fwd_bwd<false, false><<<blocks, kTrainThreads, smem, s>>>(a);
    return cudaGetLastError();
}

template <int TPW, bool BF16>
cudaError_t run_weight_grads(const WgArgs &a, uint32_t blocks, size_t smem, cudaStream_t s)
{
    cudaError_t e = allow_max_dynamic_smem(k_weight_grads<TPW, BF16>);
    if (e != cudaSuccess)
        return e;
    k_weight_grads<TPW, BF16><<<blocks, kWgThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_weight_gradients(const GridParams &grid, uint32_t n_hidden_layers, const __half *acts,
                                    const __half *dz, uint32_t n, float *grad, bool bf16, int num_sms, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    WgArgs a;
    a.acts = acts;
    a.dz = dz;
    a.grad = grad;
    a.n_inputs = grid.n_inputs;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    uint32_t blocks = (uint32_t)num_sms;
    uint32_t rows = (n + blocks - 1u) / blocks;
    rows = (rows + kWgRows - 1u) / kWgRows * kWgRows;
    blocks = (n + rows - 1u) / rows;
    a.rows_per_block = rows;
    const uint32_t acts_stride = grid.n_inputs + n_hidden_layers * kNeurons;
    const uint32_t dz_stride = n_hidden_layers * kNeurons + kOutputsPadded;
    const size_t smem = (size_t)kWgRows * ((acts_stride + 8u) + (dz_stride + 8u)) * sizeof(__half);
    const uint32_t n_tiles = 4u * (grid.n_inputs / 8u) + 32u * (n_hidden_layers - 1u) + 8u;
    const uint32_t tpw = (n_tiles + kWgWarps - 1u) / kWgWarps;
    if (tpw <= 16)
        return bf16 ? run_weight_grads<16, true>(a, blocks, smem, s) : run_weight_grads<16, false>(a, blocks, smem, s);
    if (tpw <= 24)
        return bf16 ? run_weight_grads<24, true>(a, blocks, smem, s) : run_weight_grads<24, false>(a, blocks, smem, s);
    if (tpw <= kMaxTilesPerWarp)
        return bf16 ? run_weight_grads<kMaxTilesPerWarp, true>(a, blocks, smem, s)
                    : run_weight_grads<kMaxTilesPerWarp, false>(a, blocks, smem, s);
    return cudaErrorInvalidValue;
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
