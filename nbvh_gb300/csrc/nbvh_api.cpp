// nbvh_api.cpp -- the C ABI of libnbvh (include/nbvh.h): handle lifetime, scene and BVH upload,
// parameter management, query dispatch, run-optimisation / run-inference loops and checkpoints.
//
// Host-side counterpart of the reference's NeuralBVHModule / NeuralPathModule / NeuralBVHRenderer
// surface (include/cuda/neural/neural_bvh_module.h:144-241, src/cuda/neural/path/path_module.cu,
// src/cuda/neural/neural_bvh_renderer.cu). State is per handle instead of __constant__ globals;
// errors are status codes instead of exceptions or exit().
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <exception>
#include <fstream>
#include <new>

#include "nbvh_internal.h"

using namespace nbvh;

namespace {

std::atomic<uint64_t> g_alloc_count{0};
std::atomic<int64_t> g_alloc_fail_after{-1}; // < 0: never fail

} // namespace

cudaError_t nbvh::device_alloc(void **ptr, size_t bytes)
{
    int64_t left = g_alloc_fail_after.load();
    while (left >= 0) { // injected failure: the next `left` allocations succeed, then every one fails
        if (left == 0)
            return cudaErrorMemoryAllocation;
        if (g_alloc_fail_after.compare_exchange_weak(left, left - 1))
            break;
    }
    const cudaError_t e = cudaMalloc(ptr, bytes);
    if (e == cudaSuccess)
        g_alloc_count.fetch_add(1);
    return e;
}

namespace {

// Restores the caller's current device when a call returns (the library makes the handle's device
// current for its work).
struct DeviceScope {
    int saved = -1;
    DeviceScope() { (void)cudaGetDevice(&saved); }
    ~DeviceScope()
    {
        if (saved >= 0)
            (void)cudaSetDevice(saved);
    }
};


template <typename F>
nbvh_status guarded(nbvh_handle *h, F &&f)
{
    if (!h)
        return NBVH_EINVAL;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope scope;
    try {
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        f();
        h->last_error.clear();
        return NBVH_OK;
    } catch (const Fail &e) {
        h->last_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        h->last_error = "host allocation failed";
        return NBVH_ENOMEM;
    } catch (const std::exception &e) {
        h->last_error = e.what();
        return NBVH_EINVAL;
    }
}

template <typename F>
nbvh_status guarded_free(F &&f)
{
    try {
        f();
        return NBVH_OK;
    } catch (const Fail &e) {
        return e.status;
    } catch (const std::bad_alloc &) {
        return NBVH_ENOMEM;
    } catch (...) {
        return NBVH_EINVAL;
    }
}

// -------- configuration --------

uint32_t n_inputs_of(const nbvh_config &c)
{
    return (uint32_t)c.module.input_segment_points * (uint32_t)c.hashgrid.n_levels *
           (uint32_t)c.hashgrid.n_features_per_level;
}

void validate_config(const nbvh_config &c)
{
    if (c.abi_version != NBVH_ABI_VERSION)
        fail(NBVH_EINVAL, "config abi_version mismatch");
    const int F = c.hashgrid.n_features_per_level;
    if (F != 2 && F != 4 && F != 8)
        fail(NBVH_EINVAL, "n_features_per_level must be 2, 4 or 8");
    if (c.hashgrid.n_levels < 1 || c.hashgrid.n_levels > (int)kMaxLevels)
        fail(NBVH_EINVAL, "n_levels must be in [1, 32]");
    if (c.hashgrid.log2_hashmap_size < 4 || c.hashgrid.log2_hashmap_size > 24)
        fail(NBVH_EINVAL, "log2_hashmap_size must be in [4, 24]");
    if (c.hashgrid.base_resolution < 2 || !(c.hashgrid.per_level_scale >= 1.0f))
        fail(NBVH_EINVAL, "bad grid resolution options");
    if (c.module.input_segment_points < 1 || c.module.input_segment_points > (int)kMaxPoints)
        fail(NBVH_EINVAL, "input_segment_points must be in [1, 16]");
    if (c.module.segment_distribution < 0 || c.module.segment_distribution > 2)
        fail(NBVH_EINVAL, "bad segment_distribution");
    const uint32_t ni = n_inputs_of(c);
    if (ni % 16u != 0u || ni > kMaxInputs)
        fail(NBVH_EINVAL, "points * levels * features_per_level must be a multiple of 16 and at most 128");
    if (c.network.n_neurons != (int)kNeurons)
        fail(NBVH_EINVAL, "n_neurons must be 64");
    if (c.network.n_hidden_layers < 1 || c.network.n_hidden_layers > (int)kMaxHiddenLayers)
        fail(NBVH_EINVAL, "n_hidden_layers must be in [1, 8]");
    if (c.network.precision != NBVH_PRECISION_FP16 && c.network.precision != NBVH_PRECISION_BF16 &&
        c.network.precision != NBVH_PRECISION_FP8)
        fail(NBVH_EINVAL, "network precision must be NBVH_PRECISION_FP16, _BF16 or _FP8");
    if (c.batch_size == 0 || (c.batch_size & (c.batch_size - 1u)) != 0)
        fail(NBVH_EINVAL, "batch_size must be a power of two");
    if (c.bvh.log2_bvh_max_traversals != 0)
        fail(NBVH_EINVAL, "log2_bvh_max_traversals must be 0");
    if (c.optimizer.loss_scale <= 0.f)
        fail(NBVH_EINVAL, "loss_scale must be positive");
}

// Grid geometry (tcnn's GridEncoding conventions): scale_l = exp2f(l * log2f(per_level_scale)) *
// base - 1 in single precision, here with the host C library's exp2f and log2f (a layout needs no
// GPU; a handle then takes its device's values, apply_device_level_scales); res = ceil(scale) + 1;
// entries = min(roundup8(res^3), 2^log2T).
void compute_layout(const nbvh_config &c, nbvh_param_layout &L, GridParams &g);

// tcnn evaluates grid_scale inside its encoding kernels, with CUDA's exp2f, which differs from the
// host C library's by an ulp for some arguments (5 of the 16 levels of the benchmark's grid). A
// handle encodes with its device's values, the ones tcnn would use; a level whose resolution the
// device value would change (a scale within an ulp of an integer) keeps the host value, so that the
// layout stays the one nbvh_param_layout_host reports.
void apply_device_level_scales(const nbvh_config &c, nbvh_param_layout &L, GridParams &g)
{
    const uint32_t n = L.n_levels;
    DeviceBuffer<float> d;
    cuda_check(d.resize(32u), "alloc level scales");
    const float log2_scale = std::log2(c.hashgrid.per_level_scale);
    cuda_check(launch_level_scales(log2_scale, (float)c.hashgrid.base_resolution, n, d.ptr, nullptr), "level scales");
    float s[32];
    cuda_check(cudaMemcpy(s, d.ptr, n * sizeof(float), cudaMemcpyDeviceToHost), "level scales");
    for (uint32_t l = 0; l < n; l++) {
        if ((uint32_t)std::ceil(s[l]) + 1u == g.res[l]) {
            g.scale[l] = s[l];
            L.level_scale[l] = s[l];
        }
    }
}

void compute_layout(const nbvh_config &c, nbvh_param_layout &L, GridParams &g)
{
    std::memset(&L, 0, sizeof(L));
    std::memset(&g, 0, sizeof(g));
    const uint32_t nl = (uint32_t)c.hashgrid.n_levels;
    const uint64_t hashmap = 1ull << c.hashgrid.log2_hashmap_size;
    uint64_t off = 0;
    const float log2_scale = std::log2(c.hashgrid.per_level_scale);
    for (uint32_t l = 0; l < nl; l++) {
        const float grow = std::exp2((float)l * log2_scale);
        const float s = grow * (float)c.hashgrid.base_resolution - 1.0f;
        uint32_t res = (uint32_t)std::ceil(s) + 1u;
        uint64_t dense = (uint64_t)res * res * res;
        uint64_t dense8 = (dense + 7u) & ~7ull;
        uint64_t sz = dense8 < hashmap ? dense8 : hashmap;
        L.level_offset[l] = (uint32_t)off;
        L.level_size[l] = (uint32_t)sz;
        L.level_resolution[l] = res;
        L.level_scale[l] = s;
        g.offset[l] = (uint32_t)off;
        g.size[l] = (uint32_t)sz;
        g.res[l] = res;
        g.scale[l] = s;
        g.hashed[l] = dense > sz ? 1u : 0u;
        off += sz;
    }
    L.n_levels = nl;
    L.n_inputs = n_inputs_of(c);
    const uint32_t H = (uint32_t)c.network.n_hidden_layers;
    L.n_network_params = kNeurons * L.n_inputs + (H - 1u) * kNeurons * kNeurons + kOutputsPadded * kNeurons;
    L.n_grid_entries = (uint32_t)off;
    const uint32_t F = (uint32_t)c.hashgrid.n_features_per_level;
    if ((uint64_t)L.n_network_params + (uint64_t)F * off >= (1ull << 31))
        fail(NBVH_EINVAL, "the parameter vector must stay below 2^31 values");
    L.n_params = L.n_network_params + F * L.n_grid_entries;
    L.n_features_per_level = F;
    g.n_features = F;
    g.n_levels = nl;
    g.n_points = (uint32_t)c.module.input_segment_points;
    g.n_inputs = L.n_inputs;
    g.segment_distribution = (uint32_t)c.module.segment_distribution;
}

// seeded initial parameters: Xavier-uniform matrices (rows 8..15 of the output matrix zero),
// hash-grid entries uniform in [-1e-4, 1e-4]
void init_params(const nbvh_config &c, const nbvh_param_layout &L, float *out)
{
    uint64_t state = 0x9E3779B97F4A7C15ull ^ ((uint64_t)c.seed * 0xD1B54A32D192ED03ull);
    auto next = [&]() -> double { // splitmix64 -> [0, 1)
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * 0x1p-53;
    };
    const uint32_t H = (uint32_t)c.network.n_hidden_layers;
    uint32_t o = 0;
    for (uint32_t m = 0; m <= H; m++) {
        const uint32_t rows = (m == H) ? kOutputsPadded : kNeurons;
        const uint32_t cols = (m == 0) ? L.n_inputs : kNeurons;
        const uint32_t fan_out = (m == H) ? kOutputs : kNeurons;
        const double s = std::sqrt(6.0 / (double)(cols + fan_out));
        for (uint32_t r = 0; r < rows; r++)
            for (uint32_t k = 0; k < cols; k++)
                out[o + r * cols + k] = (m == H && r >= kOutputs) ? 0.0f : (float)((2.0 * next() - 1.0) * s);
        o += rows * cols;
    }
    for (uint32_t i = 0; i < L.n_features_per_level * L.n_grid_entries; i++)
        out[L.n_network_params + i] = (float)((2.0 * next() - 1.0) * 1e-4);
}

NeuralConsts make_neural_consts(const nbvh_handle *h, uint32_t depth, bool visibility_only)
{
    const nbvh_config &c = h->cfg;
    NeuralConsts nc;
    std::memset(&nc, 0, sizeof(nc));
    nc.inference_mint_epsilon = c.bvh.inference_mint_epsilon;
    nc.inference_maxt_epsilon = c.bvh.inference_maxt_epsilon;
    nc.learning_mint_epsilon = c.bvh.learning_mint_epsilon;
    nc.learning_maxt_epsilon = c.bvh.learning_maxt_epsilon;
    nc.sampling_bbox_scaling = c.bvh.sampling_bbox_scaling;
    nc.fixed_node_dilation = c.bvh.fixed_node_dilation;
    nc.node_extent_dilation = c.bvh.node_extent_dilation;
    nc.leaf_boundary_sampling_ratio = c.bvh.leaf_boundary_sampling_ratio;
    nc.visibility_threshold =
        depth == 1u ? c.output.primary_visibility_threshold : c.output.secondary_visibility_threshold;
    nc.depth_epsilon = c.output.depth_epsilon;
    nc.fixed_depth_epsilon = c.output.fixed_depth_epsilon;
    nc.fallback_margin = c.fallback_margin;
    for (int k = 0; k < 3; k++) {
        nc.scene_min[k] = h->scene_min[k];
        nc.scene_max[k] = h->scene_max[k];
    }
    nc.bvh_lod = 0u; // rendered_lod
    nc.max_traversal_steps = c.max_traversal_steps;
    nc.visibility_only = visibility_only ? 1u : 0u;
    nc.fast_div_ok = h->neural_fast_div ? 1u : 0u;
    return nc;
}

LossConsts make_loss_consts(const nbvh_config &c, uint32_t n)
{
    LossConsts lc;
    lc.visibility_loss = c.output.visibility_loss;
    lc.depth_loss = c.output.depth_loss;
    lc.normal_loss = c.output.normal_loss;
    lc.albedo_loss = c.output.albedo_loss;
    lc.visibility_loss_scale = c.output.visibility_loss_scale;
    lc.depth_loss_scale = c.output.depth_loss_scale;
    lc.normal_loss_scale = c.output.normal_loss_scale;
    lc.albedo_loss_scale = c.output.albedo_loss_scale;
    lc.normal_linear = c.output.output_normal_linear_activation;
    lc.albedo_linear = c.output.output_albedo_linear_activation;
    lc.masking = c.output.visibility_masking_loss;
    lc.learn_normal = c.output.learn_normal;
    lc.learn_albedo = c.output.learn_albedo;
    lc.loss_scale = c.optimizer.loss_scale;
    const uint32_t dims = 2u + (c.output.learn_normal ? 3u : 0u) + (c.output.learn_albedo ? 3u : 0u);
    lc.inv_n_total = 1.0f / (float)((double)n * dims);
    return lc;
}

// Adam step size of step `step` (0-based): ExponentialDecay then the bias corrections.
float adam_step_size(const nbvh_config &c, uint32_t step)
{
    double lr = c.optimizer.learning_rate;
    if ((int64_t)step >= (int64_t)c.optimizer.decay_start && c.optimizer.decay_interval > 0)
        lr *= std::pow((double)c.optimizer.decay_base,
                       (double)(((int64_t)step - c.optimizer.decay_start) / c.optimizer.decay_interval));
    const double t = (double)step + 1.0;
    return (float)(lr * std::sqrt(1.0 - std::pow((double)c.optimizer.beta2, t)) /
                   (1.0 - std::pow((double)c.optimizer.beta1, t)));
}


void upload_bvh(nbvh_handle *h)
{
    h->model_version++;
    // nodes: two float4 per node in the reference layout
    h->classic_fast_div = nodes_in_fast_div_domain(h->nodes);
    cuda_check(h->d_nodes.resize(2u * h->nodes.size()), "alloc nodes");
    cuda_check(cudaMemcpy(h->d_nodes.ptr, h->nodes.data(), h->nodes.size() * sizeof(BVHNode), cudaMemcpyHostToDevice),
               "upload nodes");
    // pre-gathered triangle records in leaf order: {v0 | prim}, {e1 | 0}, {e2 | 0}
    const size_t nt = h->prim_indices.size();
    std::vector<float> rec(12u * nt);
    for (size_t j = 0; j < nt; j++) {
        const uint32_t p = h->prim_indices[j];
        const float *v0 = &h->vertices[3u * (size_t)h->indices[3u * p]];
        const float *v1 = &h->vertices[3u * (size_t)h->indices[3u * p + 1u]];
        const float *v2 = &h->vertices[3u * (size_t)h->indices[3u * p + 2u]];
        float *r = &rec[12u * j];
        r[0] = v0[0];
        r[1] = v0[1];
        r[2] = v0[2];
        std::memcpy(&r[3], &p, 4);
        r[4] = v1[0] - v0[0];
        r[5] = v1[1] - v0[1];
        r[6] = v1[2] - v0[2];
        r[7] = 0.f;
        r[8] = v2[0] - v0[0];
        r[9] = v2[1] - v0[1];
        r[10] = v2[2] - v0[2];
        r[11] = 0.f;
    }
    cuda_check(h->d_tris.resize(3u * nt), "alloc triangles");
    cuda_check(cudaMemcpy(h->d_tris.ptr, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice),
               "upload triangles");
    if (!h->albedo.empty()) {
        cuda_check(h->d_albedo.resize(h->albedo.size()), "alloc albedo");
        cuda_check(cudaMemcpy(h->d_albedo.ptr, h->albedo.data(), h->albedo.size() * sizeof(float), cudaMemcpyHostToDevice),
                   "upload albedo");
    } else {
        h->d_albedo.release();
    }
}

void upload_neural(nbvh_handle *h)
{
    end_tree_cut(h);
    cuda_check(h->d_neural_nodes.resize(2u * h->neural_nodes.size()), "alloc neural nodes");
    cuda_check(cudaMemcpy(h->d_neural_nodes.ptr, h->neural_nodes.data(), h->neural_nodes.size() * sizeof(BVHNode),
                          cudaMemcpyHostToDevice),
               "upload neural nodes");
    upload_inference_nodes(h);
}

} // namespace

void nbvh::upload_inference_nodes(nbvh_handle *h)
{
    h->model_version++;
    std::vector<BVHNode> dilated;
    std::vector<float> bounds;
    build_inference_nodes(h->neural_nodes, h->cfg.bvh.fixed_node_dilation, dilated, bounds);
    h->neural_fast_div = nodes_in_fast_div_domain(dilated) && coords_in_fast_div_domain(bounds.data(), bounds.size());
    cuda_check(h->d_neural_dilated.resize(2u * dilated.size()), "alloc dilated nodes");
    cuda_check(cudaMemcpy(h->d_neural_dilated.ptr, dilated.data(), dilated.size() * sizeof(BVHNode),
                          cudaMemcpyHostToDevice),
               "upload dilated nodes");
    cuda_check(h->d_neural_bounds.resize(bounds.size() / 4u), "alloc bounds");
    cuda_check(cudaMemcpy(h->d_neural_bounds.ptr, bounds.data(), bounds.size() * sizeof(float), cudaMemcpyHostToDevice),
               "upload bounds");
    h->non_neural.assign(h->neural_nodes.size(), 0u);
    h->any_non_neural = false;
    h->d_non_neural.release();
    // cuts above kMaxSortNodes nodes sort the query rays by runs of depth-first leaves
    if (h->neural_nodes.size() > kMaxSortNodes) {
        std::vector<uint32_t> keys;
        h->n_sort_bins = build_sort_keys(h->neural_nodes, kMaxSortNodes, keys);
        cuda_check(h->d_sort_key.resize(keys.size()), "alloc sort keys");
        cuda_check(cudaMemcpy(h->d_sort_key.ptr, keys.data(), keys.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                   "upload sort keys");
    } else {
        h->n_sort_bins = 0;
        h->d_sort_key.release();
    }
}

namespace {

// The MLP runs in BF16 (else FP16); its matrices are the first n_network_params parameters.
bool mlp_bf16(const nbvh_handle *h) { return h->cfg.network.precision == NBVH_PRECISION_BF16; }
uint32_t n_bf16_params(const nbvh_handle *h) { return mlp_bf16(h) ? h->layout.n_network_params : 0u; }
// nbvh_precision of the MLP
uint32_t mlp_prec(const nbvh_handle *h) { return (uint32_t)h->cfg.network.precision; }

void free_kernel_profile(nbvh_handle *h)
{
    if (!h->kprof)
        return;
    for (cudaEvent_t e : h->kprof->ev)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : h->kprof->train_ev)
        if (e)
            cudaEventDestroy(e);
    delete h->kprof;
    h->kprof = nullptr;
}
// FP32 master -> 16-bit copy: BF16 network in BF16 mode; in FP8 mode the hidden 64x64 matrices as
// FP8-E4M3 values (they follow the first matrix, 64 x n_inputs)
ParamPrecision param_precision(const nbvh_handle *h)
{
    ParamPrecision pp{n_bf16_params(h), 0u, 0u};
    if (h->cfg.network.precision == NBVH_PRECISION_FP8) {
        pp.fp8_lo = kNeurons * h->layout.n_inputs;
        pp.fp8_hi = pp.fp8_lo + ((uint32_t)h->cfg.network.n_hidden_layers - 1u) * kNeurons * kNeurons;
    }
    return pp;
}

void upload_params(nbvh_handle *h, const float *params, bool reset_adam)
{
    const uint32_t n = h->layout.n_params;
    cuda_check(h->d_params.resize(n), "alloc params");
    cuda_check(h->d_params_h.resize(n), "alloc fp16 params");
    cuda_check(cudaMemcpy(h->d_params.ptr, params, (size_t)n * sizeof(float), cudaMemcpyHostToDevice), "upload params");
    cuda_check(launch_params_to_half(h->d_params.ptr, h->d_params_h.ptr, n, param_precision(h), nullptr), "to half");
    if (reset_adam) {
        cuda_check(h->d_adam_m.resize(n), "alloc adam m");
        cuda_check(h->d_adam_v.resize(n), "alloc adam v");
        cuda_check(cudaMemset(h->d_adam_m.ptr, 0, (size_t)n * sizeof(float)), "zero m");
        cuda_check(cudaMemset(h->d_adam_v.ptr, 0, (size_t)n * sizeof(float)), "zero v");
        h->training_step = 0;
    }
    cuda_check(cudaDeviceSynchronize(), "sync");
}

void ensure_sample_state(nbvh_handle *h, uint32_t n)
{
    if (h->d_sample_state.count < sample_state_float4s(n))
        cuda_check(h->d_sample_state.resize(sample_state_float4s(n)), "alloc sampler state");
}

void ensure_train_workspace(nbvh_handle *h, uint32_t n)
{
    ensure_sample_state(h, n);
    const uint32_t P = h->grid.n_points, ni = h->layout.n_inputs, H = (uint32_t)h->cfg.network.n_hidden_layers;
    // zero-filled on allocation: a sample that node survival rejects keeps its slot's previous
    // content, which for the first step is this zero fill
    if (h->d_train_pos.count < (size_t)n * P * 3u) {
        cuda_check(h->d_train_pos.resize((size_t)n * P * 3u), "alloc train positions");
        cuda_check(cudaMemset(h->d_train_pos.ptr, 0, h->d_train_pos.count * sizeof(float)), "zero positions");
    }
    if (h->d_train_tgt.count < (size_t)n * 8u) {
        cuda_check(h->d_train_tgt.resize((size_t)n * 8u), "alloc train targets");
        cuda_check(cudaMemset(h->d_train_tgt.ptr, 0, h->d_train_tgt.count * sizeof(float)), "zero targets");
    }
    if (h->d_train_nodes.count < n) {
        cuda_check(h->d_train_nodes.resize(n), "alloc train nodes");
        cuda_check(cudaMemset(h->d_train_nodes.ptr, 0, h->d_train_nodes.count * sizeof(uint32_t)), "zero nodes");
    }
    if (h->d_train_loss.count < n) {
        cuda_check(h->d_train_loss.resize(n), "alloc sample losses");
        cuda_check(cudaMemset(h->d_train_loss.ptr, 0, h->d_train_loss.count * sizeof(float)), "zero losses");
    }
    if (h->d_train_feat.count < (size_t)n * ni)
        cuda_check(h->d_train_feat.resize((size_t)n * ni), "alloc features");
    if (h->d_train_dfeat.count < (size_t)n * ni)
        cuda_check(h->d_train_dfeat.resize((size_t)n * ni), "alloc feature gradients");
    if (h->d_train_wpacked.count < packed_weight_bytes(ni, H) / 2u)
        cuda_check(h->d_train_wpacked.resize(packed_weight_bytes(ni, H) / 2u), "alloc packed weights");
    if (h->d_status.count < 1u) {
        cuda_check(h->d_status.resize(1u), "alloc status");
        cuda_check(cudaMemset(h->d_status.ptr, 0, sizeof(uint32_t)), "reset status");
    }
    if (h->d_grad.count < h->layout.n_params)
        cuda_check(h->d_grad.resize(h->layout.n_params), "alloc grad");
}

void ensure_query_workspace(nbvh_handle *h, uint32_t n, int ctx)
{
    if (h->d_counters.count < 3u)
        cuda_check(h->d_counters.resize(3u), "alloc counters");
    grow_query_context(h, h->qctx[ctx], n);
}

// The neural query on the given stream with the given context's buffers (the handle's own
// contexts or a serving slot's): closest hit, or visibility when vis_only.
void neural_query(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, uint32_t depth, bool vis_only,
                  nbvh_neural_hit *d_hits, cudaStream_t s, int ctx, bool timed)
{
    require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
    require(h->neural_built, NBVH_ESTATE, "neural cut not built");
    if (n == 0) { // nothing to launch; the statistics of this call are all zero
        if (h->d_counters.count < 3u)
            cuda_check(h->d_counters.resize(3u), "alloc counters");
        cuda_check(cudaMemsetAsync(h->d_counters.ptr + ctx, 0, sizeof(QueryCounters), s), "reset counters");
        if (timed) {
            cuda_check(cudaEventRecord(h->ev0, s), "event");
            cuda_check(cudaEventRecord(h->ev1, s), "event");
            h->n_stat_chunks = 0;
            h->stat_ctx_mask = 1u << ctx;
        }
        h->last_launches = 0;
        h->last_rays = 0;
        return;
    }
    ensure_query_workspace(h, n, ctx);
    if (timed)
        cuda_check(cudaEventRecord(h->ev0, s), "event");
    h->last_launches = run_neural_query(h, h->qctx[ctx], h->d_counters.ptr + ctx, d_rays, n, depth, vis_only, d_hits, s);
    if (timed) { // a device-buffer call: its statistics are this context's counters
        cuda_check(cudaEventRecord(h->ev1, s), "event");
        h->n_stat_chunks = 0;
        h->stat_ctx_mask = 1u << ctx;
    }
    h->last_rays = n;
}

// Host-buffer calls run chunk after chunk on contexts 1-2; before a context's counters are reset
// by its next chunk, they are copied (on the chunk's stream) into slot `chunk` of d_stat_chunks.
void reserve_stat_chunks(nbvh_handle *h, uint32_t n, uint32_t chunk)
{
    const uint32_t chunks = n == 0 ? 0u : (uint32_t)(((uint64_t)n + chunk - 1u) / chunk);
    if (h->d_stat_chunks.count < chunks)
        cuda_check(h->d_stat_chunks.resize(chunks), "alloc statistics");
    h->n_stat_chunks = 0;
}

void snapshot_stats(nbvh_handle *h, uint32_t chunk, int ctx, cudaStream_t s)
{
    cuda_check(cudaMemcpyAsync(h->d_stat_chunks.ptr + chunk, h->d_counters.ptr + ctx, sizeof(QueryCounters),
                               cudaMemcpyDeviceToDevice, s),
               "statistics");
    h->n_stat_chunks = chunk + 1u;
}

// The closest-hit neural query on the fixed per-device scratch (noalloc_scratch): the same
// kernels as neural_query, with no allocation. Returns after the stream's work is complete, so
// the shared scratch is free again when the call returns.
void neural_query_noalloc(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, uint32_t depth,
                          nbvh_neural_hit *d_hits, cudaStream_t s)
{
    if (n > NBVH_NOALLOC_MAX_RAYS)
        fail(NBVH_EINVAL, "n = " + std::to_string(n) + " exceeds NBVH_NOALLOC_MAX_RAYS = " +
                              std::to_string(NBVH_NOALLOC_MAX_RAYS) + "; split the batch");
    require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
    require(h->neural_built, NBVH_ESTATE, "neural cut not built");
    NoallocScratch sc;
    cuda_check(noalloc_scratch(h->device, &sc), "fixed scratch address");
    if (n == 0)
        return;
    cuda_check(cudaMemsetAsync(sc.counters, 0, sizeof(QueryCounters), s), "reset counters");
    if (h->cfg.bvh.ignore_neural_blas) {
        cuda_check(launch_classic_as_neural(h->d_nodes.ptr, h->d_tris.ptr, d_rays, n, d_hits, false,
                                            h->classic_fast_div, s),
                   "classic");
    } else {
        const NeuralConsts nc = make_neural_consts(h, depth, false);
        uint32_t host_words[4] = {0, 0, 0, 0}, launches = 0;
        StepResources res;
        res.features = sc.features;
        res.outputs = sc.outputs;
        res.wpacked = sc.wpacked;
        res.perm = sc.perm;
        res.node_bins = sc.node_bins;
        res.node_cursor = sc.node_cursor;
        res.h_words = host_words;
        res.ev = nullptr;
        res.wait_ns = h->wait_limit_ns;
        res.stall = h->debug_stall;
        res.sort_key = h->n_sort_bins ? h->d_sort_key.ptr : nullptr;
        res.n_sort_bins = h->n_sort_bins;
        cuda_check(make_feature_map(sc.features, h->layout.n_inputs, (uint32_t)kNoallocRays, &res.feature_map),
                   "feature map");
        cuda_check(launch_wave_query(h->d_neural_dilated.ptr, h->d_neural_bounds.ptr,
                                     (uint32_t)h->neural_nodes.size(), h->any_non_neural ? h->d_non_neural.ptr : nullptr,
                                     h->d_params_h.ptr, h->grid, nc, (uint32_t)h->cfg.network.n_hidden_layers, d_rays,
                                     n, d_hits, sc.counters, sc.fallback_list, sc.lists, sc.wave_counts, res,
                                     mlp_prec(h), h->num_sms, s, &launches),
                   "neural query");
        if (h->any_non_neural || h->cfg.fallback_margin > 0.f)
            cuda_check(launch_classic_fallback(h->d_nodes.ptr, h->d_tris.ptr, d_rays, sc.fallback_list, sc.counters,
                                               n, d_hits, false, h->classic_fast_div, h->num_sms, s),
                       "fallback");
    }
    cuda_check(cudaStreamSynchronize(s), "stream sync");
}

} // namespace

// =============================================================================================
// C ABI
// =============================================================================================

extern "C" {

uint32_t nbvh_abi_version(void) { return NBVH_ABI_VERSION; }

const char *nbvh_status_string(nbvh_status s)
{
    switch (s) {
    case NBVH_OK: return "ok";
    case NBVH_EINVAL: return "invalid argument";
    case NBVH_ENOMEM: return "out of memory";
    case NBVH_EDEVICE: return "CUDA device error";
    case NBVH_ETIMEOUT: return "device loop step cap reached";
    case NBVH_EOVERFLOW: return "traversal stack overflow";
    case NBVH_ESTATE: return "call order violated";
    case NBVH_EIO: return "checkpoint i/o error";
    }
    return "unknown status";
}

const char *nbvh_last_error(const nbvh_handle *h) { return h ? h->last_error.c_str() : "null handle"; }

nbvh_status nbvh_config_default(nbvh_config *c)
{
    if (!c)
        return NBVH_EINVAL;
    std::memset(c, 0, sizeof(*c));
    c->abi_version = NBVH_ABI_VERSION;
    c->hashgrid.n_levels = 16;
    c->hashgrid.n_features_per_level = 2;
    c->hashgrid.log2_hashmap_size = 19;
    c->hashgrid.base_resolution = 16;
    c->hashgrid.per_level_scale = (float)std::pow(2048.0 / 16.0, 1.0 / 15.0);
    c->network.n_neurons = 64;
    c->network.n_hidden_layers = 4;
    c->network.precision = NBVH_PRECISION_FP16;
    c->optimizer.learning_rate = 1e-2f;
    c->optimizer.beta1 = 0.9f;
    c->optimizer.beta2 = 0.999f;
    c->optimizer.epsilon = 1e-8f;
    c->optimizer.l2_reg = 1e-8f;
    c->optimizer.decay_start = 10000;
    c->optimizer.decay_interval = 2000;
    c->optimizer.decay_base = 0.33f;
    c->optimizer.loss_scale = 128.0f;
    c->bvh.inference_mint_epsilon = 1e-4f;
    c->bvh.inference_maxt_epsilon = 1e-3f;
    c->bvh.learning_mint_epsilon = 1e-3f;
    c->bvh.learning_maxt_epsilon = 1e-3f;
    c->bvh.sampling_bbox_scaling = 1.5f;
    c->bvh.fixed_node_dilation = 1e-5f;
    c->bvh.node_extent_dilation = 1e-4f;
    c->bvh.leaf_boundary_sampling_ratio = 0.0f;
    c->bvh.ignore_neural_blas = 0;
    c->bvh.max_training_bounces = 1;
    c->bvh.sample_cosine_weighted = 1;
    c->bvh.backface_bounce_training = 0;
    c->bvh.log2_bvh_max_traversals = 0;
    c->output.visibility_loss = NBVH_LOSS_BCE;
    c->output.visibility_loss_scale = 1.f;
    c->output.depth_loss = NBVH_LOSS_L1;
    c->output.depth_loss_scale = 1.f;
    c->output.normal_loss = NBVH_LOSS_L1;
    c->output.normal_loss_scale = 1.f;
    c->output.albedo_loss = NBVH_LOSS_RELATIVE_L2;
    c->output.albedo_loss_scale = 1.f;
    c->output.output_normal_linear_activation = 1;
    c->output.output_albedo_linear_activation = 0;
    c->output.visibility_masking_loss = 1;
    c->output.primary_visibility_threshold = 0.5f;
    c->output.secondary_visibility_threshold = 0.5f;
    c->output.depth_epsilon = 0.2f;
    c->output.fixed_depth_epsilon = 1e-5f;
    c->output.learn_normal = 1;
    c->output.learn_albedo = 1;
    c->module.input_segment_points = 4;
    c->module.segment_distribution = NBVH_SEGMENT_EQUIDISTANT_INTERIOR;
    c->batch_size = 1u << 18;
    c->neural_bvh_max_depth = 10;
    c->max_traversal_steps = 1000;
    c->seed = 1337;
    c->fallback_margin = 0.0f;
    return NBVH_OK;
}

nbvh_status nbvh_create(const nbvh_config *cfg, int device, nbvh_handle **out)
{
    if (!cfg || !out)
        return NBVH_EINVAL;
    *out = nullptr;
    nbvh_handle *h = nullptr;
    try {
        h = new nbvh_handle();
    } catch (...) {
        return NBVH_ENOMEM;
    }
    h->device = device;
    nbvh_status st = guarded_free([&]() {
        validate_config(*cfg);
        h->cfg = *cfg;
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
            fail(NBVH_EDEVICE, "no CUDA device");
        if (device < 0 || device >= count)
            fail(NBVH_EINVAL, "bad device index");
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        cuda_check(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        cuda_check(cudaEventCreate(&h->ev0), "event");
        cuda_check(cudaEventCreate(&h->ev1), "event");
        for (int k = 0; k < 2; k++)
            cuda_check(cudaStreamCreateWithFlags(&h->pipe_stream[k], cudaStreamNonBlocking), "stream");
        cuda_check(h->d_counters.resize(3u), "alloc counters");
        cuda_check(cudaMemset(h->d_counters.ptr, 0, 3u * sizeof(QueryCounters)), "zero counters");
        cuda_check(h->d_loss_sum.resize(1u), "alloc loss");
        compute_layout(h->cfg, h->layout, h->grid);
        apply_device_level_scales(h->cfg, h->layout, h->grid);
        std::vector<float> p(h->layout.n_params);
        init_params(h->cfg, h->layout, p.data());
        upload_params(h, p.data(), true);
    });
    if (st != NBVH_OK) {
        delete h;
        return st;
    }
    *out = h;
    return NBVH_OK;
}

nbvh_status nbvh_destroy(nbvh_handle *h)
{
    if (!h)
        return NBVH_EINVAL;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    for (int k = 0; k < 2; k++) {
        if (h->pipe_stream[k])
            cudaStreamDestroy(h->pipe_stream[k]);
    }
    free_kernel_profile(h);
    if (h->ev0)
        cudaEventDestroy(h->ev0);
    if (h->ev1)
        cudaEventDestroy(h->ev1);
    for (int k = 0; k < 2; k++)
        if (h->ev_drain[k])
            cudaEventDestroy(h->ev_drain[k]);
    delete h;
    return NBVH_OK;
}

nbvh_status nbvh_set_mesh(nbvh_handle *h, const float *v, uint32_t nv, const uint32_t *idx, uint32_t nt,
                          const float *albedo)
{
    return guarded(h, [&]() {
        require(v && idx && nv > 0 && nt > 0, NBVH_EINVAL, "empty mesh");
        for (size_t i = 0; i < 3u * (size_t)nt; i++)
            require(idx[i] < nv, NBVH_EINVAL, "triangle index out of range");
        h->vertices.assign(v, v + 3u * (size_t)nv);
        h->indices.assign(idx, idx + 3u * (size_t)nt);
        if (albedo)
            h->albedo.assign(albedo, albedo + 3u * (size_t)nt);
        else
            h->albedo.clear();
        h->classic_built = false;
        h->neural_built = false;
        end_tree_cut(h);
    });
}

nbvh_status nbvh_build_classic(nbvh_handle *h)
{
    return guarded(h, [&]() {
        require(!h->indices.empty(), NBVH_ESTATE, "no mesh");
        std::string err;
        if (!build_bvh2(h->vertices, h->indices, h->nodes, h->prim_indices, err))
            fail(NBVH_EINVAL, err);
        end_tree_cut(h);
        upload_bvh(h);
        for (int k = 0; k < 3; k++) {
            h->scene_min[k] = h->nodes[0].min[k];
            h->scene_max[k] = h->nodes[0].max[k];
        }
        h->classic_built = true;
        h->neural_built = false;
        cuda_check(cudaDeviceSynchronize(), "sync");
    });
}

nbvh_status nbvh_get_classic_bvh(const nbvh_handle *hc, uint32_t *h_nodes, uint32_t *n_nodes, uint32_t *h_prims,
                                 uint32_t *n_prims)
{
    nbvh_handle *h = const_cast<nbvh_handle *>(hc);
    return guarded(h, [&]() {
        require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
        if (n_nodes)
            *n_nodes = (uint32_t)h->nodes.size();
        if (n_prims)
            *n_prims = (uint32_t)h->prim_indices.size();
        if (h_nodes)
            std::memcpy(h_nodes, h->nodes.data(), h->nodes.size() * sizeof(BVHNode));
        if (h_prims)
            std::memcpy(h_prims, h->prim_indices.data(), h->prim_indices.size() * sizeof(uint32_t));
    });
}

nbvh_status nbvh_import_neural_cut(nbvh_handle *h, const char *path)
{
    return guarded(h, [&]() {
        require(path != nullptr, NBVH_EINVAL, "null path");
        require(h->classic_built, NBVH_ESTATE, "classic BVH not built (it gives the neural scene box)");
        std::vector<BVHNode> nodes;
        std::string err;
        if (!read_nbvh(path, nodes, err))
            fail(NBVH_EIO, err);
        h->neural_nodes = std::move(nodes);
        upload_neural(h);
        h->neural_built = true;
        cuda_check(cudaDeviceSynchronize(), "sync");
    });
}

nbvh_status nbvh_export_neural_cut(nbvh_handle *h, const char *path)
{
    return guarded(h, [&]() {
        require(path != nullptr, NBVH_EINVAL, "null path");
        require(h->neural_built, NBVH_ESTATE, "neural cut not built");
        std::string err;
        if (!write_nbvh(path, h->neural_nodes, err))
            fail(NBVH_EIO, err);
    });
}

nbvh_status nbvh_begin_tree_cut(nbvh_handle *h, const nbvh_tree_cut_options *o, uint32_t start_depth)
{
    return guarded(h, [&]() {
        require(o != nullptr, NBVH_EINVAL, "null options");
        begin_tree_cut(h, *o, start_depth);
    });
}

nbvh_status nbvh_get_tree_cut_info(nbvh_handle *h, nbvh_tree_cut_info *info)
{
    return guarded(h, [&]() {
        require(info != nullptr, NBVH_EINVAL, "null info");
        std::memset(info, 0, sizeof(*info));
        const TreeCutSession &c = h->cut;
        if (!c.active)
            return;
        uint32_t words[kCutWords + kNumBvhLods];
        tree_cut_words(h, words, h->pipe_stream[0]);
        const uint32_t it = h->training_step - c.start_step;
        info->active = 1u;
        info->learning = c.learning ? 1u : 0u;
        info->n_nodes = words[kCutCount];
        info->capacity = c.capacity;
        info->iteration = it;
        info->current_learned_lod = c.current_lod;
        info->total_splits = words[kCutSplits];
        info->max_depth = words[kCutMaxDepth];
        info->expected_nodes = c.expected_nodes;
        const uint32_t max_bits = (it == 0 || c.zero_next_max) ? 0u : words[kCutMax0 + ((it - 1u) & 1u)];
        std::memcpy(&info->max_node_loss, &max_bits, 4);
        for (uint32_t l = 0; l < kNumBvhLods; l++)
            info->n_lod_nodes[l] = words[kCutWords + l];
    });
}

nbvh_status nbvh_get_tree_cut(nbvh_handle *h, uint32_t *h_nodes, uint32_t *h_stats, uint32_t *h_node_map,
                              uint32_t *n_nodes)
{
    return guarded(h, [&]() {
        require(n_nodes != nullptr, NBVH_EINVAL, "null count");
        require(h->cut.active, NBVH_ESTATE, "no tree-cut session");
        uint32_t words[kCutWords + kNumBvhLods];
        tree_cut_words(h, words, h->pipe_stream[0]);
        const uint32_t n = words[kCutCount];
        if (h_nodes || h_stats || h_node_map)
            require(*n_nodes >= n, NBVH_EINVAL, "buffers smaller than the cut");
        if (h_nodes)
            cuda_check(cudaMemcpy(h_nodes, h->d_neural_nodes.ptr, (size_t)n * sizeof(BVHNode), cudaMemcpyDeviceToHost),
                       "download nodes");
        if (h_stats)
            cuda_check(cudaMemcpy(h_stats, h->cut.d_stats.ptr, (size_t)n * 16u, cudaMemcpyDeviceToHost),
                       "download stats");
        if (h_node_map)
            cuda_check(cudaMemcpy(h_node_map, h->cut.d_map.ptr, (size_t)n * 4u, cudaMemcpyDeviceToHost),
                       "download node map");
        *n_nodes = n;
    });
}

nbvh_status nbvh_set_tree_cut_stats(nbvh_handle *h, const uint32_t *h_stats, uint32_t n_nodes)
{
    return guarded(h, [&]() {
        require(h_stats != nullptr, NBVH_EINVAL, "null stats");
        require(h->cut.active, NBVH_ESTATE, "no tree-cut session");
        uint32_t words[kCutWords + kNumBvhLods];
        tree_cut_words(h, words, h->pipe_stream[0]);
        require(n_nodes == words[kCutCount], NBVH_EINVAL, "stats count differs from the cut's node count");
        cuda_check(cudaMemcpy(h->cut.d_stats.ptr, h_stats, (size_t)n_nodes * 16u, cudaMemcpyHostToDevice),
                   "upload stats");
    });
}

nbvh_status nbvh_get_training_batch(nbvh_handle *h, float *h_positions, float *h_targets, uint32_t *h_nodes,
                                    float *h_sample_loss, uint32_t n)
{
    return guarded(h, [&]() {
        require(n <= h->d_train_nodes.count && n <= h->d_train_loss.count, NBVH_ESTATE,
                "no training batch of that size");
        const size_t P = h->grid.n_points;
        cuda_check(cudaDeviceSynchronize(), "sync");
        if (h_positions)
            cuda_check(cudaMemcpy(h_positions, h->d_train_pos.ptr, (size_t)n * P * 3u * sizeof(float),
                                  cudaMemcpyDeviceToHost),
                       "download positions");
        if (h_targets)
            cuda_check(cudaMemcpy(h_targets, h->d_train_tgt.ptr, (size_t)n * 8u * sizeof(float), cudaMemcpyDeviceToHost),
                       "download targets");
        if (h_nodes)
            cuda_check(cudaMemcpy(h_nodes, h->d_train_nodes.ptr, (size_t)n * 4u, cudaMemcpyDeviceToHost),
                       "download nodes");
        if (h_sample_loss)
            cuda_check(cudaMemcpy(h_sample_loss, h->d_train_loss.ptr, (size_t)n * 4u, cudaMemcpyDeviceToHost),
                       "download losses");
    });
}

nbvh_status nbvh_build_neural_cut(nbvh_handle *h, uint32_t max_depth)
{
    return guarded(h, [&]() {
        require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
        build_neural_cut(h->nodes, max_depth, h->neural_nodes);
        upload_neural(h);
        h->neural_built = true;
        cuda_check(cudaDeviceSynchronize(), "sync");
    });
}

nbvh_status nbvh_get_neural_bvh(const nbvh_handle *hc, uint32_t *h_nodes, uint32_t *n_nodes, float *bbox)
{
    nbvh_handle *h = const_cast<nbvh_handle *>(hc);
    return guarded(h, [&]() {
        require(h->neural_built, NBVH_ESTATE, "neural cut not built");
        if (n_nodes)
            *n_nodes = (uint32_t)h->neural_nodes.size();
        if (h_nodes)
            std::memcpy(h_nodes, h->neural_nodes.data(), h->neural_nodes.size() * sizeof(BVHNode));
        if (bbox) {
            for (int k = 0; k < 3; k++) {
                bbox[k] = h->scene_min[k];
                bbox[3 + k] = h->scene_max[k];
            }
        }
    });
}

nbvh_status nbvh_set_non_neural_leaves(nbvh_handle *h, const uint32_t *ids, uint32_t n, int flag)
{
    return guarded(h, [&]() {
        require(h->neural_built, NBVH_ESTATE, "neural cut not built");
        require(ids || n == 0, NBVH_EINVAL, "null ids");
        for (uint32_t i = 0; i < n; i++) {
            require(ids[i] < h->neural_nodes.size(), NBVH_EINVAL, "node id out of range");
            h->non_neural[ids[i]] = flag ? 1u : 0u;
        }
        h->any_non_neural = false;
        for (uint8_t f : h->non_neural)
            h->any_non_neural |= f != 0u;
        cuda_check(h->d_non_neural.resize(h->non_neural.size()), "alloc flags");
        cuda_check(cudaMemcpy(h->d_non_neural.ptr, h->non_neural.data(), h->non_neural.size(), cudaMemcpyHostToDevice),
                   "upload flags");
    });
}

nbvh_status nbvh_set_ignore_neural_blas(nbvh_handle *h, int ignore)
{
    return guarded(h, [&]() { h->cfg.bvh.ignore_neural_blas = ignore ? 1 : 0; });
}

} // extern "C"

namespace {

// The classic queries of kRaySortMin rays or more take the rays bin by bin (when ray ordering is
// on): the order buffers, grown to n, or nullptr for batch order.
const uint32_t *classic_order(nbvh_handle *h, uint32_t n)
{
    if (!h->ray_ordering || n < kRaySortMin)
        return nullptr;
    if (h->d_classic_order.count < n) {
        cuda_check(h->d_classic_order.resize(n), "alloc ray order");
        cuda_check(h->d_classic_keys.resize(n), "alloc ray bins");
    }
    if (h->d_classic_bins.count < kRayBins)
        cuda_check(h->d_classic_bins.resize(kRayBins), "alloc ray bin counts");
    return h->d_classic_order.ptr;
}

} // namespace

extern "C" {

nbvh_status nbvh_set_ray_ordering(nbvh_handle *h, int enable)
{
    return guarded(h, [&]() { h->ray_ordering = enable != 0; });
}

nbvh_status nbvh_query_closest_classic(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, nbvh_hit *d_hits,
                                       nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
        require((d_rays && d_hits) || n == 0, NBVH_EINVAL, "null buffers");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        const uint32_t *order = classic_order(h, n);
        cuda_check(cudaEventRecord(h->ev0, s), "event");
        if (order)
            cuda_check(launch_ray_order(d_rays, n, h->scene_min, h->scene_max, h->d_classic_keys.ptr,
                                        h->d_classic_bins.ptr, h->d_classic_order.ptr, h->num_sms, s),
                       "ray order");
        cuda_check(launch_classic(h->d_nodes.ptr, h->d_tris.ptr, d_rays, n, d_hits, false, order, h->classic_fast_div, s),
                   "classic");
        cuda_check(cudaEventRecord(h->ev1, s), "event");
        h->last_launches = order ? 4u : 1u;
        h->last_rays = n;
    });
}

nbvh_status nbvh_query_any_classic(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, nbvh_hit *d_hits,
                                   nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
        require((d_rays && d_hits) || n == 0, NBVH_EINVAL, "null buffers");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        const uint32_t *order = classic_order(h, n);
        cuda_check(cudaEventRecord(h->ev0, s), "event");
        if (order)
            cuda_check(launch_ray_order(d_rays, n, h->scene_min, h->scene_max, h->d_classic_keys.ptr,
                                        h->d_classic_bins.ptr, h->d_classic_order.ptr, h->num_sms, s),
                       "ray order");
        cuda_check(launch_classic(h->d_nodes.ptr, h->d_tris.ptr, d_rays, n, d_hits, true, order, h->classic_fast_div, s),
                   "classic");
        cuda_check(cudaEventRecord(h->ev1, s), "event");
        h->last_launches = 1;
        h->last_rays = n;
    });
}

nbvh_status nbvh_query_closest_neural(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, uint32_t depth,
                                      nbvh_neural_hit *d_hits, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require((d_rays && d_hits) || n == 0, NBVH_EINVAL, "null buffers");
        neural_query(h, d_rays, n, depth, false, d_hits, reinterpret_cast<cudaStream_t>(stream), 0, true);
    });
}

nbvh_status nbvh_query_visibility_neural(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, uint32_t depth,
                                         nbvh_neural_hit *d_hits, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require((d_rays && d_hits) || n == 0, NBVH_EINVAL, "null buffers");
        neural_query(h, d_rays, n, depth, true, d_hits, reinterpret_cast<cudaStream_t>(stream), 0, true);
    });
}

nbvh_status nbvh_query_closest_neural_noalloc(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, uint32_t depth,
                                              nbvh_neural_hit *d_hits, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require((d_rays && d_hits) || n == 0, NBVH_EINVAL, "null buffers");
        neural_query_noalloc(h, d_rays, n, depth, d_hits, reinterpret_cast<cudaStream_t>(stream));
    });
}

} // extern "C"

namespace {

// Host-buffer queries: chunks alternate between two streams; each chunk is copied in, queried and
// copied out on its stream, so the copies of one chunk overlap the kernel of the other.
template <typename Rec, typename Q>
void pipelined(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n, Rec *h_out, Q &&query)
{
    const uint32_t chunk = 1u << 20;
    const size_t in_bytes = (size_t)chunk * sizeof(nbvh_ray), out_bytes = (size_t)chunk * sizeof(Rec);
    for (int k = 0; k < 2; k++) {
        if (h->d_pipe_in[k].count < in_bytes)
            cuda_check(h->d_pipe_in[k].resize(in_bytes), "alloc pipeline in");
        if (h->d_pipe_out[k].count < out_bytes)
            cuda_check(h->d_pipe_out[k].resize(out_bytes), "alloc pipeline out");
    }
    uint32_t launches = 0;
    reserve_stat_chunks(h, n, chunk);
    for (uint32_t c0 = 0, ci = 0; c0 < n; c0 += chunk, ci++) {
        const int k = (int)(ci & 1u);
        const uint32_t cnt = (n - c0) < chunk ? (n - c0) : chunk;
        cudaStream_t s = h->pipe_stream[k];
        auto *din = reinterpret_cast<nbvh_ray *>(h->d_pipe_in[k].ptr);
        auto *dout = reinterpret_cast<Rec *>(h->d_pipe_out[k].ptr);
        cuda_check(cudaMemcpyAsync(din, h_rays + c0, (size_t)cnt * sizeof(nbvh_ray), cudaMemcpyHostToDevice, s), "H2D");
        query(din, cnt, dout, s, 1 + k);
        snapshot_stats(h, ci, 1 + k, s);
        launches += h->last_launches;
        cuda_check(cudaMemcpyAsync(h_out + c0, dout, (size_t)cnt * sizeof(Rec), cudaMemcpyDeviceToHost, s), "D2H");
    }
    for (int k = 0; k < 2; k++)
        cuda_check(cudaStreamSynchronize(h->pipe_stream[k]), "sync pipeline");
    h->last_launches = launches;
    h->last_rays = n;
}

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister), NULL for any
// other memory and for buffers that are not 16-byte aligned (the kernels move rays and records
// with 16-byte loads and stores).
const void *mapped_host(const void *p)
{
    if (reinterpret_cast<uintptr_t>(p) % 16u != 0u)
        return nullptr;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (attr.type != cudaMemoryTypeHost || reinterpret_cast<uintptr_t>(attr.devicePointer) % 16u != 0u)
        return nullptr;
    return attr.devicePointer;
}

// Host-buffer queries on page-locked buffers: the kernels read the rays and write the records
// over the host link themselves (NVLink-C2C on Grace), so the transfers overlap the traversal and
// the network instead of preceding and following them. One query per 2^23 rays bounds the
// device workspace.
template <typename Rec, typename Q>
bool zero_copy(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n, Rec *h_out, Q &&query)
{
    const auto *drays = static_cast<const nbvh_ray *>(mapped_host(h_rays));
    auto *dout = static_cast<Rec *>(const_cast<void *>(mapped_host(h_out)));
    if (!drays || !dout)
        return false;
    const uint32_t chunk = 1u << 23;
    uint32_t launches = 0;
    cudaStream_t s = h->pipe_stream[0];
    reserve_stat_chunks(h, n, chunk);
    for (uint32_t c0 = 0, ci = 0; c0 < n; c0 += chunk, ci++) {
        const uint32_t cnt = (n - c0) < chunk ? (n - c0) : chunk;
        query(drays + c0, cnt, dout + c0, s, 1);
        snapshot_stats(h, ci, 1, s);
        launches += h->last_launches;
    }
    cuda_check(cudaStreamSynchronize(s), "sync");
    h->last_launches = launches;
    h->last_rays = n;
    return true;
}

// Neural host query on page-locked buffers: the first pass reads the rays over the host link; the
// records are written to device memory and copied to the host in one transfer right after the
// first network step (most rays are finished by then), overlapping the remaining steps; the rays
// that finish later are listed by the decode kernel and their records copied at the end.
bool zero_copy_neural(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n, uint32_t depth, nbvh_neural_hit *h_hits)
{
    const auto *drays = static_cast<const nbvh_ray *>(mapped_host(h_rays));
    auto *dhost = static_cast<nbvh_neural_hit *>(const_cast<void *>(mapped_host(h_hits)));
    if (!drays || !dhost)
        return false;
    if (h->cfg.bvh.ignore_neural_blas || h->any_non_neural || h->cfg.fallback_margin > 0.f)
        return zero_copy(h, h_rays, n, h_hits, [&](const nbvh_ray *din, uint32_t cnt, nbvh_neural_hit *dout,
                                                    cudaStream_t s, int ctx) {
            neural_query(h, din, cnt, depth, false, dout, s, ctx, false);
        });
    require(h->classic_built && h->neural_built, NBVH_ESTATE, "scene not built");
    for (int k = 0; k < 2; k++)
        if (!h->ev_drain[k])
            cuda_check(cudaEventCreateWithFlags(&h->ev_drain[k], cudaEventDisableTiming), "event");
    const uint32_t chunk = 1u << 23;
    cudaStream_t s = h->pipe_stream[0];
    uint32_t launches = 0;
    reserve_stat_chunks(h, n, chunk);
    for (uint32_t c0 = 0, ci = 0; c0 < n; c0 += chunk, ci++) {
        const uint32_t cnt = (n - c0) < chunk ? (n - c0) : chunk;
        ensure_query_workspace(h, cnt, 1);
        if (h->d_drain_hits.count < cnt)
            cuda_check(h->d_drain_hits.resize(cnt), "alloc records");
        if (h->d_late.count < (size_t)cnt + 1u)
            cuda_check(h->d_late.resize((size_t)cnt + 1u), "alloc late list");
        bool taken = false;
        StepResources t;
        t.drain_host = dhost + c0;
        t.drain_stream = h->pipe_stream[1];
        t.drain_snap = h->ev_drain[0];
        t.drain_done = h->ev_drain[1];
        t.drain_step = 0;
        t.late_count = h->d_late.ptr;
        t.late_list = h->d_late.ptr + 1;
        t.drain_taken = &taken;
        t.ray_order_ok = false; // the first pass reads the rays over the host link: once, in order
        launches += run_neural_query(h, h->qctx[1], h->d_counters.ptr + 1, drays + c0, cnt, depth, false,
                                     h->d_drain_hits.ptr, s, &t);
        snapshot_stats(h, ci, 1, s);
        if (taken) {
            cuda_check(cudaStreamWaitEvent(s, h->ev_drain[1], 0), "wait early copy");
            cuda_check(launch_copy_late(t.late_list, t.late_count, cnt, h->d_drain_hits.ptr, dhost + c0, h->num_sms, s),
                       "late records");
            launches++;
        } else {
            cuda_check(cudaMemcpyAsync(h_hits + c0, h->d_drain_hits.ptr, (size_t)cnt * sizeof(nbvh_neural_hit),
                                       cudaMemcpyDeviceToHost, s),
                       "D2H");
        }
        cuda_check(cudaStreamSynchronize(s), "sync");
    }
    h->last_launches = launches;
    h->last_rays = n;
    return true;
}

} // namespace

extern "C" {

nbvh_status nbvh_query_closest_neural_host(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n, uint32_t depth,
                                           nbvh_neural_hit *h_hits)
{
    return guarded(h, [&]() {
        require((h_rays && h_hits) || n == 0, NBVH_EINVAL, "null buffers");
        if (n == 0 || !zero_copy_neural(h, h_rays, n, depth, h_hits))
            pipelined(h, h_rays, n, h_hits, [&](const nbvh_ray *din, uint32_t cnt, nbvh_neural_hit *dout,
                                                cudaStream_t s, int ctx) {
                neural_query(h, din, cnt, depth, false, dout, s, ctx, false);
            });
    });
}

nbvh_status nbvh_query_closest_classic_host(nbvh_handle *h, const nbvh_ray *h_rays, uint32_t n, nbvh_hit *h_hits)
{
    return guarded(h, [&]() {
        require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
        require((h_rays && h_hits) || n == 0, NBVH_EINVAL, "null buffers");
        auto q = [&](const nbvh_ray *din, uint32_t cnt, nbvh_hit *dout, cudaStream_t s, int) {
            cuda_check(launch_classic(h->d_nodes.ptr, h->d_tris.ptr, din, cnt, dout, false, nullptr,
                                      h->classic_fast_div, s),
                       "classic");
            h->last_launches = 1;
        };
        if (n == 0 || !zero_copy(h, h_rays, n, h_hits, q))
            pipelined(h, h_rays, n, h_hits, q);
    });
}

nbvh_status nbvh_query_segments(nbvh_handle *h, const nbvh_ray *d_rays, uint32_t n, uint32_t max_segments,
                                nbvh_segment *d_segments, uint32_t *d_counts, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(h->neural_built, NBVH_ESTATE, "neural cut not built");
        require((d_rays && d_counts && (d_segments || max_segments == 0)) || n == 0, NBVH_EINVAL, "null buffers");
        const NeuralConsts nc = make_neural_consts(h, 1u, false);
        cuda_check(launch_segments(h->d_neural_dilated.ptr, h->d_neural_bounds.ptr, nc, d_rays, n, max_segments,
                                   d_segments, d_counts,
                                   reinterpret_cast<cudaStream_t>(stream)),
                   "segments");
        h->last_launches = 1;
    });
}

nbvh_status nbvh_get_param_layout(const nbvh_handle *hc, nbvh_param_layout *out)
{
    nbvh_handle *h = const_cast<nbvh_handle *>(hc);
    return guarded(h, [&]() {
        require(out != nullptr, NBVH_EINVAL, "null output");
        *out = h->layout;
    });
}

nbvh_status nbvh_get_params(nbvh_handle *h, float *h_params)
{
    return guarded(h, [&]() {
        require(h_params != nullptr, NBVH_EINVAL, "null output");
        cuda_check(cudaDeviceSynchronize(), "sync");
        cuda_check(cudaMemcpy(h_params, h->d_params.ptr, (size_t)h->layout.n_params * sizeof(float),
                              cudaMemcpyDeviceToHost),
                   "download params");
    });
}

nbvh_status nbvh_set_params(nbvh_handle *h, const float *h_params)
{
    return guarded(h, [&]() {
        require(h_params != nullptr, NBVH_EINVAL, "null input");
        upload_params(h, h_params, true);
    });
}

nbvh_status nbvh_import_tcnn_weights(nbvh_handle *h, const char *path)
{
    return guarded(h, [&]() {
        require(path != nullptr, NBVH_EINVAL, "null path");
        std::vector<float> p;
        std::string err;
        if (!read_tcnn_params(path, p, err))
            fail(NBVH_EIO, "tcnn weights " + std::string(path) + ": " + err);
        if (p.size() != h->layout.n_params)
            fail(NBVH_EINVAL, "tcnn weights hold " + std::to_string(p.size()) + " parameters, the configuration " +
                                  std::to_string(h->layout.n_params));
        upload_params(h, p.data(), true);
    });
}

nbvh_status nbvh_export_tcnn_weights(nbvh_handle *h, const char *path)
{
    return guarded(h, [&]() {
        require(path != nullptr, NBVH_EINVAL, "null path");
        std::vector<float> p(h->layout.n_params);
        cuda_check(cudaDeviceSynchronize(), "sync");
        cuda_check(cudaMemcpy(p.data(), h->d_params.ptr, p.size() * sizeof(float), cudaMemcpyDeviceToHost),
                   "download params");
        std::string err;
        if (!write_tcnn_params(path, p.data(), p.size(), err))
            fail(NBVH_EIO, "tcnn weights " + std::string(path) + ": " + err);
    });
}

nbvh_status nbvh_network_inference(nbvh_handle *h, const float *d_positions, uint32_t n, float *d_outputs,
                                   nbvh_stream stream)
{
    return guarded(h, [&]() {
        require((d_positions && d_outputs) || n == 0, NBVH_EINVAL, "null buffers");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        const uint32_t ni = h->layout.n_inputs, H = (uint32_t)h->cfg.network.n_hidden_layers;
        h->last_launches = 0;
        if (n == 0)
            return;
        // the encoder writes FP16 feature rows, the tcgen05 MLP reads them by TMA
        if (h->d_infer_feat.count < (size_t)n * ni)
            cuda_check(h->d_infer_feat.resize((size_t)n * ni), "alloc feature rows");
        const uint32_t wb = packed_weight_bytes(ni, H);
        if (h->d_wpacked.count < wb / 2u)
            cuda_check(h->d_wpacked.resize(wb / 2u), "alloc packed weights");
        if (h->d_status.count < 1u)
            cuda_check(h->d_status.resize(1u), "alloc status");
        TensorMapBytes map;
        cuda_check(make_feature_map(h->d_infer_feat.ptr, ni, n, &map), "feature map");
        cuda_check(cudaMemsetAsync(h->d_status.ptr, 0, sizeof(uint32_t), s), "reset status");
        cuda_check(cudaEventRecord(h->ev0, s), "event");
        cuda_check(launch_encode_rows(h->d_params_h.ptr, h->grid, H, d_positions, n, h->d_infer_feat.ptr, mlp_bf16(h), s),
                   "encode");
        cuda_check(launch_pack_weights(h->d_params_h.ptr, ni, H, h->d_wpacked.ptr, s), "pack weights");
        cuda_check(launch_mlp_tc(map, h->d_wpacked.ptr, ni, H, n, nullptr, d_outputs, h->d_status.ptr, mlp_prec(h),
                                 h->num_sms, s, true, h->wait_limit_ns, h->debug_stall),
                   "tensor-core MLP");
        cuda_check(cudaEventRecord(h->ev1, s), "event");
        h->last_launches = 3;
        uint32_t status = 0;
        cuda_check(cudaMemcpyAsync(&status, h->d_status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "status");
        cuda_check(cudaStreamSynchronize(s), "sync");
        require((status & 2u) == 0u, NBVH_EDEVICE, "tensor-core MLP: shared memory not 1,024-byte aligned");
        require(status == 0u, NBVH_ETIMEOUT, "tensor-core MLP: a bounded wait gave up");
    });
}

nbvh_status nbvh_mlp_inference(nbvh_handle *h, const uint16_t *d_features, uint32_t n, float *d_outputs,
                               nbvh_stream stream)
{
    return guarded(h, [&]() {
        require((d_features && d_outputs) || n == 0, NBVH_EINVAL, "null buffers");
        require((reinterpret_cast<uintptr_t>(d_features) & 15u) == 0u, NBVH_EINVAL,
                "d_features must be 16-byte aligned");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        const uint32_t ni = h->layout.n_inputs, H = (uint32_t)h->cfg.network.n_hidden_layers;
        const uint32_t wb = packed_weight_bytes(ni, H);
        if (h->d_wpacked.count < wb / 2u)
            cuda_check(h->d_wpacked.resize(wb / 2u), "alloc packed weights");
        if (h->d_status.count < 1u)
            cuda_check(h->d_status.resize(1u), "alloc status");
        cuda_check(cudaMemsetAsync(h->d_status.ptr, 0, sizeof(uint32_t), s), "reset status");
        cuda_check(launch_pack_weights(h->d_params_h.ptr, ni, H, h->d_wpacked.ptr, s), "pack weights");
        if (n == 0)
            return;
        TensorMapBytes map;
        cuda_check(make_feature_map(reinterpret_cast<const __half *>(d_features), ni, n, &map), "feature map");
        cuda_check(cudaEventRecord(h->ev0, s), "event");
        cuda_check(launch_mlp_tc(map, h->d_wpacked.ptr, ni, H, n, nullptr, d_outputs, h->d_status.ptr, mlp_prec(h),
                                 h->num_sms, s, true, h->wait_limit_ns, h->debug_stall),
                   "tensor-core MLP");
        cuda_check(cudaEventRecord(h->ev1, s), "event");
        h->last_launches = 2;
        uint32_t status = 0;
        cuda_check(cudaMemcpyAsync(&status, h->d_status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "status");
        cuda_check(cudaStreamSynchronize(s), "sync");
        require((status & 2u) == 0u, NBVH_EDEVICE, "tensor-core MLP: shared memory not 1,024-byte aligned");
        require(status == 0u, NBVH_ETIMEOUT, "tensor-core MLP: a bounded wait gave up");
    });
}

nbvh_status nbvh_encode(nbvh_handle *h, const float *d_positions, uint32_t n, float *d_features, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require((d_positions && d_features) || n == 0, NBVH_EINVAL, "null buffers");
        cuda_check(launch_encode(h->d_params_h.ptr, h->grid, (uint32_t)h->cfg.network.n_hidden_layers, d_positions, n,
                                 d_features, reinterpret_cast<cudaStream_t>(stream)),
                   "encode");
        h->last_launches = 1;
    });
}

} // extern "C"

namespace {

// forward + loss + backward of one batch into h->d_grad (scaled by the loss scale) and loss_sum
void gradients_into_workspace(nbvh_handle *h, const float *d_pos, const float *d_tgt, uint32_t n, cudaStream_t s,
                              float *loss_slot, const cudaEvent_t *marks = nullptr)
{
    ensure_train_workspace(h, n);
    const uint32_t H = (uint32_t)h->cfg.network.n_hidden_layers;
    cuda_check(cudaMemsetAsync(h->d_grad.ptr, 0, (size_t)h->layout.n_params * sizeof(float), s), "zero grad");
    cuda_check(launch_train_step(h->d_params_h.ptr, h->grid, H, make_loss_consts(h->cfg, n), d_pos, d_tgt, n,
                                 h->d_train_feat.ptr, h->d_train_dfeat.ptr, h->d_train_wpacked.ptr, h->d_grad.ptr,
                                 loss_slot, h->d_train_loss.ptr, h->d_status.ptr, mlp_bf16(h),
                                 h->cfg.network.precision == NBVH_PRECISION_FP8, h->num_sms, s, h->wait_limit_ns,
                                 h->debug_stall, marks),
               "forward/backward");
}

} // namespace

extern "C" {

nbvh_status nbvh_compute_gradients(nbvh_handle *h, const float *d_positions, const float *d_targets, uint32_t n,
                                   float *d_gradients, float *h_loss, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(d_positions && d_targets && d_gradients && n > 0, NBVH_EINVAL, "null buffers");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        ensure_train_workspace(h, n);
        cuda_check(cudaMemsetAsync(h->d_loss_sum.ptr, 0, sizeof(float), s), "zero loss");
        cuda_check(cudaMemsetAsync(h->d_status.ptr, 0, sizeof(uint32_t), s), "reset status");
        gradients_into_workspace(h, d_positions, d_targets, n, s, h->d_loss_sum.ptr);
        cuda_check(cudaMemcpyAsync(d_gradients, h->d_grad.ptr, (size_t)h->layout.n_params * sizeof(float),
                                   cudaMemcpyDeviceToDevice, s),
                   "copy grad");
        cuda_check(launch_scale(d_gradients, h->layout.n_params, 1.0f / h->cfg.optimizer.loss_scale, s), "unscale");
        float loss = 0.f;
        uint32_t status = 0;
        cuda_check(cudaMemcpyAsync(&loss, h->d_loss_sum.ptr, sizeof(float), cudaMemcpyDeviceToHost, s), "loss");
        cuda_check(cudaMemcpyAsync(&status, h->d_status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "status");
        cuda_check(cudaStreamSynchronize(s), "sync");
        require(status == 0u, NBVH_ETIMEOUT, "tensor-core training kernel: a bounded wait gave up");
        if (h_loss)
            *h_loss = loss;
        h->last_launches = 4;
    });
}

nbvh_status nbvh_adam_step(nbvh_handle *h, const float *d_gradients, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(d_gradients != nullptr, NBVH_EINVAL, "null gradient");
        const nbvh_config &c = h->cfg;
        cuda_check(launch_adam(h->d_params.ptr, h->d_params_h.ptr, h->d_adam_m.ptr, h->d_adam_v.ptr, d_gradients,
                               h->layout.n_params, adam_step_size(c, h->training_step), c.optimizer.beta1,
                               c.optimizer.beta2, c.optimizer.epsilon, c.optimizer.l2_reg, 1.0f, param_precision(h),
                               reinterpret_cast<cudaStream_t>(stream)),
                   "adam");
        h->training_step++;
        h->last_launches = 1;
    });
}

nbvh_status nbvh_generate_training_batch(nbvh_handle *h, uint32_t training_step, uint32_t n, float *d_positions,
                                         float *d_targets, uint32_t *d_nodes, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(h->neural_built, NBVH_ESTATE, "neural cut not built");
        require((d_positions && d_targets) || n == 0, NBVH_EINVAL, "null buffers");
        const NeuralConsts nc = make_neural_consts(h, 1u, false);
        ensure_sample_state(h, n);
        cuda_check(launch_training_samples(h->d_neural_nodes.ptr, h->d_nodes.ptr, h->d_tris.ptr,
                                           h->albedo.empty() ? nullptr : h->d_albedo.ptr, nc, h->grid, training_step,
                                           h->cfg.batch_size, n, d_positions, d_targets, d_nodes, kNumBvhLods - 1u,
                                           nullptr, h->d_sample_state.ptr, h->classic_fast_div, h->num_sms,
                                           reinterpret_cast<cudaStream_t>(stream)),
                   "training samples");
        h->last_launches = 2;
    });
}

nbvh_status nbvh_run_optimisation(nbvh_handle *h, uint32_t steps, nbvh_train_stats *stats)
{
    return guarded(h, [&]() {
        require(h->neural_built, NBVH_ESTATE, "neural cut not built");
        const nbvh_config &c = h->cfg;
        const uint32_t n = c.batch_size;
        ensure_train_workspace(h, n);
        if (h->d_loss_sum.count < (size_t)steps + 1u)
            cuda_check(h->d_loss_sum.resize((size_t)steps + 1u), "alloc loss");
        cudaStream_t s = h->pipe_stream[0];
        cuda_check(cudaMemsetAsync(h->d_loss_sum.ptr, 0, ((size_t)steps + 1u) * sizeof(float), s), "zero loss");
        cuda_check(cudaMemsetAsync(h->d_status.ptr, 0, sizeof(uint32_t), s), "reset status");
        const NeuralConsts nc = make_neural_consts(h, 1u, false);
        const uint32_t first = h->training_step;
        float lr_t = 0.f;
        cuda_check(cudaEventRecord(h->ev0, s), "event");
        for (uint32_t i = 0; i < steps; i++) {
            NodeSurvival survival{nullptr, nullptr, 1.0f, 0.0f, 0u};
            uint32_t learned_lod = kNumBvhLods - 1u; // build_and_upload_neural_bvh starts at the coarsest LoD
            if (h->cut.active)
                tree_cut_before_step(h, survival, learned_lod);
            // with kernel profiling on, the last step records its phases
            const bool prof = h->kprof && i + 1u == steps;
            if (prof)
                cuda_check(cudaEventRecord(h->kprof->train_ev[0], s), "event");
            cuda_check(launch_training_samples(h->d_neural_nodes.ptr, h->d_nodes.ptr, h->d_tris.ptr,
                                               h->albedo.empty() ? nullptr : h->d_albedo.ptr, nc, h->grid,
                                               h->training_step, n, n, h->d_train_pos.ptr, h->d_train_tgt.ptr,
                                               h->d_train_nodes.ptr, learned_lod, &survival, h->d_sample_state.ptr,
                                               h->classic_fast_div, h->num_sms, s),
                       "training samples");
            gradients_into_workspace(h, h->d_train_pos.ptr, h->d_train_tgt.ptr, n, s, h->d_loss_sum.ptr + i,
                                     prof ? h->kprof->train_ev + 1 : nullptr);
            lr_t = adam_step_size(c, h->training_step);
            cuda_check(launch_adam(h->d_params.ptr, h->d_params_h.ptr, h->d_adam_m.ptr, h->d_adam_v.ptr, h->d_grad.ptr,
                                   h->layout.n_params, lr_t, c.optimizer.beta1, c.optimizer.beta2, c.optimizer.epsilon,
                                   c.optimizer.l2_reg, 1.0f / c.optimizer.loss_scale, param_precision(h), s),
                       "adam");
            if (prof) {
                cuda_check(cudaEventRecord(h->kprof->train_ev[5], s), "event");
                h->kprof->train_rows = n;
            }
            if (h->cut.active)
                tree_cut_after_step(h, h->d_train_loss.ptr, n, s);
            h->training_step++;
        }
        cuda_check(cudaEventRecord(h->ev1, s), "event");
        if (h->cut.active)
            tree_cut_sync(h, s);
        std::vector<float> losses(steps > 0 ? steps : 1u);
        if (steps > 0)
            cuda_check(cudaMemcpyAsync(losses.data(), h->d_loss_sum.ptr, steps * sizeof(float), cudaMemcpyDeviceToHost, s),
                       "losses");
        uint32_t status = 0;
        cuda_check(cudaMemcpyAsync(&status, h->d_status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "status");
        cuda_check(cudaStreamSynchronize(s), "sync");
        require(status == 0u, NBVH_ETIMEOUT, "tensor-core training kernel: a bounded wait gave up");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, h->ev0, h->ev1), "elapsed");
        h->last_kernel_ms = ms;
        h->last_launches = 7u * steps;
        if (stats) {
            double sum = 0.0;
            for (uint32_t i = 0; i < steps; i++)
                sum += losses[i];
            stats->steps_done = steps;
            stats->training_step = h->training_step;
            stats->last_loss = steps ? losses[steps - 1u] : 0.f;
            stats->mean_loss = steps ? (float)(sum / steps) : 0.f;
            stats->learning_rate = lr_t;
            stats->ms_per_step = steps ? ms / (float)steps : 0.f;
        }
        (void)first;
    });
}

uint32_t nbvh_training_step(const nbvh_handle *h) { return h ? h->training_step : 0u; }

} // extern "C"

namespace nbvh {

void camera_params(const nbvh_render_request *r, float du[3], float dv[3], float tl[3])
{
    // CudaBackend::update_camera, src/cuda/cuda_backend.cpp:595-611 (FP32, glm's order)
    auto sub = [](const float *a, const float *b, float *o) {
        for (int k = 0; k < 3; k++)
            o[k] = a[k] - b[k];
    };
    auto dot = [](const float *a, const float *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; };
    auto cross = [](const float *a, const float *b, float *o) {
        o[0] = a[1] * b[2] - b[1] * a[2];
        o[1] = a[2] * b[0] - b[2] * a[0];
        o[2] = a[0] * b[1] - b[0] * a[1];
    };
    auto normalize = [&](float *v) {
        float s = 1.0f / std::sqrt(dot(v, v));
        for (int k = 0; k < 3; k++)
            v[k] = v[k] * s;
    };
    const float ipy = 2.0f * std::tan((0.5f * r->yfov_degrees) * 0.0174532925199432958f);
    const float aspect = (float)r->width / (float)r->height;
    const float ipx = ipy * aspect;
    float dir[3], up[3] = {r->up[0], r->up[1], r->up[2]};
    sub(r->target, r->origin, dir);
    normalize(dir);
    normalize(up);
    float t[3];
    cross(dir, up, t);
    normalize(t);
    for (int k = 0; k < 3; k++)
        du[k] = t[k] * ipx;
    cross(du, dir, t);
    normalize(t);
    for (int k = 0; k < 3; k++)
        dv[k] = t[k] * -ipy;
    for (int k = 0; k < 3; k++)
        tl[k] = (dir[k] - du[k] * 0.5f) - dv[k] * 0.5f;
}

} // namespace nbvh

extern "C" {

nbvh_status nbvh_camera_rays(nbvh_handle *h, const nbvh_render_request *req, nbvh_ray *d_rays, nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(req && d_rays && req->width > 0 && req->height > 0, NBVH_EINVAL, "bad request");
        float du[3], dv[3], tl[3];
        camera_params(req, du, dv, tl);
        cuda_check(launch_camera_rays(req->width, req->height, req->sample_idx, req->sample_offset, req->origin, du, dv, tl,
                                      d_rays, reinterpret_cast<cudaStream_t>(stream)),
                   "camera rays");
    });
}

nbvh_status nbvh_run_inference(nbvh_handle *h, const nbvh_render_request *req, nbvh_neural_hit *d_image,
                               nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(req && d_image && req->width > 0 && req->height > 0, NBVH_EINVAL, "bad request");
        const uint32_t n = req->width * req->height;
        if (h->d_pipe_in[0].count < (size_t)n * sizeof(nbvh_ray))
            cuda_check(h->d_pipe_in[0].resize((size_t)n * sizeof(nbvh_ray)), "alloc camera rays");
        auto *rays = reinterpret_cast<nbvh_ray *>(h->d_pipe_in[0].ptr);
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        float du[3], dv[3], tl[3];
        camera_params(req, du, dv, tl);
        cuda_check(launch_camera_rays(req->width, req->height, req->sample_idx, req->sample_offset, req->origin, du, dv, tl,
                                      rays, s),
                   "camera rays");
        neural_query(h, rays, n, 1u, false, d_image, s, 0, true);
        cuda_check(cudaStreamSynchronize(s), "sync");
    });
}

nbvh_status nbvh_render_path(nbvh_handle *h, const nbvh_path_request *req, float *d_image, uint64_t *rays_traced,
                             nbvh_stream stream)
{
    return guarded(h, [&]() {
        require(h->classic_built && h->neural_built, NBVH_ESTATE, "scene not built");
        if (h->d_counters.count < 3u)
            cuda_check(h->d_counters.resize(3u), "alloc counters");
        require(req != nullptr, NBVH_EINVAL, "null request");
        const uint64_t traced = render_path_core(h, h->qctx[0], h->d_counters.ptr, h->path, req, d_image,
                                                 reinterpret_cast<cudaStream_t>(stream),
                                                 req->camera.sample_idx * req->spp);
        h->n_stat_chunks = 0;
        h->stat_ctx_mask = 1u;
        if (rays_traced)
            *rays_traced = traced;
    });
}

nbvh_status nbvh_last_query_stats(nbvh_handle *h, nbvh_query_stats *out)
{
    return guarded(h, [&]() {
        require(out != nullptr, NBVH_EINVAL, "null output");
        cuda_check(cudaDeviceSynchronize(), "sync");
        std::vector<QueryCounters> c;
        if (h->n_stat_chunks) {
            c.resize(h->n_stat_chunks);
            cuda_check(cudaMemcpy(c.data(), h->d_stat_chunks.ptr, c.size() * sizeof(QueryCounters),
                                  cudaMemcpyDeviceToHost),
                       "statistics");
        } else {
            QueryCounters all[3];
            cuda_check(cudaMemcpy(all, h->d_counters.ptr, sizeof(all), cudaMemcpyDeviceToHost), "counters");
            for (int k = 0; k < 3; k++)
                if (h->stat_ctx_mask >> k & 1u)
                    c.push_back(all[k]);
        }
        std::memset(out, 0, sizeof(*out));
        out->rays = h->last_rays;
        for (size_t k = 0; k < c.size(); k++) {
            out->segments += c[k].segments;
            out->step_capped += c[k].step_capped;
            out->stack_overflow += c[k].stack_overflow;
            out->fallback += c[k].fallback;
        }
    });
}

nbvh_status nbvh_set_kernel_profile(nbvh_handle *h, int enable)
{
    return guarded(h, [&]() {
        if (enable && !h->kprof) {
            auto *p = new KernelProfile();
            h->kprof = p; // freed with its events by free_kernel_profile, also on failure here
            for (uint32_t k = 0; k < 2u * kMaxProfiledLaunches; k++)
                cuda_check(cudaEventCreate(&p->ev[k]), "event");
            for (uint32_t k = 0; k < 6u; k++)
                cuda_check(cudaEventCreate(&p->train_ev[k]), "event");
        } else if (!enable && h->kprof) {
            cuda_check(cudaDeviceSynchronize(), "sync");
            free_kernel_profile(h);
        }
    });
}

nbvh_status nbvh_last_kernel_profile(nbvh_handle *h, nbvh_kernel_profile *out)
{
    return guarded(h, [&]() {
        require(out != nullptr, NBVH_EINVAL, "null output");
        require(h->kprof != nullptr, NBVH_ESTATE, "kernel profiling is off (nbvh_set_kernel_profile)");
        std::memset(out, 0, sizeof(*out));
        const KernelProfile &p = *h->kprof;
        // the query's last kernels (decode, tail, fallback) follow its last encoder launch
        cuda_check(cudaDeviceSynchronize(), "sync");
        for (uint32_t k = 0; k + 1u < p.used; k += 2u) {
            float t = 0.f;
            cuda_check(cudaEventElapsedTime(&t, p.ev[k], p.ev[k + 1u]), "elapsed");
            out->encode_ms += t;
            out->encode_launches++;
        }
        if (h->d_counters.ptr) {
            QueryCounters c;
            cuda_check(cudaMemcpy(&c, h->d_counters.ptr, sizeof(c), cudaMemcpyDeviceToHost), "counters");
            out->encoded_segments = c.encoded;
            out->segments = c.segments;
        }
        if (p.train_rows) {
            float t[5];
            for (int k = 0; k < 5; k++)
                cuda_check(cudaEventElapsedTime(&t[k], p.train_ev[k], p.train_ev[k + 1]), "elapsed");
            out->train_sample_ms = t[0];
            out->train_encode_ms = t[1];
            out->train_mlp_ms = t[2];
            out->train_scatter_ms = t[3];
            out->train_adam_ms = t[4];
            out->train_rows = p.train_rows;
        }
    });
}

nbvh_status nbvh_debug_set_wait_limit(nbvh_handle *h, uint64_t ns)
{
    return guarded(h, [&]() { h->wait_limit_ns = ns; });
}

nbvh_status nbvh_debug_inject_stall(nbvh_handle *h, int enable)
{
    return guarded(h, [&]() { h->debug_stall = enable != 0; });
}

nbvh_status nbvh_debug_fail_allocations(int64_t after)
{
    g_alloc_fail_after.store(after < 0 ? -1 : after);
    return NBVH_OK;
}

nbvh_status nbvh_debug_alloc_count(uint64_t *out)
{
    if (!out)
        return NBVH_EINVAL;
    *out = g_alloc_count.load();
    return NBVH_OK;
}

nbvh_status nbvh_debug_device_level_scales(const nbvh_config *cfg, int device, float *out)
{
    if (!cfg || !out || cfg->hashgrid.n_levels <= 0 || cfg->hashgrid.n_levels > 32 ||
        !(cfg->hashgrid.per_level_scale > 0.0f))
        return NBVH_EINVAL;
    DeviceScope scope;
    if (cudaSetDevice(device) != cudaSuccess)
        return NBVH_EDEVICE;
    const uint32_t n = (uint32_t)cfg->hashgrid.n_levels;
    float *d = nullptr;
    if (cudaMalloc(&d, 32u * sizeof(float)) != cudaSuccess)
        return NBVH_ENOMEM;
    // log2 of the level scale on the host in single precision, as tcnn's GridEncoding does
    const float log2_scale = std::log2(cfg->hashgrid.per_level_scale);
    cudaError_t e = launch_level_scales(log2_scale, (float)cfg->hashgrid.base_resolution, n, d, nullptr);
    if (e == cudaSuccess)
        e = cudaMemcpy(out, d, n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? NBVH_OK : NBVH_EDEVICE;
}

nbvh_status nbvh_last_kernel_time(nbvh_handle *h, float *ms, uint32_t *launches)
{
    return guarded(h, [&]() {
        cuda_check(cudaEventSynchronize(h->ev1), "event sync");
        float t = 0.f;
        cuda_check(cudaEventElapsedTime(&t, h->ev0, h->ev1), "elapsed");
        if (ms)
            *ms = t;
        if (launches)
            *launches = h->last_launches;
    });
}

} // extern "C"

// ---------------------------------------------------------------------------------------------
// Checkpoints: own binary format "NBVHCKP1"
// ---------------------------------------------------------------------------------------------

namespace {

constexpr char kMagic[8] = {'N', 'B', 'V', 'H', 'C', 'K', 'P', '1'};

template <typename T>
void wr_vec(std::ofstream &f, const std::vector<T> &v)
{
    uint64_t n = v.size();
    f.write(reinterpret_cast<const char *>(&n), 8);
    if (n)
        f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(n * sizeof(T)));
}

template <typename T>
void rd_vec(std::ifstream &f, std::vector<T> &v, uint64_t max_elems)
{
    uint64_t n = 0;
    f.read(reinterpret_cast<char *>(&n), 8);
    if (!f || n > max_elems)
        fail(NBVH_EIO, "malformed checkpoint");
    v.resize(n);
    if (n)
        f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(T)));
    if (!f)
        fail(NBVH_EIO, "truncated checkpoint");
}

} // namespace

extern "C" {

nbvh_status nbvh_save(nbvh_handle *h, const char *path)
{
    return guarded(h, [&]() {
        require(path != nullptr, NBVH_EINVAL, "null path");
        std::ofstream f(path, std::ios::binary);
        if (!f)
            fail(NBVH_EIO, "cannot open checkpoint for writing");
        cuda_check(cudaDeviceSynchronize(), "sync");
        const uint32_t np = h->layout.n_params;
        std::vector<float> p(np), m(np), v(np);
        cuda_check(cudaMemcpy(p.data(), h->d_params.ptr, np * sizeof(float), cudaMemcpyDeviceToHost), "params");
        cuda_check(cudaMemcpy(m.data(), h->d_adam_m.ptr, np * sizeof(float), cudaMemcpyDeviceToHost), "adam m");
        cuda_check(cudaMemcpy(v.data(), h->d_adam_v.ptr, np * sizeof(float), cudaMemcpyDeviceToHost), "adam v");
        f.write(kMagic, 8);
        f.write(reinterpret_cast<const char *>(&h->cfg), sizeof(nbvh_config));
        f.write(reinterpret_cast<const char *>(&h->training_step), 4);
        uint32_t flags = (h->classic_built ? 1u : 0u) | (h->neural_built ? 2u : 0u);
        f.write(reinterpret_cast<const char *>(&flags), 4);
        wr_vec(f, h->vertices);
        wr_vec(f, h->indices);
        wr_vec(f, h->albedo);
        wr_vec(f, h->nodes);
        wr_vec(f, h->prim_indices);
        wr_vec(f, h->neural_nodes);
        wr_vec(f, h->non_neural);
        f.write(reinterpret_cast<const char *>(h->scene_min), 12);
        f.write(reinterpret_cast<const char *>(h->scene_max), 12);
        wr_vec(f, p);
        wr_vec(f, m);
        wr_vec(f, v);
        if (!f)
            fail(NBVH_EIO, "checkpoint write failed");
    });
}

nbvh_status nbvh_load(nbvh_handle *h, const char *path)
{
    return guarded(h, [&]() {
        require(path != nullptr, NBVH_EINVAL, "null path");
        std::ifstream f(path, std::ios::binary);
        if (!f)
            fail(NBVH_EIO, "cannot open checkpoint");
        char magic[8];
        f.read(magic, 8);
        if (!f || std::memcmp(magic, kMagic, 8) != 0)
            fail(NBVH_EIO, "not an nbvh checkpoint");
        nbvh_config cfg;
        f.read(reinterpret_cast<char *>(&cfg), sizeof(cfg));
        uint32_t step = 0, flags = 0;
        f.read(reinterpret_cast<char *>(&step), 4);
        f.read(reinterpret_cast<char *>(&flags), 4);
        if (!f)
            fail(NBVH_EIO, "truncated checkpoint");
        validate_config(cfg);
        const uint64_t lim = 1ull << 31;
        std::vector<float> verts, albedo, p, m, v;
        std::vector<uint32_t> idx, prims;
        std::vector<BVHNode> nodes, neural;
        std::vector<uint8_t> non_neural;
        rd_vec(f, verts, lim);
        rd_vec(f, idx, lim);
        rd_vec(f, albedo, lim);
        rd_vec(f, nodes, lim);
        rd_vec(f, prims, lim);
        rd_vec(f, neural, lim);
        rd_vec(f, non_neural, lim);
        float smin[3], smax[3];
        f.read(reinterpret_cast<char *>(smin), 12);
        f.read(reinterpret_cast<char *>(smax), 12);
        rd_vec(f, p, lim);
        rd_vec(f, m, lim);
        rd_vec(f, v, lim);
        nbvh_param_layout L;
        GridParams g;
        compute_layout(cfg, L, g);
        if (p.size() != L.n_params || m.size() != L.n_params || v.size() != L.n_params)
            fail(NBVH_EIO, "checkpoint parameters do not match its configuration");
        if (idx.size() % 3u != 0u || verts.size() % 3u != 0u || non_neural.size() != neural.size())
            fail(NBVH_EIO, "malformed checkpoint mesh");
        for (uint32_t i : idx)
            if (i >= verts.size() / 3u)
                fail(NBVH_EIO, "checkpoint triangle index out of range");
        // commit
        apply_device_level_scales(cfg, L, g);
        h->cfg = cfg;
        h->layout = L;
        h->grid = g;
        h->vertices.swap(verts);
        h->indices.swap(idx);
        h->albedo.swap(albedo);
        h->nodes.swap(nodes);
        h->prim_indices.swap(prims);
        h->neural_nodes.swap(neural);
        std::memcpy(h->scene_min, smin, 12);
        std::memcpy(h->scene_max, smax, 12);
        h->classic_built = (flags & 1u) && !h->nodes.empty();
        h->neural_built = (flags & 2u) && !h->neural_nodes.empty();
        if (h->classic_built)
            upload_bvh(h);
        if (h->neural_built) {
            upload_neural(h);
            h->non_neural = non_neural;
            h->any_non_neural = false;
            for (uint8_t x : h->non_neural)
                h->any_non_neural |= x != 0u;
            if (h->any_non_neural) {
                cuda_check(h->d_non_neural.resize(h->non_neural.size()), "alloc flags");
                cuda_check(cudaMemcpy(h->d_non_neural.ptr, h->non_neural.data(), h->non_neural.size(),
                                      cudaMemcpyHostToDevice),
                           "upload flags");
            }
        }
        upload_params(h, p.data(), true);
        cuda_check(cudaMemcpy(h->d_adam_m.ptr, m.data(), m.size() * sizeof(float), cudaMemcpyHostToDevice), "adam m");
        cuda_check(cudaMemcpy(h->d_adam_v.ptr, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice), "adam v");
        h->training_step = step;
    });
}

// ---------------------------------------------------------------------------------------------
// Host-only utilities
// ---------------------------------------------------------------------------------------------

nbvh_status nbvh_build_bvh2_host(const float *v, uint32_t nv, const uint32_t *idx, uint32_t nt, uint32_t *h_nodes,
                                 uint32_t *n_nodes, uint32_t *h_prims)
{
    return guarded_free([&]() {
        require(v && idx && nv > 0 && nt > 0 && h_nodes && n_nodes && h_prims, NBVH_EINVAL, "bad arguments");
        for (size_t i = 0; i < 3u * (size_t)nt; i++)
            require(idx[i] < nv, NBVH_EINVAL, "triangle index out of range");
        std::vector<float> verts(v, v + 3u * (size_t)nv);
        std::vector<uint32_t> ind(idx, idx + 3u * (size_t)nt);
        std::vector<BVHNode> nodes;
        std::vector<uint32_t> prims;
        std::string err;
        if (!build_bvh2(verts, ind, nodes, prims, err))
            fail(NBVH_EINVAL, err);
        std::memcpy(h_nodes, nodes.data(), nodes.size() * sizeof(BVHNode));
        *n_nodes = (uint32_t)nodes.size();
        std::memcpy(h_prims, prims.data(), prims.size() * sizeof(uint32_t));
    });
}

nbvh_status nbvh_build_neural_cut_host(const uint32_t *h_nodes, uint32_t n_nodes, uint32_t max_depth,
                                       uint32_t *h_neural, uint32_t *n_neural)
{
    return guarded_free([&]() {
        require(h_nodes && n_nodes > 0 && h_neural && n_neural, NBVH_EINVAL, "bad arguments");
        std::vector<BVHNode> nodes(n_nodes);
        std::memcpy(nodes.data(), h_nodes, (size_t)n_nodes * sizeof(BVHNode));
        std::vector<BVHNode> neural;
        build_neural_cut(nodes, max_depth, neural);
        require(neural.size() <= *n_neural, NBVH_EINVAL, "neural node buffer too small");
        std::memcpy(h_neural, neural.data(), neural.size() * sizeof(BVHNode));
        *n_neural = (uint32_t)neural.size();
    });
}

nbvh_status nbvh_param_layout_host(const nbvh_config *cfg, nbvh_param_layout *out)
{
    return guarded_free([&]() {
        require(cfg && out, NBVH_EINVAL, "null argument");
        validate_config(*cfg);
        GridParams g;
        compute_layout(*cfg, *out, g);
    });
}

nbvh_status nbvh_init_params_host(const nbvh_config *cfg, float *h_params)
{
    return guarded_free([&]() {
        require(cfg && h_params, NBVH_EINVAL, "null argument");
        validate_config(*cfg);
        nbvh_param_layout L;
        GridParams g;
        compute_layout(*cfg, L, g);
        init_params(*cfg, L, h_params);
    });
}

nbvh_status nbvh_host_alloc(size_t bytes, void **out)
{
    if (!out)
        return NBVH_EINVAL;
    *out = nullptr;
    cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
    if (e == cudaErrorMemoryAllocation)
        return NBVH_ENOMEM;
    return e == cudaSuccess ? NBVH_OK : NBVH_EDEVICE;
}

nbvh_status nbvh_host_free(void *ptr)
{
    if (!ptr)
        return NBVH_OK;
    return cudaFreeHost(ptr) == cudaSuccess ? NBVH_OK : NBVH_EDEVICE;
}

} // extern "C"

// ---------------------------------------------------------------------------------------------
// Query and path-tracing cores shared with the serving loop (nbvh_server.cpp)
// ---------------------------------------------------------------------------------------------

namespace nbvh {

// Grows a query context to n rays for the handle's cut and network (allocates device and pinned
// memory; no kernel runs).
void grow_query_context(const nbvh_handle *h, QueryContext &q, uint32_t n)
{
    // record every device buffer's address: a capture of this context holds them
    const void *before[14] = {q.fallback_list.ptr, q.wave_counts.ptr, q.node_bins.ptr, q.node_cursor.ptr,
                              q.wpacked.ptr,       q.od0[0].ptr,       q.stack[0].ptr,  q.stack[1].ptr,
                              q.features.ptr,      q.outputs.ptr,      q.perm.ptr,      q.meta[1].ptr,
                              q.ray_keys.ptr,      q.ray_bins.ptr};
    if (q.fallback_list.count < n)
        cuda_check(q.fallback_list.resize(n), "alloc fallback list");
    if (q.wave_counts.count < 8u)
        cuda_check(q.wave_counts.resize(8u), "alloc wave counters");
    if (!q.h_words) {
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&q.h_words), 4u * sizeof(uint32_t), cudaHostAllocDefault),
                   "pinned counters");
        for (int k = 0; k < 4; k++)
            q.h_words[k] = 0;
    }
    const size_t cut = h->neural_nodes.size();
    if (q.node_bins.count < 2u * kSubBins * cut) { // room for the octant sub-bins of every node
        cuda_check(q.node_bins.resize(2u * kSubBins * cut), "alloc node counts");
        cuda_check(q.node_cursor.resize(2u * kSubBins * cut), "alloc node cursors");
    }
    const uint32_t wb = packed_weight_bytes(h->layout.n_inputs, (uint32_t)h->cfg.network.n_hidden_layers);
    if (q.wpacked.count < wb / 2u)
        cuda_check(q.wpacked.resize(wb / 2u), "alloc packed weights");
    if (q.ray_bins.count < kRayBins)
        cuda_check(q.ray_bins.resize(kRayBins), "alloc ray bin counts");
    if (!q.ev)
        cuda_check(cudaEventCreateWithFlags(&q.ev, cudaEventDisableTiming), "event");
    if (q.capacity < n || q.features.count < (size_t)n * h->layout.n_inputs) {
        for (int k = 0; k < 2; k++) {
            cuda_check(q.od0[k].resize(n), "alloc wave state");
            cuda_check(q.od1[k].resize(n), "alloc wave state");
            cuda_check(q.nv[k].resize(n), "alloc wave state");
            cuda_check(q.ar[k].resize(n), "alloc wave state");
            cuda_check(q.meta[k].resize(n), "alloc wave state");
            cuda_check(q.stack[k].resize((size_t)kNeuralStackSize * n), "alloc wave stacks");
        }
        cuda_check(q.features.resize((size_t)n * h->layout.n_inputs), "alloc feature rows");
        cuda_check(q.outputs.resize((size_t)n * kOutputs), "alloc network outputs");
        cuda_check(q.perm.resize(n), "alloc node order");
        cuda_check(q.ray_keys.resize(n), "alloc ray bins");
        q.capacity = n;
    }
    const void *after[14] = {q.fallback_list.ptr, q.wave_counts.ptr, q.node_bins.ptr, q.node_cursor.ptr,
                             q.wpacked.ptr,       q.od0[0].ptr,       q.stack[0].ptr,  q.stack[1].ptr,
                             q.features.ptr,      q.outputs.ptr,      q.perm.ptr,      q.meta[1].ptr,
                             q.ray_keys.ptr,      q.ray_bins.ptr};
    if (std::memcmp(before, after, sizeof(before)) != 0)
        q.generation++;
}

// The neural query itself on explicit per-call buffers (context q, counters): reads only the
// handle's scene, cut and parameters, so several contexts may run it at once on different
// streams. Returns the number of kernels launched.
uint32_t run_neural_query(const nbvh_handle *h, QueryContext &q, QueryCounters *counters, const nbvh_ray *d_rays,
                          uint32_t n, uint32_t depth, bool vis_only, nbvh_neural_hit *d_hits, cudaStream_t s,
                          const StepResources *tune)
{
    uint32_t *list = q.fallback_list.ptr;
    if (!tune || tune->resume_from == 0u)
        cuda_check(cudaMemsetAsync(counters, 0, sizeof(QueryCounters), s), "reset counters");
    if (h->cfg.bvh.ignore_neural_blas) {
        // the non-neural BLAS switch: the mesh goes to the classic traversal
        // (include/cuda/neural/neural_bvh_module_common.cuh:323)
        cuda_check(launch_classic_as_neural(h->d_nodes.ptr, h->d_tris.ptr, d_rays, n, d_hits, vis_only,
                                            h->classic_fast_div, s),
                   "classic");
        return 1u;
    }
    const NeuralConsts nc = make_neural_consts(h, depth, vis_only);
    WaveList lists[2];
    for (int k = 0; k < 2; k++)
        lists[k] = WaveList{q.od0[k].ptr, q.od1[k].ptr, q.nv[k].ptr, q.ar[k].ptr, q.meta[k].ptr, q.stack[k].ptr, q.capacity};
    uint32_t launches = 0;
    StepResources res;
    res.features = q.features.ptr;
    res.outputs = q.outputs.ptr;
    res.wpacked = q.wpacked.ptr;
    res.perm = q.perm.ptr;
    res.ray_keys = (h->ray_ordering && (!tune || tune->ray_order_ok)) ? q.ray_keys.ptr : nullptr;
    res.ray_bins = q.ray_bins.ptr;
    res.node_bins = q.node_bins.ptr;
    res.node_cursor = q.node_cursor.ptr;
    res.sub_bins = q.node_bins.count >= 2u * kSubBins * h->neural_nodes.size();
    // the ray-order keys are consumed by the placement before the first pass: the rows' sort bins
    // reuse the buffer from then on
    res.row_keys = q.ray_keys.count >= q.capacity ? q.ray_keys.ptr : nullptr;
    res.h_words = q.h_words;
    res.ev = q.ev;
    res.wait_ns = h->wait_limit_ns;
    res.stall = h->debug_stall;
    if (tune) {
        res.visits_per_round = tune->visits_per_round;
        res.encode_blocks_per_sm = tune->encode_blocks_per_sm;
        res.unchecked_steps = tune->unchecked_steps;
        res.capture_only = tune->capture_only;
        res.resume_from = tune->resume_from;
        res.drain_host = tune->drain_host;
        res.drain_stream = tune->drain_stream;
        res.drain_snap = tune->drain_snap;
        res.drain_done = tune->drain_done;
        res.drain_step = tune->drain_step;
        res.late_list = tune->late_list;
        res.late_count = tune->late_count;
        res.drain_taken = tune->drain_taken;
        res.stage_cut = tune->stage_cut;
    }
    res.sort_key = h->n_sort_bins ? h->d_sort_key.ptr : nullptr;
    res.n_sort_bins = h->n_sort_bins;
    if (h->kprof && !tune && &q == &h->qctx[0]) {
        h->kprof->used = 0;
        res.prof = h->kprof;
    }
    cuda_check(make_feature_map(q.features.ptr, h->layout.n_inputs, q.capacity, &res.feature_map), "feature map");
    cuda_check(launch_wave_query(h->d_neural_dilated.ptr, h->d_neural_bounds.ptr, (uint32_t)h->neural_nodes.size(),
                                 h->any_non_neural ? h->d_non_neural.ptr : nullptr, h->d_params_h.ptr, h->grid, nc,
                                 (uint32_t)h->cfg.network.n_hidden_layers, d_rays, n, d_hits, counters, list, lists,
                                 q.wave_counts.ptr, res, mlp_prec(h), h->num_sms, s, &launches),
               "neural query");
    if (tune && tune->capture_only)
        return launches; // the rest runs after the captured part is replayed
    if (h->any_non_neural || h->cfg.fallback_margin > 0.f) {
        cuda_check(launch_classic_fallback(h->d_nodes.ptr, h->d_tris.ptr, d_rays, list, counters, n, d_hits, vis_only,
                                           h->classic_fast_div, h->num_sms, s),
                   "fallback");
        launches++;
    }
    return launches;
}

// Path tracing on explicit buffers (the handle's or a serving slot's): raygen, then per bounce the
// neural query of the live paths and the shade / scatter step (one host read of the surviving
// count per bounce), then the per-pixel mean. Returns the rays queried.
uint64_t render_path_core(const nbvh_handle *h, QueryContext &q, QueryCounters *counters, PathBuffers &pb,
                          const nbvh_path_request *req, float *d_image, cudaStream_t s, uint32_t sample_base,
                          PathQuery *query)
{
    require(req && d_image, NBVH_EINVAL, "null request or image");
    const nbvh_render_request &cam = req->camera;
    require(cam.width > 0 && cam.height > 0 && req->spp > 0, NBVH_EINVAL, "empty image");
    const uint64_t n64 = (uint64_t)cam.width * cam.height * req->spp;
    require(n64 <= (1ull << 26), NBVH_EINVAL, "width * height * spp exceeds 2^26 paths");
    const uint32_t n = (uint32_t)n64;
    if (pb.thr.count < n) {
        cuda_check(pb.thr.resize(n), "alloc path throughput");
        cuda_check(pb.rad.resize(n), "alloc path radiance");
        for (int k = 0; k < 2; k++) {
            cuda_check(pb.rays[k].resize(n), "alloc path rays");
            cuda_check(pb.ids[k].resize(n), "alloc path ids");
        }
        cuda_check(pb.hits.resize(n), "alloc path hits");
    }
    if (pb.count.count < 1u)
        cuda_check(pb.count.resize(1u), "alloc path count");
    if (!pb.h_count)
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&pb.h_count), sizeof(uint32_t), cudaHostAllocDefault),
                   "pinned path count");
    if (!query)
        grow_query_context(h, q, n);
    PathArgs a{};
    camera_params(&cam, a.du, a.dv, a.tl);
    for (int k = 0; k < 3; k++) {
        a.origin[k] = cam.origin[k];
        a.ground_albedo[k] = req->ground_albedo[k];
        a.sky_zenith[k] = req->sky_zenith[k];
        a.sky_horizon[k] = req->sky_horizon[k];
    }
    a.width = cam.width;
    a.height = cam.height;
    a.spp = req->spp;
    a.n_paths = n;
    a.sample_base = sample_base;
    a.sample_offset = cam.sample_offset;
    a.seed = req->seed;
    a.max_bounces = req->max_bounces;
    a.has_ground = req->has_ground ? 1u : 0u;
    a.ground_y = req->ground_height;
    a.thr = pb.thr.ptr;
    a.rad = pb.rad.ptr;
    a.rays_out = pb.rays[0].ptr;
    a.ids_out = pb.ids[0].ptr;
    cuda_check(launch_path_raygen(a, s), "path raygen");
    uint32_t count = n;
    int cur = 0;
    uint64_t traced = 0;
    for (uint32_t bounce = 0; count > 0 && bounce <= req->max_bounces; bounce++) {
        const nbvh_neural_hit *hits = pb.hits.ptr;
        if (query)
            hits = (*query)(pb.rays[cur].ptr, count, bounce == 0 ? 1u : 2u);
        else
            run_neural_query(h, q, counters, pb.rays[cur].ptr, count, bounce == 0 ? 1u : 2u, false, pb.hits.ptr, s);
        traced += count;
        cuda_check(cudaMemsetAsync(pb.count.ptr, 0, sizeof(uint32_t), s), "reset path count");
        a.rays_in = pb.rays[cur].ptr;
        a.ids_in = pb.ids[cur].ptr;
        a.hits = hits;
        a.rays_out = pb.rays[cur ^ 1].ptr;
        a.ids_out = pb.ids[cur ^ 1].ptr;
        a.count_out = pb.count.ptr;
        cuda_check(launch_path_shade(a, count, bounce, s), "path shade");
        cuda_check(cudaMemcpyAsync(pb.h_count, pb.count.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "count");
        cuda_check(cudaStreamSynchronize(s), "sync");
        count = *pb.h_count;
        cur ^= 1;
    }
    cuda_check(launch_path_resolve(a, d_image, s), "path resolve");
    cuda_check(cudaStreamSynchronize(s), "sync");
    return traced;
}

} // namespace nbvh
