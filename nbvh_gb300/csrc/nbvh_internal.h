// nbvh_internal.h -- host-side internals of libnbvh (handle, device layouts, kernel launchers).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nbvh.h"

namespace nbvh {

// Host-side errors: thrown inside the library, turned into an nbvh_status at the C ABI.
struct Fail {
    nbvh_status status;
    std::string msg;
};

[[noreturn]] inline void fail(nbvh_status s, const std::string &m) { throw Fail{s, m}; }

inline void require(bool cond, nbvh_status s, const char *msg)
{
    if (!cond)
        fail(s, msg);
}

inline void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation)
            fail(NBVH_ENOMEM, std::string(what) + ": " + cudaGetErrorString(e));
        if (e == cudaErrorTimeout)
            fail(NBVH_ETIMEOUT, std::string(what) + ": a bounded device-side wait gave up");
        fail(NBVH_EDEVICE, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

constexpr uint32_t kNeuralStackSize = 24;  // NEURAL_STACK_SIZE, include/cuda/neural/accel/neural_bvh.cuh:22
constexpr uint32_t kClassicStackSize = 32; // CudaBVH2::intersect stack, include/cuda/accel/bvh2.cuh:22
constexpr uint32_t kNoNeuralChild = 0xFFFFFFFFu;
// NeuralBVH2Node leaf kinds (include/cuda/neural/accel/neural_bvh2.cuh:14-30): prim_count 1 is a
// final leaf (a classic leaf), 2 + l a leaf of LoD l (l in [0, 7), 0 the finest).
constexpr uint32_t kLeafFinal = 1u;
constexpr uint32_t kLeafLodBase = 2u;
constexpr uint32_t kNumBvhLods = 7u;
constexpr uint32_t kMaxLevels = 32;
constexpr uint32_t kMaxPoints = 16;
constexpr uint32_t kOutputs = 8;      // visibility, depth, normal(3), albedo(3)
constexpr uint32_t kOutputsPadded = 16;
constexpr uint32_t kNeurons = 64;
constexpr uint32_t kMaxInputs = 128;
constexpr uint32_t kMaxHiddenLayers = 8;

// 32-byte BVH2 node in the reference layout (include/base/accel/bvh.h:66-72).
struct BVHNode {
    float min[3];
    uint32_t prim_count;
    float max[3];
    uint32_t left_or_prim_offset;
};
static_assert(sizeof(BVHNode) == 32, "node layout");

// Hash-grid geometry shared by every kernel (copied into shared memory at kernel start).
// Kernels keep a copy in shared memory with 16-byte aligned data (matrices, ldmatrix tiles) placed
// right after it, so its size stays a multiple of 16 bytes: n_features comes with three words of
// padding.
struct GridParams {
    uint32_t n_levels;
    uint32_t n_points;
    uint32_t n_inputs;
    uint32_t segment_distribution;
    uint32_t offset[kMaxLevels];
    uint32_t size[kMaxLevels];
    uint32_t res[kMaxLevels];
    uint32_t hashed[kMaxLevels];
    float scale[kMaxLevels];
    uint32_t n_features; // per level: 2, 4 or 8 FP16 values per table entry
    uint32_t pad[3];
};
static_assert(sizeof(GridParams) % 16 == 0, "GridParams must keep 16-byte alignment after it");
// bytes a shared-memory copy of GridParams takes before the 16-byte aligned data that follows it
constexpr size_t kGridParamsSmem = (sizeof(GridParams) + 15u) & ~size_t(15);

// Constants of the neural traversal and decode (NeuralBVHRendererConstants /
// PathTracingOutputConstants subsets).
struct NeuralConsts {
    float inference_mint_epsilon, inference_maxt_epsilon;
    float learning_mint_epsilon, learning_maxt_epsilon;
    float sampling_bbox_scaling;
    float fixed_node_dilation, node_extent_dilation;
    float leaf_boundary_sampling_ratio;
    float visibility_threshold; // primary or secondary, chosen per call
    float depth_epsilon, fixed_depth_epsilon;
    float fallback_margin;
    float scene_min[3], scene_max[3];
    uint32_t bvh_lod;
    uint32_t max_traversal_steps;
    uint32_t visibility_only;
    uint32_t fast_div_ok; // every box coordinate of the cut is +0 or has magnitude in [2^-60, 2^11]
};

struct LossConsts {
    int32_t visibility_loss, depth_loss, normal_loss, albedo_loss;
    float visibility_loss_scale, depth_loss_scale, normal_loss_scale, albedo_loss_scale;
    int32_t normal_linear, albedo_linear, masking, learn_normal, learn_albedo;
    float loss_scale;
    float inv_n_total; // 1 / (n * dims)
};

// Device counters of one query (nbvh_query_stats) plus the work queue head.
struct QueryCounters {
    uint32_t queue_head;
    uint32_t segments;
    uint32_t step_capped;
    uint32_t stack_overflow;
    uint32_t fallback;
    uint32_t fallback_count; // entries written to the fallback list
    uint32_t work_count;     // rays that enter at least one leaf (compacted by the first pass)
    uint32_t encoded;        // segments whose features the wavefront encoder (k_wave_encode) computed
};

// Opt-in device timing of the wavefront encoder: one event pair around each k_wave_encode launch
// of a query (steps before the tail kernel; kMaxProfiledLaunches at most).
constexpr uint32_t kMaxProfiledLaunches = 32;
struct KernelProfile {
    cudaEvent_t ev[2 * kMaxProfiledLaunches] = {};
    uint32_t used = 0; // events recorded by the last profiled query
    // the last step of the last profiled run-optimisation call: before sampling, before the
    // encoding, before the tensor-core passes, after them, after the grid scatter, after Adam
    cudaEvent_t train_ev[6] = {};
    uint32_t train_rows = 0; // 0: no training step profiled yet
};

// One state list of the wavefront neural query (structure of arrays, `capacity` rays):
// od0 = {o, best_t}, od1 = {d, seg_mint}, meta = {seg_maxt bits, seg_node, ray id,
// segments | stack size << 16 | flags << 24}, nv = {normal, visibility}, ar = {albedo, rng bits},
// stack = [kNeuralStackSize][capacity] node indices.
struct WaveList {
    float4 *od0, *od1, *nv, *ar;
    uint4 *meta;
    uint32_t *stack;
    uint32_t capacity;
};

// Device allocations of the library's buffers: a count (nbvh_debug_alloc_count) and an injected
// failure (nbvh_debug_fail_allocations) for tests of the NBVH_ENOMEM paths.
cudaError_t device_alloc(void **ptr, size_t bytes);

template <typename T>
struct DeviceBuffer {
    T *ptr = nullptr;
    size_t count = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer() { release(); }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
    cudaError_t resize(size_t n)
    {
        if (n == count && ptr)
            return cudaSuccess;
        release();
        if (n == 0)
            return cudaSuccess;
        cudaError_t e = device_alloc(reinterpret_cast<void **>(&ptr), n * sizeof(T));
        if (e == cudaSuccess)
            count = n;
        else
            ptr = nullptr;
        return e;
    }
};

// Buffers of one query context: the two wavefront state lists, the rotating list counters, the
// fallback list, the feature rows / outputs of a step, the packed weights, and pinned words for
// the host's end-of-batch check.
struct QueryContext {
    DeviceBuffer<float4> od0[2], od1[2], nv[2], ar[2];
    DeviceBuffer<uint4> meta[2];
    DeviceBuffer<uint32_t> stack[2];
    DeviceBuffer<uint32_t> wave_counts;
    DeviceBuffer<uint32_t> fallback_list;
    DeviceBuffer<__half> features; // [capacity][n_inputs]
    DeviceBuffer<float> outputs;   // [capacity][8]
    DeviceBuffer<__half> wpacked;
    DeviceBuffer<uint32_t> perm;                   // [capacity]
    DeviceBuffer<uint16_t> ray_keys;               // [capacity] coherence bin of each ray
    DeviceBuffer<uint32_t> ray_bins;               // [kRayBins]
    DeviceBuffer<uint32_t> node_bins, node_cursor; // [2][cut nodes]
    uint32_t capacity = 0;
    uint64_t generation = 0;     // incremented whenever a buffer is reallocated
    uint32_t *h_words = nullptr; // 4 pinned words
    cudaEvent_t ev = nullptr;
    ~QueryContext()
    {
        if (h_words)
            cudaFreeHost(h_words);
        if (ev)
            cudaEventDestroy(ev);
    }
};

// Path tracing (k_path.cu): arguments of the raygen / shade / resolve kernels and the per-render
// buffers (per-path throughput and radiance, ping-pong ray and path-id lists, hits, list length).
struct PathArgs {
    float origin[3], du[3], dv[3], tl[3];
    uint32_t width, height, spp, n_paths, sample_base, sample_offset, seed, max_bounces;
    uint32_t has_ground;
    float ground_y;
    float ground_albedo[3];
    float sky_zenith[3], sky_horizon[3];
    float4 *thr; // rgb throughput, rng bits in w
    float4 *rad; // rgb radiance
    const nbvh_ray *rays_in;
    const uint32_t *ids_in;
    const nbvh_neural_hit *hits;
    nbvh_ray *rays_out;
    uint32_t *ids_out;
    uint32_t *count_out;
};

// One instance of an instanced scene: object-to-world affine map [A | b] (row-major 3x4), A^-1,
// the world box of the model's scene box, and whether the map is the identity (rays pass as they
// are).
struct InstanceArgs {
    float xform[12];
    float inv[9];
    float box_min[3], box_max[3];
    uint32_t identity;
    uint32_t instance;
};

struct PathBuffers {
    DeviceBuffer<float4> thr, rad;
    DeviceBuffer<nbvh_ray> rays[2];
    DeviceBuffer<uint32_t> ids[2];
    DeviceBuffer<nbvh_neural_hit> hits;
    DeviceBuffer<uint32_t> count;
    uint32_t *h_count = nullptr;
    ~PathBuffers()
    {
        if (h_count)
            cudaFreeHost(h_count);
    }
};

cudaError_t launch_path_raygen(const PathArgs &a, cudaStream_t s);
cudaError_t launch_path_shade(const PathArgs &a, uint32_t count_in, uint32_t bounce, cudaStream_t s);
cudaError_t launch_path_resolve(const PathArgs &a, float *image, cudaStream_t s);
// (ray, instance) pairs of one model's instances (group, device array) appended to the object list
cudaError_t launch_inst_group(const InstanceArgs *group, uint32_t n_group, const nbvh_ray *rays, uint32_t n,
                              nbvh_ray *obj_rays, uint32_t *obj_ids, float *obj_scale, uint32_t *obj_inst,
                              uint32_t *count, uint32_t capacity, cudaStream_t s);
cudaError_t launch_inst_reset(unsigned long long *keys, nbvh_neural_hit *hits, uint32_t n, cudaStream_t s);
// closest entry per world ray (64-bit atomic min of distance and entry) and its world record
cudaError_t launch_inst_vote_finalize(const InstanceArgs *all, const nbvh_neural_hit *obj_hits, const uint32_t *obj_ids,
                                      const float *obj_scale, const uint32_t *obj_inst, uint32_t total,
                                      unsigned long long *keys, nbvh_neural_hit *hits, uint32_t n, cudaStream_t s);

} // namespace nbvh

namespace nbvh {

// BvhSplitScheduler (include/cuda/neural/utils/bvh_split_scheduler.h:13-145)
struct SplitScheduler {
    int splitting_interval = 50, last_split_iteration = 2000, start_split_num = 1;
    float split_scaling = 2.0f, split_interval_scaling = 2.0f;
    int lod_decision_type = 0;
    int total_splits = 0; // expected over the whole schedule (m_stats.total_splits)
    int current_num_splits = 1, current_splitting_interval = 50, current_total_splits = 0;
    void configure(const nbvh_tree_cut_options &o);
    void reset();
    int get_bvh_splits(int iteration);
    // update_stats_and_reset: node count after n_iterations; graph (may be NULL) gets the splits
    // of each iteration capped by the leaves
    uint32_t expected(uint32_t start_nodes, uint32_t n_iterations, uint32_t *graph);
    bool should_assign_new_lod(int iteration, int current_lod, int num_lods_learned, int max_lods) const;
};

// A handle's learned-tree-cut session: the device holds nodes (in the handle's neural node array,
// sized for the whole classic BVH), per-node statistics, the neural -> classic node map and the
// TreeCutWord words; the host keeps the schedule.
struct TreeCutSession {
    bool active = false;
    bool learning = false;
    bool dirty = false;         // the device cut changed since the host copy was refreshed
    bool all_assigned = false;
    bool zero_next_max = false;
    nbvh_tree_cut_options opt{};
    SplitScheduler sched;
    uint32_t start_step = 0;
    uint32_t capacity = 0;
    uint32_t current_lod = 6;
    uint32_t expected_nodes = 0;
    DeviceBuffer<uint32_t> d_stats, d_map, d_keys, d_words;
};

} // namespace nbvh

struct nbvh_handle {
    std::mutex mu;
    std::string last_error;
    nbvh_config cfg{};
    int device = 0;

    // scene (host)
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    std::vector<float> albedo;
    std::vector<nbvh::BVHNode> nodes;
    std::vector<uint32_t> prim_indices;
    std::vector<nbvh::BVHNode> neural_nodes;
    std::vector<uint8_t> non_neural;
    float scene_min[3] = {0, 0, 0}, scene_max[3] = {0, 0, 0};
    bool classic_built = false, neural_built = false;

    // scene (device)
    nbvh::DeviceBuffer<float4> d_nodes;        // 2 float4 per node
    nbvh::DeviceBuffer<float4> d_tris;         // 3 float4 per triangle record (v0|prim, e1, e2)
    nbvh::DeviceBuffer<float> d_albedo;        // 3 per triangle (original order)
    nbvh::DeviceBuffer<float4> d_neural_nodes; // 2 float4 per node
    nbvh::DeviceBuffer<float4> d_neural_dilated; // inference copy: boxes dilated by fixed_node_dilation
    nbvh::DeviceBuffer<float4> d_neural_bounds;  // union of the dilated leaf boxes below each node
    nbvh::DeviceBuffer<uint32_t> d_sort_key;     // leaf -> sort bin for cuts above kMaxSortNodes nodes
    uint32_t n_sort_bins = 0;
    nbvh::DeviceBuffer<uint8_t> d_non_neural;
    bool any_non_neural = false;
    bool neural_fast_div = false;  // box coordinates of the cut inside the fast-division domain
    bool classic_fast_div = false; // same for the classic BVH

    // parameters
    nbvh_param_layout layout{};
    nbvh::GridParams grid{};
    std::vector<float> h_params; // FP32 master (host mirror, refreshed on demand)
    nbvh::DeviceBuffer<float> d_params;   // FP32 master
    nbvh::DeviceBuffer<__half> d_params_h; // 16-bit copy used by the kernels (MLP part FP16 or BF16, grid FP16)
    nbvh::DeviceBuffer<__half> d_wpacked;  // network matrices in the tensor-core operand layout
    nbvh::DeviceBuffer<__half> d_infer_feat; // feature rows of nbvh_network_inference
    nbvh::DeviceBuffer<uint32_t> d_status; // error word of kernels with bounded waits
    nbvh::DeviceBuffer<float> d_adam_m, d_adam_v;
    nbvh::DeviceBuffer<float> d_grad;
    uint32_t training_step = 0;

    // training workspace
    nbvh::DeviceBuffer<float> d_train_pos, d_train_tgt;
    nbvh::DeviceBuffer<float4> d_sample_state; // scratch of the training-ray search
    nbvh::DeviceBuffer<uint32_t> d_train_nodes;
    nbvh::DeviceBuffer<__half> d_train_feat;    // n x n_inputs encoded features (16-bit)
    nbvh::DeviceBuffer<__half> d_train_dfeat;   // n x n_inputs gradients of the features (16-bit)
    nbvh::DeviceBuffer<__half> d_train_wpacked; // network matrices in the tensor-core operand layout
    nbvh::DeviceBuffer<float> d_train_loss;  // per row loss (sum over output channels)
    nbvh::DeviceBuffer<float> d_loss_sum;
    nbvh::TreeCutSession cut;
    uint64_t model_version = 0; // bumped whenever a device array that queries read is reallocated

    // path-tracing workspace
    nbvh::PathBuffers path;

    // query workspace
    nbvh::DeviceBuffer<nbvh::QueryCounters> d_counters;
    // what nbvh_last_query_stats sums: the counters of the contexts in stat_ctx_mask (device-buffer
    // calls), or the n_stat_chunks per-chunk copies in d_stat_chunks (host-buffer calls, whose
    // chunks reuse a context's counters)
    nbvh::DeviceBuffer<nbvh::QueryCounters> d_stat_chunks;
    uint32_t n_stat_chunks = 0;
    uint32_t stat_ctx_mask = 1u;
    nbvh::DeviceBuffer<uint32_t> d_fallback_list;
    nbvh::QueryCounters last_counters{};
    uint32_t last_rays = 0;
    float last_kernel_ms = 0.f;
    nbvh::KernelProfile *kprof = nullptr; // set by nbvh_set_kernel_profile
    uint32_t last_launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_drain[2] = {nullptr, nullptr}; // early host copy of the records: taken, done
    nbvh::DeviceBuffer<uint32_t> d_late;           // late-finishing ray ids: [0] count, then the list
    nbvh::DeviceBuffer<nbvh_neural_hit> d_drain_hits;

    // host-buffer query pipeline
    cudaStream_t pipe_stream[2] = {nullptr, nullptr};
    void *pinned_in[2] = {nullptr, nullptr};
    void *pinned_out[2] = {nullptr, nullptr};
    size_t pinned_chunk = 0;
    nbvh::DeviceBuffer<uint8_t> d_pipe_in[2], d_pipe_out[2];
    nbvh::QueryContext qctx[3]; // 0: device-buffer calls, 1-2: the host-buffer pipeline streams

    int num_sms = 0;
    uint64_t wait_limit_ns = 0; // nbvh_debug_set_wait_limit (0: the kernels' default of one second)
    bool ray_ordering = true;   // nbvh_set_ray_ordering: batches of kRaySortMin rays or more taken bin by bin
    nbvh::DeviceBuffer<uint16_t> d_classic_keys;  // ray order of the classic queries
    nbvh::DeviceBuffer<uint32_t> d_classic_bins, d_classic_order;
    bool debug_stall = false;   // nbvh_debug_inject_stall
};

namespace nbvh {

// ---- kernel launchers (defined in the .cu files) ----
cudaError_t launch_classic(const float4 *nodes, const float4 *tris, const nbvh_ray *rays, uint32_t n,
                           nbvh_hit *hits, bool any_hit, const uint32_t *ray_list, bool fast_div, cudaStream_t s);

// Fallback pass: rays listed in `list` (count read on the device from counters) are answered by
// the classic BLAS and written into neural hit records.
cudaError_t launch_classic_fallback(const float4 *nodes, const float4 *tris, const nbvh_ray *rays,
                                    const uint32_t *list, const QueryCounters *counters,
                                    uint32_t max_list, nbvh_neural_hit *hits, bool any_hit, bool fast_div,
                                    int num_sms, cudaStream_t s);

cudaError_t launch_classic_as_neural(const float4 *nodes, const float4 *tris, const nbvh_ray *rays,
                                     uint32_t n, nbvh_neural_hit *hits, bool any_hit, bool fast_div, cudaStream_t s);

// Shared memory a block may take on sm_103 (static + dynamic).
constexpr int kMaxDynamicSmem = 227 * 1024;

// Every kernel with dynamic shared memory gets the same MaxDynamicSharedMemorySize attribute: the
// block limit minus the kernel's static shared memory. A launch then only needs its own size to
// fit, and threads launching one kernel for models of different sizes never lower the limit under
// each other.
template <typename K>
inline cudaError_t allow_max_dynamic_smem(K kernel)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kMaxDynamicSmem - (int)fa.sharedSizeBytes);
}

// Coherence bins of the rays of a query (24 direction classes, octant x dominant axis, x 8^3 origin
// cells of the scene box grown by half its size on every side): the first pass and the classic kernel take the rays bin
// by bin, so that the rays of a warp start near one another in the same direction. Batches below
// kRaySortMin rays are taken in batch order: the ordering's three launches (about 50 us) pay only
// on larger batches (measured: 2^22 uniform rays, classic 1.49 -> 1.09 ms; a 389K-ray camera batch,
// already coherent, 0.174 -> 0.213 ms).
constexpr uint32_t kRayBins = 12288; // 24 direction classes x 8^3 origin cells
constexpr uint32_t kRaySortMin = 1u << 19;

// Cuts with more nodes than this are not sorted by node between steps (the sort scans the node
// counts in shared memory).
constexpr uint32_t kMaxSortNodes = 8192;
constexpr uint32_t kSubBins = 8; // octants of a leaf box

// Opaque 128-byte CUDA tensor map (CUtensorMap) built on the host for TMA copies.
struct alignas(64) TensorMapBytes {
    unsigned char bytes[128];
};

// Per-query resources of the step loop besides the state lists: the FP16 feature rows and the
// network outputs of the current step, the packed weights, the tensor map over the feature rows,
// and the host words the end-of-batch check copies the 4 wave counters into (pinned, with ev
// recorded after the copy; when ev is null, h_words may be pageable and the host waits on the
// stream instead).
// How the FP32 master parameters become the 16-bit copy the kernels read.
struct ParamPrecision {
    uint32_t n_bf16; // the first n_bf16 parameters as BF16
    uint32_t fp8_lo, fp8_hi; // these as FP8-E4M3 values (scale 2^6) in FP16
};

struct StepResources {
    __half *features;
    float *outputs;
    __half *wpacked;
    uint32_t *perm;        // [capacity] rows in leaf-node order (nullptr: no sorting); before the first
                           // step, the order in which the first pass takes the rays
    uint16_t *ray_keys = nullptr; // [capacity] coherence bins of the rays (nullptr: rays in batch order)
    uint32_t *ray_bins = nullptr; // [kRayBins] counts, then placement cursors, of those bins
    uint32_t *node_bins;   // [2][n_cut_nodes]
    uint32_t *node_cursor; // [2][n_cut_nodes]
    TensorMapBytes feature_map;
    uint32_t *h_words;
    cudaEvent_t ev;
    // launch parameters (0 = default) and the graph-capture split of the step loop
    uint32_t visits_per_round = 0;     // node visits per traversal round between lane refills
    uint32_t encode_blocks_per_sm = 0; // blocks of 256 encoder threads per SM
    uint32_t unchecked_steps = 0;      // steps launched before the first host check
    bool capture_only = false;         // enqueue the unchecked steps and a counter copy, then return
    uint32_t resume_from = 0;          // > 0: skip the first pass and continue the checked loop here
    // early host copy of the records (page-locked destination, device address): taken on
    // drain_stream after the decode of step drain_step; rays finishing later go to late_list
    nbvh_neural_hit *drain_host = nullptr;
    cudaStream_t drain_stream = nullptr;
    cudaEvent_t drain_snap = nullptr, drain_done = nullptr;
    uint32_t drain_step = 0;
    uint32_t *late_list = nullptr;  // [n]
    uint32_t *late_count = nullptr;
    bool *drain_taken = nullptr;    // set when the early copy was enqueued
    // sort bins of the leaves of a cut above kMaxSortNodes nodes (NULL: one bin per node)
    const uint32_t *sort_key = nullptr;
    uint32_t n_sort_bins = 0;
    KernelProfile *prof = nullptr; // record encoder launch events (not under stream capture)
    uint64_t wait_ns = 0;          // time limit of the tensor-core kernels' phase waits (0: default)
    bool ray_order_ok = true;      // false: rays in host memory read over the link, taken in batch order
    // decode and tail kernels with the cut staged in shared memory (when it fits) instead of read
    // through L1; off by default: through L1 the tail runs two blocks per SM instead of one, more
    // gathers in flight (2,047-node cut, 2^22 rays: 3.33 against 3.37 ms per query)
    bool stage_cut = false;
    // the rows of each leaf in kSubBins sort bins by the octant of their segment midpoint (needs
    // node_bins / node_cursor of 2 x kSubBins x the cut's nodes)
    bool sub_bins = false;
    // [capacity] 16-bit sort bin of each listed row, written by the kernel that appends the row and
    // read by the sort (nullptr: the sort recomputes the bins); may be the ray-order key buffer,
    // which is free once the first pass has taken the rays
    uint16_t *row_keys = nullptr;
    bool stall = false;            // failure-path tests: the MLP kernels wait on a barrier nothing arrives at
};

// Scratch of the allocation-free neural query: one static device buffer per device holding, for
// NBVH_NOALLOC_MAX_RAYS rays, both wave lists, the feature rows and outputs of a step, the packed
// weights, the node-sort buffers, the fallback list, the counters and the wave counters. Every region starts on a
// 256-byte boundary.
struct NoallocScratch {
    WaveList lists[2];
    __half *features;
    float *outputs;
    __half *wpacked;
    uint32_t *perm;
    uint32_t *node_bins;
    uint32_t *node_cursor;
    uint32_t *fallback_list;
    QueryCounters *counters;
    uint32_t *wave_counts;
};
constexpr size_t kNoallocRays = NBVH_NOALLOC_MAX_RAYS;
static_assert(kNoallocRays % 64u == 0u, "regions must stay 256-byte aligned");
constexpr size_t kNoallocListBytes = kNoallocRays * (4u * sizeof(float4) + sizeof(uint4) + kNeuralStackSize * 4u);
constexpr size_t kNoallocFeatureBytes = kNoallocRays * kMaxInputs * 2u;
constexpr size_t kNoallocOutputBytes = kNoallocRays * kOutputs * 4u;
constexpr size_t kNoallocWeightBytes = // W0 at most 64 x 128, at most 7 more 64 x 64, output 16 x 64
    ((kNeurons * kMaxInputs + (kMaxHiddenLayers - 1u) * kNeurons * kNeurons + kOutputsPadded * kNeurons) * 2u + 255u) &
    ~size_t(255);
constexpr size_t kNoallocSortBytes = kNoallocRays * 4u + 4u * kMaxSortNodes * 4u; // perm, bins, cursors
constexpr size_t kNoallocBytes = 2u * kNoallocListBytes + kNoallocFeatureBytes + kNoallocOutputBytes +
                                 kNoallocWeightBytes + kNoallocSortBytes + kNoallocRays * 4u + 256u + 256u;
// The buffer's address on `device` (which must be current): looked up on the first call for that
// device and cached. Fails with cudaErrorInvalidDevice for device ids beyond the cache.
cudaError_t noalloc_scratch(int device, NoallocScratch *out);

// Wavefront neural query (k_query.cu): first-leaf pass, then batches of K3 -> K4 -> K2 steps,
// the list length checked by the host after each batch. Returns when the loop has finished;
// cudaErrorTimeout if a bounded wait inside the tensor-core MLP gave up.
cudaError_t launch_wave_query(const float4 *dilated_nodes, const float4 *bounds, uint32_t n_cut_nodes,
                              const uint8_t *non_neural, const __half *params_h, const GridParams &grid,
                              const NeuralConsts &nc, uint32_t n_hidden_layers, const nbvh_ray *rays, uint32_t n,
                              nbvh_neural_hit *hits, QueryCounters *counters, uint32_t *fallback_list,
                              const WaveList lists[2], uint32_t *wave_counts, const StepResources &res, uint32_t prec,
                              int num_sms, cudaStream_t s, uint32_t *launches);

// Sets the shared-memory attributes of every variant of the query's kernels with dynamic shared
// memory (decode, tail, tensor-core MLP) on the current device. A direct query sets those of the
// variants it launches; a stream capture cannot, so the serving loop calls this before capturing.
cudaError_t configure_query_kernels();

// order[0..n) = the ray ids bin by bin (coherence bins over the scene box, kRayBins of them);
// keys: n, bins: kRayBins device words of scratch. Three kernels and a memset on the stream.
cudaError_t launch_ray_order(const nbvh_ray *rays, uint32_t n, const float scene_min[3], const float scene_max[3],
                             uint16_t *keys, uint32_t *bins, uint32_t *order, int num_sms, cudaStream_t s);

cudaError_t launch_segments(const float4 *dilated_nodes, const float4 *bounds, const NeuralConsts &nc,
                            const nbvh_ray *rays, uint32_t n, uint32_t max_segments, nbvh_segment *segs,
                            uint32_t *counts, cudaStream_t s);

// The FP16 (BF16 when bf16) hash-grid features of n rows of encoded positions into rows of
// n_inputs values (the tcgen05 MLP's input layout).
cudaError_t launch_encode_rows(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                               const float *positions, uint32_t n, __half *features, bool bf16, cudaStream_t s);

// tcgen05 fully fused MLP (k_mlp_tc.cu): weights packed into the tensor-core operand layout, then
// 128-row tiles of FP16 inputs (row-major [rows][n_inputs], 16-byte aligned) fed by TMA through
// the tensor map of make_feature_map. The rows processed are min(*d_count, rows) when d_count is
// given (a length produced on the device), else rows. status receives a nonzero word if a bounded
// wait inside the kernel gave up. configure = false skips setting the kernel's shared-memory
// attribute (during stream capture, after an earlier launch set it).
uint32_t packed_weight_bytes(uint32_t n_inputs, uint32_t n_hidden_layers);
cudaError_t launch_pack_weights(const __half *params_h, uint32_t n_inputs, uint32_t n_hidden_layers, __half *packed,
                                cudaStream_t s);
// allow_swizzle = false: always 8-value boxes, so that a 128-row tile lands in shared memory in
// the unswizzled K-major core-matrix layout (column block c of 8 values at c * 2,048 bytes).
cudaError_t make_feature_map(const __half *features, uint32_t n_inputs, uint32_t rows, TensorMapBytes *out,
                             bool allow_swizzle = true);
// wait_ns: time limit of the kernel's phase waits (0: the default of one second). stall (failure-path
// tests): one wait on an mbarrier that nothing arrives at, which runs out after wait_ns.
// MaxDynamicSharedMemorySize of the tensor-core MLP's variants (FP16, BF16, FP8) on the current device.
cudaError_t configure_mlp_tc();
cudaError_t launch_mlp_tc(const TensorMapBytes &feature_map, const __half *wpacked, uint32_t n_inputs,
                          uint32_t n_hidden_layers, uint32_t rows, const uint32_t *d_count, float *outputs,
                          uint32_t *status, uint32_t prec, int num_sms, cudaStream_t s, bool configure = true,
                          uint64_t wait_ns = 0, bool stall = false);

cudaError_t launch_encode(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                          const float *positions, uint32_t n, float *features, cudaStream_t s);

// words of the device state: node count, the heuristic maximum of the two most recent steps (bits of
// a non-negative float), the deepest node, splits done, an error flag (capacity exceeded)
enum TreeCutWord : uint32_t {
    kCutCount = 0,
    kCutMax0 = 1,
    kCutMax1 = 2,
    kCutMaxDepth = 3,
    kCutSplits = 4,
    kCutError = 5,
    kCutWords = 8
};

struct TreeCutArgs {
    float4 *nodes;          // neural nodes, 2 float4 each, `capacity` of them
    const float4 *classic;  // classic nodes
    uint32_t *stats;        // 4 words per node: f32 loss, iter_alive, depth, samples
    uint32_t *node_map;     // neural node -> classic node
    uint32_t *keys;         // scratch, one word per node
    uint32_t *words;        // TreeCutWord
    uint32_t capacity;
};

// Node survival of the training sampler: stats / max_word NULL (or disabled) keeps every sample.
struct NodeSurvival {
    const uint32_t *stats;
    const uint32_t *max_word; // heuristic maximum of the previous step; NULL reads as 0
    float scale;
    float min_prob;
    uint32_t enabled;
};

// Training rays of one step: the leaf-segment search, then the labels (two kernels). state:
// sample_state_float4s(n) float4 of device scratch.
inline size_t sample_state_float4s(uint32_t n) { return (size_t)n * 3u + 1u; }
cudaError_t launch_training_samples(const float4 *neural_nodes, const float4 *nodes, const float4 *tris,
                                    const float *albedo, const NeuralConsts &nc, const GridParams &grid,
                                    uint32_t training_step, uint32_t batch_size, uint32_t n, float *positions,
                                    float *targets, uint32_t *sample_nodes, uint32_t learned_lod,
                                    const NodeSurvival *survival, float4 *state, bool classic_fast_div, int num_sms,
                                    cudaStream_t s);

// One training pass over n rows (positions n x points x 3, targets n x 8): the hash-grid features
// into `features` (n x n_inputs, 16-bit), the network matrices packed into `wpacked`
// (packed_weight_bytes), forward + composite loss + backward on the tcgen05 tensor cores (the
// weight gradients added to grad, the loss sum into *loss_sum, per-row losses into sample_loss
// when not NULL, the 16-bit feature gradients into dfeat, n x n_inputs), then the hash-grid
// gradient scattered into grad + n_network_params. grad holds the gradient times the loss scale.
// status receives a nonzero word if a bounded wait inside the tensor-core kernel gave up.
cudaError_t launch_train_step(const __half *params_h, const GridParams &grid, uint32_t n_hidden_layers,
                              const LossConsts &lc, const float *positions, const float *targets, uint32_t n,
                              __half *features, __half *dfeat, __half *wpacked, float *grad, float *loss_sum,
                              float *sample_loss, uint32_t *status, bool bf16, bool fp8, int num_sms, cudaStream_t s,
                              uint64_t wait_ns = 0, bool stall = false, const cudaEvent_t *marks = nullptr);
// (marks, when given: 4 events recorded before the encoding, before and after the tensor-core
// passes, and after the grid scatter)

// ---- learned tree cut (k_tree_cut.cu) ----
// Copies the records of the late-listed rays from src (device) to dst (page-locked host).
cudaError_t launch_copy_late(const uint32_t *late, const uint32_t *late_count, uint32_t n, const nbvh_neural_hit *src,
                             nbvh_neural_hit *dst, int num_sms, cudaStream_t s);

cudaError_t launch_cut_accumulate(const float *sample_loss, const uint32_t *sample_nodes, uint32_t n, uint32_t dims,
                                  uint32_t *stats, cudaStream_t s);
cudaError_t launch_cut_alive_max(const TreeCutArgs &a, uint32_t slot, int num_sms, cudaStream_t s);
cudaError_t launch_cut_split(const TreeCutArgs &a, uint32_t k, uint32_t lod, cudaStream_t s);
cudaError_t launch_cut_assign_lod(const TreeCutArgs &a, uint32_t lod, int num_sms, cudaStream_t s);

cudaError_t launch_scale(float *data, size_t n, float scale, cudaStream_t s);

cudaError_t launch_adam(float *params, __half *params_h, float *m, float *v, const float *grad, uint32_t n,
                        float lr_t, float beta1, float beta2, float eps, float l2_reg, float grad_scale,
                        const ParamPrecision &pp, cudaStream_t s);

// 16-bit copy of the FP32 parameters: the first pp.n_bf16 (the network matrices when the MLP runs
// in BF16) as BF16, [pp.fp8_lo, pp.fp8_hi) (the hidden matrices in FP8 mode) as FP8-E4M3 values at
// scale 2^6 held in FP16, the rest as FP16.
cudaError_t launch_params_to_half(const float *params, __half *params_h, uint32_t n, const ParamPrecision &pp,
                                  cudaStream_t s);

// scale_l of levels 0 .. n-1 (n <= 32) evaluated on the device: exp2f(l * log2_scale) * base - 1
cudaError_t launch_level_scales(float log2_scale, float base, uint32_t n, float *out, cudaStream_t s);
cudaError_t launch_camera_rays(uint32_t width, uint32_t height, uint32_t sample_idx, uint32_t sample_offset,
                               const float *origin, const float *du, const float *dv, const float *top_left,
                               nbvh_ray *rays, cudaStream_t s);

// ---- host builders (bvh_builder.cpp) ----
// Binned-SAH BVH2 with leaves of 1..2 triangles; children of a node are adjacent; returns false
// when the tree depth exceeds the traversal stack.
bool build_bvh2(const std::vector<float> &vertices, const std::vector<uint32_t> &indices,
                std::vector<BVHNode> &nodes, std::vector<uint32_t> &prim_indices, std::string &err);
// Sort bins of the leaves of a cut (rendered LoD): leaves in depth-first order split into at most
// max_bins runs of equal length; interior nodes get bin 0. Returns the number of bins.
uint32_t build_sort_keys(const std::vector<BVHNode> &neural, uint32_t max_bins, std::vector<uint32_t> &keys);
void build_neural_cut(const std::vector<BVHNode> &nodes, uint32_t max_depth, std::vector<BVHNode> &neural,
                      std::vector<uint32_t> *node_map = nullptr, std::vector<uint32_t> *depth = nullptr);
void build_inference_nodes(const std::vector<BVHNode> &neural, float dil, std::vector<BVHNode> &dilated,
                           std::vector<float> &bounds);
// true when every coordinate is +0 or has magnitude in [2^-60, 2^11] (no -0, no subnormal range),
// the box-coordinate precondition of the fast slab division
bool coords_in_fast_div_domain(const float *c, size_t n);
bool nodes_in_fast_div_domain(const std::vector<BVHNode> &nodes);

} // namespace nbvh

namespace nbvh {

// Grows a query context to n rays for the handle's cut and network (allocates device and pinned
// memory; no kernel runs).
void grow_query_context(const nbvh_handle *h, QueryContext &q, uint32_t n);

// The neural query on explicit per-call buffers (context q, counters): reads only the handle's
// scene, cut and parameters, so several contexts may run it at once on different streams.
// `tune` (may be null) carries launch parameters and the graph-capture split of the step loop.
// Returns the kernels launched.
uint32_t run_neural_query(const nbvh_handle *h, QueryContext &q, QueryCounters *counters, const nbvh_ray *d_rays,
                          uint32_t n, uint32_t depth, bool vis_only, nbvh_neural_hit *d_hits, cudaStream_t s,
                          const StepResources *tune = nullptr);

// Neural query used by the path tracer for one bounce: answers n rays at `rays` with closest-hit
// depth `depth` on the stream and returns where the hits are.
struct PathQuery {
    virtual const nbvh_neural_hit *operator()(const nbvh_ray *rays, uint32_t n, uint32_t depth) = 0;
    virtual ~PathQuery() = default;
};

// Path tracing on explicit buffers; returns the rays queried over all bounces. Sample k of a pixel
// (k < req->spp) uses the camera jitter of frame sample sample_base + k (a whole frame:
// camera.sample_idx * spp; a chunk of a frame's samples starts further in). `query` (may be null)
// replaces the direct neural query of each bounce (the serving loop's graph replays).
uint64_t render_path_core(const nbvh_handle *h, QueryContext &q, QueryCounters *counters, PathBuffers &pb,
                          const nbvh_path_request *req, float *d_image, cudaStream_t s, uint32_t sample_base,
                          PathQuery *query = nullptr);

// Pinhole camera basis of a render request (CudaBackend::update_camera, src/cuda/cuda_backend.cpp:595-611).
void camera_params(const nbvh_render_request *r, float du[3], float dv[3], float tl[3]);

} // namespace nbvh

namespace nbvh {

// ---- learned tree cut (nbvh_tree_cut.cpp) ----
void validate_tree_cut_options(const nbvh_tree_cut_options &o);
void begin_tree_cut(nbvh_handle *h, const nbvh_tree_cut_options &o, uint32_t start_depth);
void end_tree_cut(nbvh_handle *h);
TreeCutArgs tree_cut_args(nbvh_handle *h);
void tree_cut_before_step(nbvh_handle *h, NodeSurvival &survival, uint32_t &learned_lod);
void tree_cut_after_step(nbvh_handle *h, const float *sample_loss, uint32_t n, cudaStream_t s);
void tree_cut_words(nbvh_handle *h, uint32_t *words, cudaStream_t s); // kCutWords + kNumBvhLods words
void tree_cut_sync(nbvh_handle *h, cudaStream_t s);
// inference copies of the neural cut (dilated boxes, subtree bounds) from h->neural_nodes
void upload_inference_nodes(nbvh_handle *h);

// The reference's .nbvh neural-cut file (nbvh_format.cpp): read (with structural validation) and write.
bool validate_cut(const std::vector<BVHNode> &nodes, std::string &err);
bool read_nbvh(const std::string &path, std::vector<BVHNode> &nodes, std::string &err);
bool write_nbvh(const std::string &path, const std::vector<BVHNode> &nodes, std::string &err);
// tcnn trainer weights (JSON text of trainer->serialize): parameters as FP32 (16-bit widened)
bool read_tcnn_params(const char *path, std::vector<float> &params, std::string &err);
bool write_tcnn_params(const char *path, const float *params, uint64_t n, std::string &err);

} // namespace nbvh
