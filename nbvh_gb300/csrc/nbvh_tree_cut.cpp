// nbvh_tree_cut.cpp -- host side of the learned tree cut: the split scheduler, the session state
// of a handle and the per-step launches that run inside nbvh_run_optimisation.
//
// Reference: NeuralBVHRenderer::render's tree-cut branch (src/cuda/neural/neural_bvh_renderer.cu:
// 196-282), BvhSplitScheduler (include/cuda/neural/utils/bvh_split_scheduler.h:13-145),
// reinitialise_tree_cut_learning_data (src/cuda/neural/neural_bvh_renderer_init.cu:61-74) and
// build_and_upload_neural_bvh (src/cuda/neural/neural_bvh_renderer_accel.cpp:504-557). The
// reference copies the maximum and the split list to the host and splits there every step; here
// the node count, the maximum and the split stay on the device and the host only schedules.
#include <cstring>

#include "nbvh_internal.h"

namespace nbvh {

void SplitScheduler::configure(const nbvh_tree_cut_options &o)
{
    splitting_interval = o.splitting_interval;
    last_split_iteration = o.last_split_iteration;
    start_split_num = o.start_split_num;
    split_scaling = o.split_scaling;
    split_interval_scaling = o.split_interval_scaling;
    lod_decision_type = o.lod_decision_type;
    reset();
}

void SplitScheduler::reset()
{
    current_num_splits = start_split_num;
    current_splitting_interval = splitting_interval;
    current_total_splits = 0;
}

int SplitScheduler::get_bvh_splits(int iteration)
{
    if (iteration == 0)
        reset();
    if (iteration > last_split_iteration)
        return 0;
    int n = 0;
    if (iteration % splitting_interval == 0) {
        n = current_num_splits;
        current_total_splits += n;
    }
    if (current_splitting_interval > 0 && iteration % current_splitting_interval == 0) {
        // int *= float in the reference: the product in float, truncated back to int
        current_num_splits = (int)((float)current_num_splits * split_scaling);
        current_splitting_interval = (int)((float)current_splitting_interval * split_interval_scaling);
    }
    return n;
}

uint32_t SplitScheduler::expected(uint32_t start_nodes, uint32_t n_iterations, uint32_t *graph)
{
    uint64_t nodes = start_nodes;
    uint32_t total = 0;
    for (uint32_t i = 0; i < n_iterations; i++) {
        const uint64_t leaves = (nodes + 1u) / 2u;
        int k = get_bvh_splits((int)i);
        if (k > 0) {
            if ((uint64_t)k > leaves)
                k = (int)leaves;
            total += (uint32_t)k;
            nodes += 2u * (uint64_t)k;
        }
        if (graph)
            graph[i] = (uint32_t)k > 0 ? (uint32_t)k : 0u;
    }
    total_splits = (int)total;
    reset();
    return nodes > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)nodes;
}

bool SplitScheduler::should_assign_new_lod(int iteration, int current_lod, int num_lods_learned, int max_lods) const
{
    bool assign;
    if (lod_decision_type == 0) {
        const int next = (max_lods - current_lod) * last_split_iteration / num_lods_learned;
        assign = next <= iteration;
    } else {
        const int next = (max_lods - current_lod) * total_splits / num_lods_learned;
        assign = next <= current_total_splits;
    }
    return assign || iteration >= last_split_iteration;
}

void validate_tree_cut_options(const nbvh_tree_cut_options &o)
{
    require(o.splitting_interval > 0, NBVH_EINVAL, "splitting_interval must be positive");
    require(o.last_split_iteration >= 0, NBVH_EINVAL, "last_split_iteration must be non-negative");
    require(o.start_split_num >= 0, NBVH_EINVAL, "start_split_num must be non-negative");
    require(o.split_scaling >= 0.0f && o.split_interval_scaling >= 0.0f, NBVH_EINVAL, "negative scaling");
    require(o.num_lods_learned >= 1 && o.num_lods_learned <= (int)kNumBvhLods, NBVH_EINVAL,
            "num_lods_learned must be in [1, 7]");
    require(o.lod_decision_type == 0 || o.lod_decision_type == 1, NBVH_EINVAL, "unknown lod_decision_type");
    require(o.min_rr_survival_prob >= 0.0f && o.survival_probability_scale >= 0.0f, NBVH_EINVAL,
            "negative survival probability");
}

TreeCutArgs tree_cut_args(nbvh_handle *h)
{
    TreeCutSession &c = h->cut;
    TreeCutArgs a;
    a.nodes = h->d_neural_nodes.ptr;
    a.classic = h->d_nodes.ptr;
    a.stats = c.d_stats.ptr;
    a.node_map = c.d_map.ptr;
    a.keys = c.d_keys.ptr;
    a.words = c.d_words.ptr;
    a.capacity = c.capacity;
    return a;
}

void end_tree_cut(nbvh_handle *h)
{
    TreeCutSession &c = h->cut;
    c.active = false;
    c.learning = false;
    c.d_stats.release();
    c.d_map.release();
    c.d_keys.release();
    c.d_words.release();
}

void begin_tree_cut(nbvh_handle *h, const nbvh_tree_cut_options &o, uint32_t start_depth)
{
    validate_tree_cut_options(o);
    require(h->classic_built, NBVH_ESTATE, "classic BVH not built");
    TreeCutSession &c = h->cut;
    end_tree_cut(h);
    std::vector<uint32_t> node_map, depth;
    build_neural_cut(h->nodes, start_depth, h->neural_nodes, &node_map, &depth);
    const uint32_t n = (uint32_t)h->neural_nodes.size();
    c.capacity = (uint32_t)h->nodes.size();
    // neural nodes: the device array holds the largest cut this classic BVH allows
    cuda_check(h->d_neural_nodes.resize(2u * (size_t)c.capacity), "alloc neural nodes");
    cuda_check(cudaMemcpy(h->d_neural_nodes.ptr, h->neural_nodes.data(), (size_t)n * sizeof(BVHNode),
                          cudaMemcpyHostToDevice),
               "upload neural nodes");
    upload_inference_nodes(h);
    std::vector<uint32_t> stats(4u * (size_t)n, 0u);
    for (uint32_t i = 0; i < n; i++) {
        stats[4u * i + 1u] = 1u; // iter_alive starts at 1 (traverse_and_build_neural_bvh)
        stats[4u * i + 2u] = depth[i];
    }
    cuda_check(c.d_stats.resize(4u * (size_t)c.capacity), "alloc tree-cut stats");
    cuda_check(c.d_map.resize(c.capacity), "alloc node map");
    cuda_check(c.d_keys.resize(c.capacity), "alloc selection keys");
    cuda_check(c.d_words.resize(kCutWords + kNumBvhLods), "alloc tree-cut words");
    cuda_check(cudaMemcpy(c.d_stats.ptr, stats.data(), stats.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
               "upload tree-cut stats");
    cuda_check(cudaMemcpy(c.d_map.ptr, node_map.data(), node_map.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
               "upload node map");
    std::vector<uint32_t> words(kCutWords + kNumBvhLods, 0u);
    words[kCutCount] = n;
    uint32_t max_depth = 0;
    for (uint32_t d : depth)
        max_depth = d > max_depth ? d : max_depth;
    words[kCutMaxDepth] = max_depth;
    cuda_check(cudaMemcpy(c.d_words.ptr, words.data(), words.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
               "upload tree-cut words");
    c.opt = o;
    c.sched.configure(o);
    c.expected_nodes = c.sched.expected(n, (uint32_t)o.last_split_iteration + 1u, nullptr);
    c.start_step = h->training_step;
    c.current_lod = kNumBvhLods - 1u;
    c.all_assigned = false;
    c.zero_next_max = false;
    c.learning = o.tree_cut_learning != 0;
    c.active = true;
    c.dirty = false;
    h->neural_built = true;
}

void tree_cut_before_step(nbvh_handle *h, NodeSurvival &survival, uint32_t &learned_lod)
{
    TreeCutSession &c = h->cut;
    const uint32_t it = h->training_step - c.start_step;
    learned_lod = c.current_lod;
    survival.enabled = c.opt.training_node_survival ? 1u : 0u;
    survival.stats = c.d_stats.ptr;
    // the maximum of the previous step; 0 for the first step (and after the last LoD assignment,
    // whose reinitialise_tree_cut_learning_data(1) zeroes the host copy)
    survival.max_word = (it == 0 || c.zero_next_max) ? nullptr : c.d_words.ptr + kCutMax0 + ((it - 1u) & 1u);
    survival.scale = c.opt.survival_probability_scale;
    survival.min_prob = c.opt.min_rr_survival_prob;
    c.zero_next_max = false;
}

void tree_cut_after_step(nbvh_handle *h, const float *sample_loss, uint32_t n, cudaStream_t s)
{
    TreeCutSession &c = h->cut;
    const uint32_t it = h->training_step - c.start_step;
    const nbvh_config &cfg = h->cfg;
    const uint32_t dims = 2u + (cfg.output.learn_normal ? 3u : 0u) + (cfg.output.learn_albedo ? 3u : 0u);
    const TreeCutArgs a = tree_cut_args(h);
    cuda_check(launch_cut_accumulate(sample_loss, h->d_train_nodes.ptr, n, dims, c.d_stats.ptr, s), "tree-cut loss");
    cuda_check(launch_cut_alive_max(a, kCutMax0 + (it & 1u), h->num_sms, s), "tree-cut maximum");
    if (!c.learning)
        return;
    const int k = c.sched.get_bvh_splits((int)it);
    if (k > 0) {
        cuda_check(launch_cut_split(a, (uint32_t)k, c.current_lod, s), "tree-cut split");
        c.dirty = true;
    }
    if (c.opt.num_lods_learned > 1 && !c.all_assigned) {
        if (c.sched.should_assign_new_lod((int)it, (int)c.current_lod, c.opt.num_lods_learned, (int)kNumBvhLods)) {
            if (c.current_lod != kNumBvhLods - 1u)
                cuda_check(launch_cut_assign_lod(a, c.current_lod, h->num_sms, s), "tree-cut LoD");
            cuda_check(cudaMemcpyAsync(c.d_words.ptr + kCutWords + c.current_lod, c.d_words.ptr + kCutCount,
                                       sizeof(uint32_t), cudaMemcpyDeviceToDevice, s),
                       "LoD node count");
            c.all_assigned = c.current_lod == 0u;
            if (!c.all_assigned)
                c.current_lod--;
            else
                c.learning = false;
            c.dirty = true;
        }
        if (c.all_assigned)
            c.zero_next_max = true;
    }
}

void tree_cut_words(nbvh_handle *h, uint32_t *words, cudaStream_t s)
{
    cuda_check(cudaMemcpyAsync(words, h->cut.d_words.ptr, (kCutWords + kNumBvhLods) * sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, s),
               "tree-cut words");
    cuda_check(cudaStreamSynchronize(s), "sync");
}

void tree_cut_sync(nbvh_handle *h, cudaStream_t s)
{
    TreeCutSession &c = h->cut;
    uint32_t words[kCutWords + kNumBvhLods];
    tree_cut_words(h, words, s);
    require(words[kCutError] == 0u, NBVH_EOVERFLOW, "tree cut outgrew the classic BVH");
    if (!c.dirty)
        return;
    const uint32_t n = words[kCutCount];
    h->neural_nodes.resize(n);
    cuda_check(cudaMemcpy(h->neural_nodes.data(), h->d_neural_nodes.ptr, (size_t)n * sizeof(BVHNode),
                          cudaMemcpyDeviceToHost),
               "download neural nodes");
    upload_inference_nodes(h);
    c.dirty = false;
}

} // namespace nbvh

extern "C" {

nbvh_status nbvh_tree_cut_options_default(nbvh_tree_cut_options *o)
{
    if (!o)
        return NBVH_EINVAL;
    std::memset(o, 0, sizeof(*o));
    o->tree_cut_learning = 1;
    o->splitting_interval = 50;
    o->last_split_iteration = 2000;
    o->start_split_num = 1;
    o->split_scaling = 2.0f;
    o->split_interval_scaling = 2.0f;
    o->num_lods_learned = 1;
    o->lod_decision_type = 0;
    o->training_node_survival = 1;
    o->survival_probability_scale = 1.0f;
    o->min_rr_survival_prob = 0.005f;
    return NBVH_OK;
}

nbvh_status nbvh_split_schedule_host(const nbvh_tree_cut_options *o, uint32_t start_nodes, uint32_t n_iterations,
                                     uint32_t *h_splits, uint32_t *expected_nodes)
{
    if (!o || start_nodes == 0)
        return NBVH_EINVAL;
    try {
        nbvh::validate_tree_cut_options(*o);
        nbvh::SplitScheduler sched;
        sched.configure(*o);
        const uint32_t nodes = sched.expected(start_nodes, n_iterations, h_splits);
        if (expected_nodes)
            *expected_nodes = nodes;
        return NBVH_OK;
    } catch (const nbvh::Fail &e) {
        return e.status;
    } catch (...) {
        return NBVH_EINVAL;
    }
}

} // extern "C"
