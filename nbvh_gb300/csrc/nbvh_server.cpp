// nbvh_server.cpp -- serving loop: many clients' ray-query and render requests of uneven size
// against several resident N-BVH models on one GPU (the reference renders one model in one
// process and has nothing like it; this is the serving form of its neural query).
//
//  * Slots. n_slots worker threads, each with its own CUDA stream, query context, ray / hit /
//    image buffers and path-tracing buffers, sized once from the HBM budget (admission: a request
//    is admitted when a slot is free; a slot's share of the budget bounds what it holds).
//  * Continuous batching. A free slot takes the oldest pending query work, else the oldest pending
//    render work; pending query requests for the same model and depth are merged into one batch up
//    to the slot's capacity (larger requests are split into chunks, each a batch of its own).
//    Requests that arrive while others run are taken by the next slot that frees up, so batches of
//    different requests overlap on the device.
//  * Query lane. query_slots of the slots take query requests only and launch on streams of the
//    device's highest priority (the others on its lowest), so a latency-bound query batch neither
//    waits for a slot behind long renders nor queues behind their kernels for SMs: the block
//    scheduler starts its blocks first as resident ones finish. While the lane runs a batch, the
//    render slots hold back their next bounce query (for at most kYieldMs), so the lane's kernels
//    meet only the render work already on the device.
//  * Graphs. A query batch is padded to a power-of-two bucket; the first part of its query (the
//    first-leaf pass and the first steps) is captured once per (slot, model, bucket) as a CUDA graph
//    and replayed; the host then checks the list length and finishes any remaining steps directly.
//  * Autotuning. When a model is added, each bucket's launch parameters (node visits per traversal
//    round, encoder blocks per SM) are chosen by timing the candidates on rays through the model's
//    scene box.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <random>
#include <thread>
#include <vector>

#include "nbvh_internal.h"

using namespace nbvh;

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t kMinBucket = 1u << 12;
constexpr uint32_t kGraphSteps = 8;          // steps inside the captured graph
constexpr uint64_t kBytesPerRay = 1024;      // query + path buffers per ray of slot capacity (upper bound)
constexpr int kYieldMs = 20;                 // longest a render bounce waits for the query lane

struct Tuning {
    uint32_t visits = 0, encode_blocks = 0;
    bool stage_cut = false;
};

struct Model {
    nbvh_handle *h = nullptr;
    std::map<uint32_t, Tuning> tune; // by bucket
};

struct Request {
    uint64_t ticket = 0;
    nbvh_request req{};
    Clock::time_point submitted, started, done_at;
    uint32_t chunks = 0, chunks_done = 0;
    nbvh_status status = NBVH_OK;
    uint64_t rays_traced = 0;
    bool done = false;
    std::vector<float> accum; // render split over spp: summed chunk images
    std::mutex accum_mu;      // guards accum (not the server's lock: summing an image takes a while)
};

struct Work {
    std::shared_ptr<Request> r;
    uint32_t offset = 0, count = 0; // query: ray range; render: spp range
};

struct GraphKey {
    uint32_t model, bucket, depth;
    bool operator<(const GraphKey &o) const
    {
        return model != o.model ? model < o.model : bucket != o.bucket ? bucket < o.bucket : depth < o.depth;
    }
};

struct Slot {
    cudaStream_t stream = nullptr;
    bool query_only = false; // a slot of the query lane
    QueryContext q;
    DeviceBuffer<QueryCounters> counters;
    DeviceBuffer<nbvh_ray> rays;
    DeviceBuffer<nbvh_neural_hit> hits;
    DeviceBuffer<float> image;
    PathBuffers path;
    uint32_t capacity = 0;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::map<uint32_t, uint64_t> model_versions; // model_version of each model when its graphs were made
    std::thread thread;
    ~Slot()
    {
        for (auto &g : graphs)
            if (g.second)
                cudaGraphExecDestroy(g.second);
        if (stream)
            cudaStreamDestroy(stream);
    }
};

uint32_t bucket_of(uint32_t n)
{
    uint32_t b = kMinBucket;
    while (b < n)
        b <<= 1;
    return b;
}

// Rays that cannot hit anything (far outside every scene, pointing away): padding of a bucket.
void fill_dead_rays(nbvh_ray *h, uint32_t n)
{
    for (uint32_t i = 0; i < n; i++)
        h[i] = nbvh_ray{{1e30f, 1e30f, 1e30f}, 1e-4f, {1.f, 0.f, 0.f}, 0.f};
}

} // namespace

struct nbvh_server {
    nbvh_server_config cfg{};
    int device = 0;
    int num_sms = 0;
    std::vector<Model> models;
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Work> pending;
    std::map<uint64_t, std::shared_ptr<Request>> requests;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::string last_error;
    // statistics
    std::vector<double> latencies_ms;
    uint64_t rays_traced = 0, batches = 0, merged = 0, requests_done = 0, graphs_captured = 0, graph_replays = 0;
    Clock::time_point first_submit, last_done;
    bool any_submit = false;
    nbvh_ray *dead = nullptr; // device buffer of padding rays (max bucket)
    uint32_t idle_query_slots = 0; // query-lane slots waiting for work (guarded by mu)
    // query-lane batches on the device; render bounces wait for 0 (guarded by lane_mu)
    std::mutex lane_mu;
    std::condition_variable lane_cv;
    uint32_t lane_busy = 0;
};

namespace {

template <typename F>
nbvh_status server_guarded(nbvh_server *s, F &&f)
{
    if (!s)
        return NBVH_EINVAL;
    try {
        cuda_check(cudaSetDevice(s->device), "cudaSetDevice");
        f();
        return NBVH_OK;
    } catch (const Fail &e) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->last_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        return NBVH_ENOMEM;
    } catch (const std::exception &e) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->last_error = e.what();
        return NBVH_EINVAL;
    }
}

bool graphable(const nbvh_server *srv, const nbvh_handle *h)
{
    return srv->cfg.use_graphs && !h->cfg.bvh.ignore_neural_blas && !h->any_non_neural && h->cfg.fallback_margin <= 0.f;
}

StepResources tuning_of(const Model &m, uint32_t bucket)
{
    StepResources t;
    auto it = m.tune.find(bucket);
    if (it != m.tune.end()) {
        t.visits_per_round = it->second.visits;
        t.encode_blocks_per_sm = it->second.encode_blocks;
        t.stage_cut = it->second.stage_cut;
    }
    return t;
}

// Captures (once) the graph of a padded batch of `bucket` rays in the slot's buffers: the first-leaf
// pass and the first kGraphSteps steps, ending with a copy of the wave counters to the host. Nothing
// runs; the kernels' attributes are set beforehand (a captured launch cannot set them). A shape
// whose capture fails is recorded without a graph and keeps running directly.
cudaGraphExec_t ensure_graph(nbvh_server *srv, Slot &sl, uint32_t model_id, uint32_t bucket, uint32_t depth)
{
    const GraphKey key{model_id, bucket, depth};
    auto g = sl.graphs.find(key);
    if (g != sl.graphs.end())
        return g->second;
    const Model &m = srv->models[model_id];
    StepResources cap = tuning_of(m, bucket);
    cap.unchecked_steps = kGraphSteps;
    cap.capture_only = true;
    cudaGraphExec_t exec = nullptr;
    // the captured launches cannot set kernel attributes: set those of every variant first
    cuda_check(configure_query_kernels(), "kernel attributes");
    if (cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
        bool ok = true;
        try {
            run_neural_query(m.h, sl.q, sl.counters.ptr, sl.rays.ptr, bucket, depth, false, sl.hits.ptr, sl.stream, &cap);
        } catch (...) {
            ok = false;
        }
        cudaGraph_t graph = nullptr;
        ok = cudaStreamEndCapture(sl.stream, &graph) == cudaSuccess && ok && graph != nullptr;
        if (ok && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
            exec = nullptr;
        if (graph)
            cudaGraphDestroy(graph);
    }
    cudaGetLastError(); // a failed capture leaves no sticky error; clear the last one
    sl.graphs.emplace(key, exec);
    if (exec) {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->graphs_captured++;
    }
    return exec;
}

// Runs the neural query of a batch of n rays already in the slot's ray buffer: padded to its
// bucket, the captured graph replayed (when graphs are on), then the host-checked remainder.
void slot_query(nbvh_server *srv, Slot &sl, uint32_t model_id, uint32_t n, uint32_t depth)
{
    const Model &m = srv->models[model_id];
    const uint32_t bucket = std::min(bucket_of(n), sl.capacity);
    if (bucket > n) // pad the batch with rays that miss everything
        cuda_check(cudaMemcpyAsync(sl.rays.ptr + n, srv->dead, (size_t)(bucket - n) * sizeof(nbvh_ray),
                                   cudaMemcpyDeviceToDevice, sl.stream),
                   "pad batch");
    const StepResources tune = tuning_of(m, bucket);
    nbvh_handle *h = m.h;
    // a model whose device arrays were reallocated since its graphs were captured (a new cut, a
    // grown learned cut, a new mesh) drops them; the context is resized for the new cut first
    auto ver = sl.model_versions.find(model_id);
    if (ver == sl.model_versions.end()) {
        sl.model_versions[model_id] = h->model_version;
    } else if (ver->second != h->model_version) {
        const uint64_t gen = sl.q.generation;
        grow_query_context(h, sl.q, sl.capacity);
        for (auto g = sl.graphs.begin(); g != sl.graphs.end();) {
            if (sl.q.generation != gen || g->first.model == model_id) {
                if (g->second)
                    cudaGraphExecDestroy(g->second);
                g = sl.graphs.erase(g);
            } else {
                ++g;
            }
        }
        ver->second = h->model_version;
    }
    cudaGraphExec_t exec = graphable(srv, h) ? ensure_graph(srv, sl, model_id, bucket, depth) : nullptr;
    if (!exec) {
        run_neural_query(h, sl.q, sl.counters.ptr, sl.rays.ptr, bucket, depth, false, sl.hits.ptr, sl.stream, &tune);
        return;
    }
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->graph_replays++;
    }
    cuda_check(cudaGraphLaunch(exec, sl.stream), "graph launch");
    cuda_check(cudaStreamSynchronize(sl.stream), "graph sync");
    if (sl.q.h_words[3] != 0u)
        fail(NBVH_ETIMEOUT, "tensor-core MLP: a bounded wait gave up");
    if (sl.q.h_words[kGraphSteps % 3u] == 0u)
        return; // the list of the first step after the graph is empty: done
    StepResources rest = tune;
    rest.resume_from = kGraphSteps;
    run_neural_query(h, sl.q, sl.counters.ptr, sl.rays.ptr, bucket, depth, false, sl.hits.ptr, sl.stream, &rest);
}

// The path tracer's per-bounce query on a slot: the bounce's rays are copied into the slot's ray
// buffer and answered like a query batch (bucket, graph), the hits read from the slot's hit buffer.
struct SlotPathQuery : PathQuery {
    nbvh_server *srv;
    Slot *sl;
    uint32_t model;
    SlotPathQuery(nbvh_server *s, Slot *l, uint32_t m) : srv(s), sl(l), model(m) {}
    const nbvh_neural_hit *operator()(const nbvh_ray *rays, uint32_t n, uint32_t depth) override
    {
        if (srv->cfg.query_slots > 0u && !sl->query_only) { // yield to a query-lane batch in flight
            std::unique_lock<std::mutex> lock(srv->lane_mu);
            srv->lane_cv.wait_for(lock, std::chrono::milliseconds(kYieldMs), [&] { return srv->lane_busy == 0u; });
        }
        cuda_check(cudaMemcpyAsync(sl->rays.ptr, rays, (size_t)n * sizeof(nbvh_ray), cudaMemcpyDeviceToDevice,
                                   sl->stream),
                   "bounce rays");
        slot_query(srv, *sl, model, n, depth);
        return sl->hits.ptr;
    }
};

void complete(nbvh_server *srv, const Work &w, nbvh_status st, uint64_t traced)
{
    Request &r = *w.r;
    bool last;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        if (st != NBVH_OK)
            r.status = st;
        r.rays_traced += traced;
        srv->rays_traced += traced;
        last = ++r.chunks_done == r.chunks;
    }
    if (!last)
        return;
    // every chunk is done: nothing else touches the request's image until it is marked done, so the
    // average is formed without the server's lock (which the slots need to take new work)
    if (r.req.kind == NBVH_REQUEST_RENDER && r.status == NBVH_OK && r.chunks > 1u) {
        const uint32_t px = r.req.render.camera.width * r.req.render.camera.height;
        const float inv = 1.0f / (float)r.req.render.spp;
        for (size_t i = 0; i < (size_t)px * 4u; i++)
            r.req.h_image[i] = (i % 4u == 3u) ? 1.0f : r.accum[i] * inv;
        r.accum.clear();
        r.accum.shrink_to_fit();
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    r.done = true;
    r.done_at = Clock::now();
    srv->last_done = r.done_at;
    srv->requests_done++;
    srv->latencies_ms.push_back(std::chrono::duration<double, std::milli>(r.done_at - r.submitted).count());
    srv->cv_done.notify_all();
}

// Marks a query-lane batch as on the device for its lifetime (render bounces wait meanwhile).
struct LaneBusy {
    nbvh_server *srv;
    bool on;
    LaneBusy(nbvh_server *s, bool lane) : srv(s), on(lane)
    {
        if (on) {
            std::lock_guard<std::mutex> lock(srv->lane_mu);
            srv->lane_busy++;
        }
    }
    ~LaneBusy()
    {
        if (on) {
            {
                std::lock_guard<std::mutex> lock(srv->lane_mu);
                srv->lane_busy--;
            }
            srv->lane_cv.notify_all();
        }
    }
};

void run_batch(nbvh_server *srv, Slot &sl, std::vector<Work> &batch)
{
    const nbvh_request &q0 = batch[0].r->req;
    const LaneBusy busy(srv, sl.query_only && q0.kind == NBVH_REQUEST_QUERY);
    try {
        cuda_check(cudaSetDevice(srv->device), "cudaSetDevice");
        if (q0.kind == NBVH_REQUEST_QUERY) {
            uint32_t n = 0;
            for (auto &w : batch) {
                cuda_check(cudaMemcpyAsync(sl.rays.ptr + n, w.r->req.h_rays + w.offset, (size_t)w.count * sizeof(nbvh_ray),
                                           cudaMemcpyHostToDevice, sl.stream),
                           "rays in");
                n += w.count;
            }
            slot_query(srv, sl, q0.model, n, q0.depth ? q0.depth : 1u);
            n = 0;
            for (auto &w : batch) {
                cuda_check(cudaMemcpyAsync(w.r->req.h_hits + w.offset, sl.hits.ptr + n,
                                           (size_t)w.count * sizeof(nbvh_neural_hit), cudaMemcpyDeviceToHost, sl.stream),
                           "hits out");
                n += w.count;
            }
            cuda_check(cudaStreamSynchronize(sl.stream), "sync");
            for (auto &w : batch)
                complete(srv, w, NBVH_OK, w.count);
        } else {
            Work &w = batch[0];
            nbvh_path_request pr = q0.render;
            // samples [offset, offset + count) of the frame: the same paths the whole frame would trace
            pr.spp = w.count;
            const uint32_t px = pr.camera.width * pr.camera.height;
            SlotPathQuery pq(srv, &sl, q0.model);
            const uint64_t traced =
                render_path_core(srv->models[q0.model].h, sl.q, sl.counters.ptr, sl.path, &pr, sl.image.ptr, sl.stream,
                                 q0.render.camera.sample_idx * q0.render.spp + w.offset, &pq);
            if (w.r->chunks == 1u) { // the whole frame: its image as it is
                cuda_check(cudaMemcpy(q0.h_image, sl.image.ptr, (size_t)px * 4u * sizeof(float), cudaMemcpyDeviceToHost),
                           "image out");
            } else {
                std::vector<float> img((size_t)px * 4u);
                cuda_check(cudaMemcpy(img.data(), sl.image.ptr, img.size() * sizeof(float), cudaMemcpyDeviceToHost),
                           "image out");
                Request &r = *w.r;
                std::lock_guard<std::mutex> lock(r.accum_mu);
                for (size_t i = 0; i < img.size(); i++)
                    r.accum[i] += img[i] * (float)w.count; // chunk mean x chunk samples
            }
            complete(srv, w, NBVH_OK, traced);
        }
    } catch (const Fail &e) {
        {
            std::lock_guard<std::mutex> lock(srv->mu);
            srv->last_error = e.msg;
        }
        cudaStreamSynchronize(sl.stream);
        for (auto &w : batch)
            complete(srv, w, e.status, 0);
    } catch (...) {
        cudaStreamSynchronize(sl.stream);
        for (auto &w : batch)
            complete(srv, w, NBVH_EDEVICE, 0);
    }
}

// The pending work a slot takes next: the oldest query work, else (for a slot outside the query
// lane) the oldest work of any kind; end() when there is none for it. While a slot of the query lane
// is idle, the other slots leave query work to it (it runs at the higher stream priority).
std::deque<Work>::iterator next_work(nbvh_server *srv, const Slot &sl)
{
    const bool take_queries = sl.query_only || srv->idle_query_slots == 0u;
    std::deque<Work>::iterator first_render = srv->pending.end();
    for (auto it = srv->pending.begin(); it != srv->pending.end(); ++it) {
        if (it->r->req.kind == NBVH_REQUEST_QUERY) {
            if (take_queries)
                return it;
        } else if (first_render == srv->pending.end()) {
            first_render = it;
        }
    }
    return sl.query_only ? srv->pending.end() : first_render;
}

void slot_loop(nbvh_server *srv, Slot *sl)
{
    cudaSetDevice(srv->device);
    for (;;) {
        std::vector<Work> batch;
        {
            std::unique_lock<std::mutex> lock(srv->mu);
            if (sl->query_only)
                srv->idle_query_slots++;
            srv->cv_work.wait(lock, [&] { return srv->stop || next_work(srv, *sl) != srv->pending.end(); });
            if (sl->query_only)
                srv->idle_query_slots--;
            const auto pick = next_work(srv, *sl);
            if (pick == srv->pending.end())
                return; // stopping, and nothing left that this slot takes
            Work first = *pick;
            srv->pending.erase(pick);
            if (sl->query_only && !srv->pending.empty())
                srv->cv_work.notify_all(); // the lane is busy now: the other slots may take queries
            if (first.r->chunks_done == 0 && first.offset == 0)
                first.r->started = Clock::now();
            batch.push_back(first);
            if (first.r->req.kind == NBVH_REQUEST_QUERY) {
                // merge later query work for the same model and depth while it fits the slot
                uint32_t total = first.count;
                for (auto it = srv->pending.begin(); it != srv->pending.end();) {
                    const nbvh_request &q = it->r->req;
                    if (q.kind == NBVH_REQUEST_QUERY && q.model == first.r->req.model && q.depth == first.r->req.depth &&
                        total + it->count <= sl->capacity) {
                        total += it->count;
                        batch.push_back(*it);
                        it = srv->pending.erase(it);
                    } else {
                        ++it;
                    }
                }
                srv->merged += batch.size() - 1u;
            }
            srv->batches++;
        }
        run_batch(srv, *sl, batch);
    }
}

// Chooses, per bucket, the node visits per traversal round, the encoder blocks per SM and the cut
// variant of the decode and tail kernels (staged in shared memory or read through L1) that give
// the shortest query on rays through the model's scene box (CUDA events on slot 0's stream).
void autotune(nbvh_server *srv, uint32_t model_id)
{
    Slot &sl = *srv->slots[0];
    Model &m = srv->models[model_id];
    const nbvh_handle *h = m.h;
    const float *lo = h->scene_min, *hi = h->scene_max;
    std::mt19937 rng(1234u + model_id);
    std::uniform_real_distribution<float> u(0.f, 1.f);
    std::vector<nbvh_ray> host(sl.capacity);
    for (auto &r : host) {
        for (int k = 0; k < 3; k++) {
            const float c = 0.5f * (lo[k] + hi[k]), e = 0.75f * (hi[k] - lo[k]);
            r.o[k] = c + (2.f * u(rng) - 1.f) * e;
        }
        const float z = 2.f * u(rng) - 1.f, a = 6.2831853f * u(rng), rr = std::sqrt(std::max(0.f, 1.f - z * z));
        r.d[0] = rr * std::cos(a);
        r.d[1] = rr * std::sin(a);
        r.d[2] = z;
        r.tmin = 1e-4f;
        r.tmax = 3.4028234663852886e38f;
    }
    cuda_check(cudaMemcpy(sl.rays.ptr, host.data(), host.size() * sizeof(nbvh_ray), cudaMemcpyHostToDevice), "tune rays");
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    const uint32_t visits[3] = {8u, 12u, 16u}, enc[2] = {3u, 4u};
    for (uint32_t b = kMinBucket; b <= sl.capacity; b <<= 2) {
        float best = 1e30f;
        Tuning pick;
        for (uint32_t v : visits)
            for (uint32_t eb : enc)
                for (bool stage : {false, true}) {
                    StepResources t;
                    t.visits_per_round = v;
                    t.encode_blocks_per_sm = eb;
                    t.stage_cut = stage;
                    run_neural_query(h, sl.q, sl.counters.ptr, sl.rays.ptr, b, 1u, false, sl.hits.ptr, sl.stream, &t);
                    float ms_total = 0.f;
                    for (int rep = 0; rep < 2; rep++) {
                        cuda_check(cudaEventRecord(e0, sl.stream), "event");
                        run_neural_query(h, sl.q, sl.counters.ptr, sl.rays.ptr, b, 1u, false, sl.hits.ptr, sl.stream, &t);
                        cuda_check(cudaEventRecord(e1, sl.stream), "event");
                        cuda_check(cudaEventSynchronize(e1), "event sync");
                        float ms = 0.f;
                        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                        ms_total += ms;
                    }
                    if (ms_total < best) {
                        best = ms_total;
                        pick.visits = v;
                        pick.encode_blocks = eb;
                        pick.stage_cut = stage;
                    }
                }
        // buckets between the tuned powers of four take the nearest tuned value below
        m.tune[b] = pick;
        if ((b << 1) <= sl.capacity)
            m.tune[b << 1] = pick;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

} // namespace

extern "C" {

nbvh_status nbvh_server_config_default(nbvh_server_config *cfg)
{
    if (!cfg)
        return NBVH_EINVAL;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->n_slots = 4;
    cfg->max_batch_rays = 1u << 22;
    cfg->hbm_budget_bytes = 150ull << 30;
    cfg->use_graphs = 1;
    cfg->autotune = 1;
    cfg->query_slots = 0;
    return NBVH_OK;
}

nbvh_status nbvh_server_create(const nbvh_server_config *cfg, int device, nbvh_server **out)
{
    if (!cfg || !out || cfg->n_slots == 0 || cfg->n_slots > 64 || cfg->max_batch_rays < kMinBucket ||
        cfg->query_slots >= cfg->n_slots)
        return NBVH_EINVAL;
    auto *srv = new (std::nothrow) nbvh_server();
    if (!srv)
        return NBVH_ENOMEM;
    srv->cfg = *cfg;
    srv->device = device;
    const nbvh_status st = server_guarded(srv, [&]() {
        cuda_check(cudaDeviceGetAttribute(&srv->num_sms, cudaDevAttrMultiProcessorCount, device), "device query");
        // admission by the HBM budget: every slot holds buffers for its capacity, all within budget
        uint64_t per_slot = cfg->hbm_budget_bytes / cfg->n_slots / kBytesPerRay;
        uint32_t cap = (uint32_t)std::min<uint64_t>(per_slot, cfg->max_batch_rays);
        uint32_t pow2 = kMinBucket;
        while ((pow2 << 1) <= cap)
            pow2 <<= 1;
        require(cap >= kMinBucket, NBVH_EINVAL, "HBM budget too small for one minimal batch per slot");
        cap = pow2;
        int least_priority = 0, greatest_priority = 0; // numerically lower = higher priority
        cuda_check(cudaDeviceGetStreamPriorityRange(&least_priority, &greatest_priority), "stream priorities");
        std::vector<nbvh_ray> dead(cap);
        fill_dead_rays(dead.data(), cap);
        cuda_check(cudaMalloc(&srv->dead, (size_t)cap * sizeof(nbvh_ray)), "alloc padding rays");
        cuda_check(cudaMemcpy(srv->dead, dead.data(), dead.size() * sizeof(nbvh_ray), cudaMemcpyHostToDevice), "padding");
        for (uint32_t i = 0; i < cfg->n_slots; i++) {
            auto sl = std::make_unique<Slot>();
            sl->capacity = cap;
            sl->query_only = i < cfg->query_slots;
            const int priority = cfg->query_slots == 0 ? 0 : sl->query_only ? greatest_priority : least_priority;
            cuda_check(cudaStreamCreateWithPriority(&sl->stream, cudaStreamNonBlocking, priority), "stream");
            cuda_check(sl->counters.resize(1u), "alloc counters");
            cuda_check(sl->rays.resize(cap), "alloc slot rays");
            cuda_check(sl->hits.resize(cap), "alloc slot hits");
            cuda_check(sl->image.resize((size_t)cap * 4u), "alloc slot image");
            srv->slots.push_back(std::move(sl));
        }
    });
    if (st != NBVH_OK) {
        if (srv->dead)
            cudaFree(srv->dead);
        delete srv;
        return st;
    }
    *out = srv;
    return NBVH_OK;
}

nbvh_status nbvh_server_add_model(nbvh_server *srv, nbvh_handle *h, uint32_t *model_id)
{
    return server_guarded(srv, [&]() {
        require(h && model_id, NBVH_EINVAL, "null model");
        require(h->classic_built && h->neural_built, NBVH_ESTATE, "model scene not built");
        require(h->device == srv->device, NBVH_EINVAL, "model lives on another device");
        {
            std::lock_guard<std::mutex> lock(srv->mu);
            require(srv->slots.empty() || !srv->slots[0]->thread.joinable(), NBVH_ESTATE,
                    "models must be added before the first request");
        }
        Model m;
        m.h = h;
        srv->models.push_back(m);
        const uint32_t id = (uint32_t)srv->models.size() - 1u;
        // size every slot's query context for this model now, so serving never allocates; a context
        // whose buffers moved drops its captured graphs (they hold the old addresses)
        for (auto &sl : srv->slots) {
            const uint64_t gen = sl->q.generation;
            grow_query_context(h, sl->q, sl->capacity);
            if (sl->q.generation != gen) {
                for (auto &g : sl->graphs)
                    if (g.second)
                        cudaGraphExecDestroy(g.second);
                sl->graphs.clear();
            }
        }
        if (srv->cfg.autotune) {
            autotune(srv, id);
        } else { // one direct query sets the kernels' attributes before any capture
            Slot &s0 = *srv->slots[0];
            cuda_check(cudaMemcpy(s0.rays.ptr, srv->dead, kMinBucket * sizeof(nbvh_ray), cudaMemcpyDeviceToDevice),
                       "warm rays");
            run_neural_query(h, s0.q, s0.counters.ptr, s0.rays.ptr, kMinBucket, 1u, false, s0.hits.ptr, s0.stream);
        }
        // capture every slot's graphs for this model now, so the first requests do not pay for it
        if (graphable(srv, h))
            for (auto &sl : srv->slots)
                for (uint32_t b = kMinBucket; b <= sl->capacity; b <<= 1)
                    for (uint32_t depth = 1; depth <= 2; depth++)
                        ensure_graph(srv, *sl, id, b, depth);
        for (auto &sl : srv->slots)
            sl->model_versions[id] = h->model_version;
        *model_id = id;
    });
}

nbvh_status nbvh_server_submit(nbvh_server *srv, const nbvh_request *req, uint64_t *ticket)
{
    return server_guarded(srv, [&]() {
        require(req && ticket, NBVH_EINVAL, "null request");
        require(req->model < srv->models.size(), NBVH_EINVAL, "unknown model");
        auto r = std::make_shared<Request>();
        r->req = *req;
        r->submitted = Clock::now();
        std::vector<Work> works;
        const uint32_t cap = srv->slots[0]->capacity;
        if (req->kind == NBVH_REQUEST_QUERY) {
            require((req->h_rays && req->h_hits) || req->n_rays == 0, NBVH_EINVAL, "null buffers");
            for (uint32_t off = 0; off < req->n_rays; off += cap)
                works.push_back(Work{r, off, std::min(cap, req->n_rays - off)});
        } else if (req->kind == NBVH_REQUEST_RENDER) {
            const nbvh_path_request &p = req->render;
            require(req->h_image && p.camera.width > 0 && p.camera.height > 0 && p.spp > 0, NBVH_EINVAL, "bad render");
            const uint64_t px = (uint64_t)p.camera.width * p.camera.height;
            require(px <= cap, NBVH_EINVAL, "image larger than a slot's capacity");
            const uint32_t per = (uint32_t)std::max<uint64_t>(1u, cap / px); // samples per chunk
            for (uint32_t off = 0; off < p.spp; off += per)
                works.push_back(Work{r, off, std::min(per, p.spp - off)});
            r->accum.assign((size_t)px * 4u, 0.f);
        } else {
            fail(NBVH_EINVAL, "unknown request kind");
        }
        std::lock_guard<std::mutex> lock(srv->mu);
        r->ticket = srv->next_ticket++;
        r->chunks = (uint32_t)works.size();
        if (!srv->any_submit) {
            srv->any_submit = true;
            srv->first_submit = r->submitted;
        }
        srv->requests[r->ticket] = r;
        if (works.empty()) { // zero rays: done at once
            r->done = true;
            r->done_at = r->submitted;
        }
        for (auto &w : works)
            srv->pending.push_back(w);
        // start the workers on the first request
        for (auto &sl : srv->slots)
            if (!sl->thread.joinable())
                sl->thread = std::thread(slot_loop, srv, sl.get());
        *ticket = r->ticket;
        srv->cv_work.notify_all();
    });
}

nbvh_status nbvh_server_wait(nbvh_server *srv, uint64_t ticket, uint32_t timeout_ms, nbvh_request_result *result)
{
    if (!srv)
        return NBVH_EINVAL;
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->requests.find(ticket);
    if (it == srv->requests.end())
        return NBVH_EINVAL;
    std::shared_ptr<Request> r = it->second;
    if (!srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), [&] { return r->done; }))
        return NBVH_ETIMEOUT;
    if (result) {
        result->status = r->status;
        result->latency_ms = std::chrono::duration<double, std::milli>(r->done_at - r->submitted).count();
        result->queue_ms = r->chunks ? std::chrono::duration<double, std::milli>(r->started - r->submitted).count() : 0.0;
        result->rays_traced = r->rays_traced;
    }
    srv->requests.erase(it);
    return r->status;
}

nbvh_status nbvh_server_get_stats(nbvh_server *srv, nbvh_server_stats *out)
{
    if (!srv || !out)
        return NBVH_EINVAL;
    std::lock_guard<std::mutex> lock(srv->mu);
    std::memset(out, 0, sizeof(*out));
    out->requests_done = srv->requests_done;
    out->rays_traced = srv->rays_traced;
    out->batches = srv->batches;
    out->merged_requests = srv->merged;
    out->slot_capacity_rays = srv->slots.empty() ? 0u : srv->slots[0]->capacity;
    out->graphs_captured = srv->graphs_captured;
    out->graph_replays = srv->graph_replays;
    std::vector<double> l = srv->latencies_ms;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) { return l[std::min(l.size() - 1u, (size_t)(p * (double)(l.size() - 1u) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = l.back();
        double sum = 0.0;
        for (double v : l)
            sum += v;
        out->mean_ms = sum / (double)l.size();
    }
    if (srv->any_submit && srv->requests_done > 0)
        out->busy_seconds = std::chrono::duration<double>(srv->last_done - srv->first_submit).count();
    return NBVH_OK;
}

nbvh_status nbvh_server_reset_stats(nbvh_server *srv)
{
    if (!srv)
        return NBVH_EINVAL;
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->latencies_ms.clear();
    srv->rays_traced = srv->batches = srv->merged = srv->requests_done = srv->graph_replays = 0;
    srv->any_submit = false;
    return NBVH_OK;
}

const char *nbvh_server_last_error(nbvh_server *srv)
{
    if (!srv)
        return "null server";
    std::lock_guard<std::mutex> lock(srv->mu);
    return srv->last_error.c_str();
}

nbvh_status nbvh_server_destroy(nbvh_server *srv)
{
    if (!srv)
        return NBVH_EINVAL;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
        srv->cv_work.notify_all();
    }
    for (auto &sl : srv->slots)
        if (sl->thread.joinable())
            sl->thread.join();
    cudaSetDevice(srv->device);
    srv->slots.clear();
    if (srv->dead)
        cudaFree(srv->dead);
    delete srv;
    return NBVH_OK;
}

} // extern "C"
