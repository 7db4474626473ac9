// nbvh_scene.cpp -- instanced scenes: several neural BLAS placed by affine transforms, queried and
// path traced together.
//
// The reference renders one neural BLAS per scene and pre-transforms vertices instead of
// instancing (src/cuda/neural/neural_bvh_renderer_init.cu:23-25, src/base/scene.cpp:38-44,225-226);
// its TLAS (include/cuda/accel/tlas.cuh:123-324) walks BLAS roots. Here each bounce (or query)
// tests its rays against every instance's world box, lists for each model the (ray, instance)
// pairs whose ray enters one of its instances, answers each model's list with one neural query in
// object space, and keeps the closest hit per ray in world space (k_path.cu: k_inst_*). Scenes
// hold a few tens of instances, so the box tests are a flat loop rather than a tree.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>

#include "nbvh_internal.h"

using namespace nbvh;

namespace {

struct ModelContext {
    QueryContext q;
    DeviceBuffer<QueryCounters> counters;
};

} // namespace

struct nbvh_scene {
    std::mutex mu;
    std::string last_error;
    int device = 0;
    struct Instance {
        nbvh_handle *model;
        InstanceArgs args;
    };
    std::vector<Instance> instances;
    std::map<const nbvh_handle *, std::unique_ptr<ModelContext>> contexts;
    DeviceBuffer<nbvh_ray> obj_rays;
    DeviceBuffer<uint32_t> obj_ids;
    DeviceBuffer<float> obj_scale;
    DeviceBuffer<nbvh_neural_hit> obj_hits;
    DeviceBuffer<uint32_t> count;
    DeviceBuffer<nbvh_neural_hit> bounce_hits;
    DeviceBuffer<uint32_t> obj_inst;
    DeviceBuffer<unsigned long long> keys;
    // instances grouped by model (one query per model and bounce), and all instances by id
    struct Group {
        nbvh_handle *model;
        DeviceBuffer<InstanceArgs> args;
        uint32_t n = 0;
    };
    std::vector<std::unique_ptr<Group>> groups;
    DeviceBuffer<InstanceArgs> all_args;
    bool groups_dirty = true;
    size_t obj_capacity = 0;
    uint32_t *h_count = nullptr;
    QueryContext unused_q; // render_path_core takes a context; the scene's query brings its own
    PathBuffers path;
    ~nbvh_scene()
    {
        if (h_count)
            cudaFreeHost(h_count);
    }
};

namespace {

template <typename F>
nbvh_status scene_guarded(nbvh_scene *sc, F &&f)
{
    if (!sc)
        return NBVH_EINVAL;
    std::lock_guard<std::mutex> lock(sc->mu);
    try {
        cuda_check(cudaSetDevice(sc->device), "cudaSetDevice");
        f();
        sc->last_error.clear();
        return NBVH_OK;
    } catch (const Fail &e) {
        sc->last_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        sc->last_error = "host allocation failed";
        return NBVH_ENOMEM;
    } catch (const std::exception &e) {
        sc->last_error = e.what();
        return NBVH_EINVAL;
    }
}

void ensure_object_capacity(nbvh_scene *sc, size_t m)
{
    if (sc->obj_capacity >= m)
        return;
    cuda_check(sc->obj_rays.resize(m), "alloc object rays");
    cuda_check(sc->obj_ids.resize(m), "alloc object ids");
    cuda_check(sc->obj_scale.resize(m), "alloc object scales");
    cuda_check(sc->obj_hits.resize(m), "alloc object hits");
    cuda_check(sc->obj_inst.resize(m), "alloc object instances");
    sc->obj_capacity = m;
}

void ensure_scene_buffers(nbvh_scene *sc, uint32_t n)
{
    ensure_object_capacity(sc, n);
    if (sc->keys.count < n)
        cuda_check(sc->keys.resize(n), "alloc keys");
    if (sc->count.count < 1u)
        cuda_check(sc->count.resize(1u), "alloc count");
    if (!sc->h_count)
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&sc->h_count), sizeof(uint32_t), cudaHostAllocDefault),
                   "pinned count");
}

ModelContext &context_of(nbvh_scene *sc, nbvh_handle *model, uint32_t n)
{
    auto &slot = sc->contexts[model];
    if (!slot) {
        slot.reset(new ModelContext());
        cuda_check(slot->counters.resize(1u), "alloc counters");
    }
    grow_query_context(model, slot->q, n);
    return *slot;
}

void upload_groups(nbvh_scene *sc)
{
    if (!sc->groups_dirty)
        return;
    sc->groups.clear();
    std::vector<InstanceArgs> all;
    std::map<nbvh_handle *, std::vector<InstanceArgs>> by_model;
    std::vector<nbvh_handle *> order;
    for (const auto &inst : sc->instances) {
        all.push_back(inst.args);
        if (!by_model.count(inst.model))
            order.push_back(inst.model);
        by_model[inst.model].push_back(inst.args);
    }
    cuda_check(sc->all_args.resize(all.size()), "alloc instances");
    cuda_check(cudaMemcpy(sc->all_args.ptr, all.data(), all.size() * sizeof(InstanceArgs), cudaMemcpyHostToDevice),
               "upload instances");
    for (nbvh_handle *m : order) {
        std::unique_ptr<nbvh_scene::Group> g(new nbvh_scene::Group());
        g->model = m;
        const auto &v = by_model[m];
        g->n = (uint32_t)v.size();
        cuda_check(g->args.resize(v.size()), "alloc instance group");
        cuda_check(cudaMemcpy(g->args.ptr, v.data(), v.size() * sizeof(InstanceArgs), cudaMemcpyHostToDevice),
                   "upload instance group");
        sc->groups.push_back(std::move(g));
    }
    sc->groups_dirty = false;
}

// Closest hit over all instances for n world rays (device buffers); the record's `reserved` word
// is the instance that gave it (~0: none). Per model, every (ray, instance) pair whose ray enters
// the instance's world box is listed and the whole list answered by one query of the model; the
// closest entry per ray wins.
void scene_query(nbvh_scene *sc, const nbvh_ray *d_rays, uint32_t n, uint32_t depth, nbvh_neural_hit *d_hits,
                 cudaStream_t s)
{
    ensure_scene_buffers(sc, n);
    upload_groups(sc);
    cuda_check(launch_inst_reset(sc->keys.ptr, d_hits, n, s), "reset records");
    std::vector<uint32_t> start(sc->groups.size() + 1u, 0u);
    for (int attempt = 0; attempt < 2; attempt++) {
        cuda_check(cudaMemsetAsync(sc->count.ptr, 0, sizeof(uint32_t), s), "reset count");
        for (size_t gi = 0; gi < sc->groups.size(); gi++) {
            const auto &g = *sc->groups[gi];
            cuda_check(launch_inst_group(g.args.ptr, g.n, d_rays, n, sc->obj_rays.ptr, sc->obj_ids.ptr,
                                         sc->obj_scale.ptr, sc->obj_inst.ptr, sc->count.ptr,
                                         (uint32_t)sc->obj_capacity, s),
                       "instance rays");
            cuda_check(cudaMemcpyAsync(sc->h_count, sc->count.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                       "count");
            cuda_check(cudaStreamSynchronize(s), "sync");
            start[gi + 1u] = *sc->h_count;
        }
        if (start.back() <= sc->obj_capacity)
            break;
        // more (ray, instance) pairs than room (the kernel wrote only what fits): grow, list again
        ensure_object_capacity(sc, (size_t)start.back() + start.back() / 4u);
    }
    for (size_t gi = 0; gi < sc->groups.size(); gi++) {
        const uint32_t m = start[gi + 1u] - start[gi];
        if (m == 0)
            continue;
        nbvh_handle *model = sc->groups[gi]->model;
        ModelContext &mc = context_of(sc, model, m);
        run_neural_query(model, mc.q, mc.counters.ptr, sc->obj_rays.ptr + start[gi], m, depth, false,
                         sc->obj_hits.ptr + start[gi], s);
    }
    cuda_check(launch_inst_vote_finalize(sc->all_args.ptr, sc->obj_hits.ptr, sc->obj_ids.ptr, sc->obj_scale.ptr,
                                         sc->obj_inst.ptr, start.back(), sc->keys.ptr, d_hits, n, s),
               "closest instance hits");
}

struct SceneBounceQuery : PathQuery {
    nbvh_scene *sc;
    cudaStream_t s;
    const nbvh_neural_hit *operator()(const nbvh_ray *rays, uint32_t n, uint32_t depth) override
    {
        if (sc->bounce_hits.count < n)
            cuda_check(sc->bounce_hits.resize(n), "alloc bounce records");
        scene_query(sc, rays, n, depth, sc->bounce_hits.ptr, s);
        return sc->bounce_hits.ptr;
    }
};

bool invert3(const double a[9], double inv[9])
{
    const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
    const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    if (!(std::fabs(det) > 1e-20) || !std::isfinite(det))
        return false;
    const double r = 1.0 / det;
    inv[0] = c00 * r;
    inv[1] = (a[2] * a[7] - a[1] * a[8]) * r;
    inv[2] = (a[1] * a[5] - a[2] * a[4]) * r;
    inv[3] = c01 * r;
    inv[4] = (a[0] * a[8] - a[2] * a[6]) * r;
    inv[5] = (a[2] * a[3] - a[0] * a[5]) * r;
    inv[6] = c02 * r;
    inv[7] = (a[1] * a[6] - a[0] * a[7]) * r;
    inv[8] = (a[0] * a[4] - a[1] * a[3]) * r;
    return true;
}

} // namespace

extern "C" {

nbvh_status nbvh_scene_create(int device, nbvh_scene **out)
{
    if (!out)
        return NBVH_EINVAL;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return NBVH_EDEVICE;
    }
    nbvh_scene *sc = new (std::nothrow) nbvh_scene();
    if (!sc)
        return NBVH_ENOMEM;
    sc->device = device;
    *out = sc;
    return NBVH_OK;
}

nbvh_status nbvh_scene_destroy(nbvh_scene *sc)
{
    if (!sc)
        return NBVH_EINVAL;
    cudaSetDevice(sc->device);
    cudaDeviceSynchronize();
    delete sc;
    return NBVH_OK;
}

const char *nbvh_scene_last_error(const nbvh_scene *sc) { return sc ? sc->last_error.c_str() : "null scene"; }

nbvh_status nbvh_scene_add_instance(nbvh_scene *sc, nbvh_handle *model, const float *object_to_world,
                                    uint32_t *instance_id)
{
    return scene_guarded(sc, [&]() {
        require(model && object_to_world && instance_id, NBVH_EINVAL, "null argument");
        require(model->device == sc->device, NBVH_EINVAL, "model lives on another device");
        require(model->classic_built && model->neural_built, NBVH_ESTATE, "model scene not built");
        InstanceArgs a{};
        std::memcpy(a.xform, object_to_world, sizeof(a.xform));
        const double A[9] = {a.xform[0], a.xform[1], a.xform[2], a.xform[4], a.xform[5],
                             a.xform[6], a.xform[8], a.xform[9], a.xform[10]};
        double inv[9];
        require(invert3(A, inv), NBVH_EINVAL, "transform is not invertible");
        for (int k = 0; k < 9; k++)
            a.inv[k] = (float)inv[k];
        const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
        a.identity = std::memcmp(a.xform, id, sizeof(id)) == 0 ? 1u : 0u;
        // world box: the eight corners of the model's scene box
        for (int k = 0; k < 3; k++) {
            a.box_min[k] = FLT_MAX;
            a.box_max[k] = -FLT_MAX;
        }
        for (int c = 0; c < 8; c++) {
            const float p[3] = {(c & 1) ? model->scene_max[0] : model->scene_min[0],
                                (c & 2) ? model->scene_max[1] : model->scene_min[1],
                                (c & 4) ? model->scene_max[2] : model->scene_min[2]};
            for (int row = 0; row < 3; row++) {
                const double w = (double)a.xform[4 * row] * p[0] + (double)a.xform[4 * row + 1] * p[1] +
                                 (double)a.xform[4 * row + 2] * p[2] + (double)a.xform[4 * row + 3];
                a.box_min[row] = std::fmin(a.box_min[row], (float)w);
                a.box_max[row] = std::fmax(a.box_max[row], (float)w);
            }
        }
        // conservative by a relative 1e-5 of the extent against rounding of the corners
        for (int k = 0; k < 3; k++) {
            const float pad = 1e-5f * (a.box_max[k] - a.box_min[k]) + 1e-6f;
            a.box_min[k] -= pad;
            a.box_max[k] += pad;
        }
        a.instance = (uint32_t)sc->instances.size();
        sc->instances.push_back({model, a});
        sc->groups_dirty = true;
        *instance_id = a.instance;
    });
}

nbvh_status nbvh_scene_query_closest(nbvh_scene *sc, const nbvh_ray *d_rays, uint32_t n, uint32_t depth,
                                     nbvh_neural_hit *d_hits, nbvh_stream stream)
{
    return scene_guarded(sc, [&]() {
        require((d_rays && d_hits) || n == 0, NBVH_EINVAL, "null buffers");
        require(!sc->instances.empty(), NBVH_ESTATE, "scene has no instances");
        if (n == 0)
            return;
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        scene_query(sc, d_rays, n, depth, d_hits, s);
        cuda_check(cudaStreamSynchronize(s), "sync");
    });
}

nbvh_status nbvh_scene_render_path(nbvh_scene *sc, const nbvh_path_request *req, float *d_image,
                                   uint64_t *rays_traced, nbvh_stream stream)
{
    return scene_guarded(sc, [&]() {
        require(req && d_image, NBVH_EINVAL, "null request or image");
        require(!sc->instances.empty(), NBVH_ESTATE, "scene has no instances");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        SceneBounceQuery q;
        q.sc = sc;
        q.s = s;
        const uint64_t traced =
            render_path_core(sc->instances[0].model, sc->unused_q, nullptr, sc->path, req, d_image, s,
                             req->camera.sample_idx * req->spp, &q);
        if (rays_traced)
            *rays_traced = traced;
    });
}

} // extern "C"
