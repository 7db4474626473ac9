// bvh_builder.cpp -- host construction of the classic BVH2 and of the fixed neural tree cut.
//
// The reference builds its BLAS with madmann91/bvh v2 DefaultBuilder (Quality::High, leaves of
// 1..2 primitives; src/cuda/cuda_backend.cpp:270-310), converts it to 32-byte BVH2Node records
// whose two children are adjacent (include/base/accel/bvh.h:66-72, src/base/accel/bvh.cpp:133-151)
// and pads flat boxes by 1e-4 (src/cuda/cuda_backend.cpp:212-223). That library is not part of the
// reference tree, so this file is an own binned-SAH builder producing the same node format and
// leaf size. Closest-hit results depend on the topology only through exact distance ties. Meshes
// of 65,536 triangles or more build on several host threads with a result identical to the
// single-threaded build (4M triangles: 7.7 s on one thread, 2.9 s on eight).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr int kBins = 32;
constexpr int kMaxDepth = 31; // the traversal stack has 32 entries
constexpr float kBoxRegularisation = 1e-4f; // BBOX_REGULARISATION, include/cuda/cuda_backend.h:14

struct Box {
    float mn[3], mx[3];
    void reset()
    {
        for (int k = 0; k < 3; k++) {
            mn[k] = INFINITY;
            mx[k] = -INFINITY;
        }
    }
    void grow(const Box &b)
    {
        for (int k = 0; k < 3; k++) {
            mn[k] = std::min(mn[k], b.mn[k]);
            mx[k] = std::max(mx[k], b.mx[k]);
        }
    }
    void grow(const float *p)
    {
        for (int k = 0; k < 3; k++) {
            mn[k] = std::min(mn[k], p[k]);
            mx[k] = std::max(mx[k], p[k]);
        }
    }
    double half_area() const
    {
        double dx = std::max(0.0, (double)mx[0] - mn[0]), dy = std::max(0.0, (double)mx[1] - mn[1]),
               dz = std::max(0.0, (double)mx[2] - mn[2]);
        return dx * dy + dy * dz + dz * dx;
    }
};

struct Prims {
    const std::vector<Box> &boxes;
    const std::vector<float> &centroids; // 3 per primitive
    std::vector<uint32_t> &prims;
};

// Runs f(i) for i in [0, n) on up to `threads` threads (in order on the calling thread for 1).
template <typename F>
void parallel_for(uint32_t n, unsigned threads, F &&f)
{
    if (threads <= 1u || n <= 1u) {
        for (uint32_t i = 0; i < n; i++)
            f(i);
        return;
    }
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        for (uint32_t i = next.fetch_add(1u); i < n; i = next.fetch_add(1u))
            f(i);
    };
    std::vector<std::thread> pool;
    const unsigned m = std::min<unsigned>(threads, n) - 1u;
    for (unsigned k = 0; k < m; k++)
        pool.emplace_back(worker);
    worker();
    for (auto &t : pool)
        t.join();
}

// Node box, centroid box and the 32 SAH bins of every axis (over the centroid box `cb`, for the
// axes where it is not flat) of prims[begin, end). Boxes merge by min / max and bins by sums, so a
// range cut into chunks and merged in any order gives exactly the sequential result.
struct Bins {
    Box bb[3][kBins];
    uint32_t bc[3][kBins];
    void reset()
    {
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < kBins; b++) {
                bb[a][b].reset();
                bc[a][b] = 0;
            }
    }
    void merge(const Bins &o)
    {
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < kBins; b++) {
                bb[a][b].grow(o.bb[a][b]);
                bc[a][b] += o.bc[a][b];
            }
    }
};

void range_bounds(const Prims &P, uint32_t begin, uint32_t end, Box &nb, Box &cb)
{
    nb.reset();
    cb.reset();
    for (uint32_t i = begin; i < end; i++) {
        nb.grow(P.boxes[P.prims[i]]);
        cb.grow(&P.centroids[3u * P.prims[i]]);
    }
}

void bin_range(const Prims &P, uint32_t begin, uint32_t end, const Box &cb, Bins &out)
{
    out.reset();
    for (int axis = 0; axis < 3; axis++) {
        const float lo = cb.mn[axis], hi = cb.mx[axis];
        if (!(hi > lo))
            continue;
        const float scale = (float)kBins / (hi - lo);
        for (uint32_t i = begin; i < end; i++) {
            int b = (int)((P.centroids[3u * P.prims[i] + axis] - lo) * scale);
            b = std::min(std::max(b, 0), kBins - 1);
            out.bb[axis][b].grow(P.boxes[P.prims[i]]);
            out.bc[axis][b]++;
        }
    }
}

// Ranges of at least this many primitives are bounded and binned by several threads.
constexpr uint32_t kParallelRange = 131072;

struct Task {
    uint32_t ni, begin, end;
    int depth;
};

// One node of the build: its box, and either a leaf (mid = end) or the split position of the
// primitives (partitioned in place). Binned SAH over 32 bins per axis; an object-median split when
// no bin boundary separates the primitives or when the depth budget demands it.
struct Split {
    Box nb;
    bool leaf;
    uint32_t mid;
};

Split split_node(const Prims &P, const Task &t, unsigned threads)
{
    Split r;
    Box cb;
    const uint32_t count = t.end - t.begin;
    const bool par = threads > 1u && count >= kParallelRange;
    const uint32_t chunks = par ? threads : 1u;
    const uint32_t per = (count + chunks - 1u) / chunks;
    if (par) {
        std::vector<Box> nbs(chunks), cbs(chunks);
        parallel_for(chunks, threads, [&](uint32_t c) {
            const uint32_t b = t.begin + std::min(count, c * per), e = t.begin + std::min(count, c * per + per);
            range_bounds(P, b, e, nbs[c], cbs[c]);
        });
        r.nb.reset();
        cb.reset();
        for (uint32_t c = 0; c < chunks; c++) {
            r.nb.grow(nbs[c]);
            cb.grow(cbs[c]);
        }
    } else {
        range_bounds(P, t.begin, t.end, r.nb, cb);
    }
    r.leaf = count <= 2u;
    r.mid = t.end;
    if (r.leaf)
        return r;
    uint32_t mid = t.begin + count / 2u;
    // With the remaining depth budget a balanced split must still fit: beyond half of the
    // budget's capacity fall back to an object-median split.
    const int levels_left = kMaxDepth - t.depth;
    const bool force_median = levels_left < 31 && (double)count > std::ldexp(1.0, levels_left);
    bool split_found = false;
    if (!force_median) {
        Bins bins;
        if (par) {
            std::vector<Bins> part(chunks);
            parallel_for(chunks, threads, [&](uint32_t c) {
                const uint32_t b = t.begin + std::min(count, c * per), e = t.begin + std::min(count, c * per + per);
                bin_range(P, b, e, cb, part[c]);
            });
            bins = part[0];
            for (uint32_t c = 1; c < chunks; c++)
                bins.merge(part[c]);
        } else {
            bin_range(P, t.begin, t.end, cb, bins);
        }
        double best_cost = INFINITY;
        int best_axis = -1, best_bin = -1;
        for (int axis = 0; axis < 3; axis++) {
            if (!(cb.mx[axis] > cb.mn[axis]))
                continue;
            const Box *bb = bins.bb[axis];
            const uint32_t *bc = bins.bc[axis];
            double right_area[kBins];
            uint32_t right_count[kBins];
            Box acc;
            acc.reset();
            uint32_t cnt = 0;
            for (int b = kBins - 1; b > 0; b--) {
                acc.grow(bb[b]);
                cnt += bc[b];
                right_area[b] = acc.half_area();
                right_count[b] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (int b = 0; b < kBins - 1; b++) {
                acc.grow(bb[b]);
                cnt += bc[b];
                if (cnt == 0 || right_count[b + 1] == 0)
                    continue;
                double cost = acc.half_area() * cnt + right_area[b + 1] * right_count[b + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_bin = b;
                }
            }
        }
        if (best_axis >= 0) {
            const float lo = cb.mn[best_axis], hi = cb.mx[best_axis];
            const float scale = (float)kBins / (hi - lo);
            auto it = std::partition(P.prims.begin() + t.begin, P.prims.begin() + t.end, [&](uint32_t p) {
                int b = (int)((P.centroids[3u * p + best_axis] - lo) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= best_bin;
            });
            mid = (uint32_t)(it - P.prims.begin());
            split_found = mid > t.begin && mid < t.end;
        }
    }
    if (!split_found) {
        // object median along the largest centroid extent
        int axis = 0;
        float ext = cb.mx[0] - cb.mn[0];
        for (int k = 1; k < 3; k++)
            if (cb.mx[k] - cb.mn[k] > ext) {
                ext = cb.mx[k] - cb.mn[k];
                axis = k;
            }
        mid = t.begin + count / 2u;
        std::nth_element(P.prims.begin() + t.begin, P.prims.begin() + mid, P.prims.begin() + t.end,
                         [&](uint32_t a, uint32_t b) {
                             float ca = P.centroids[3u * a + axis], cb2 = P.centroids[3u * b + axis];
                             return ca < cb2 || (ca == cb2 && a < b);
                         });
    }
    r.mid = mid;
    return r;
}

void set_node(BVHNode &n, const Split &sp, uint32_t begin, uint32_t left)
{
    for (int k = 0; k < 3; k++) {
        n.min[k] = sp.nb.mn[k];
        n.max[k] = sp.nb.mx[k];
    }
    n.prim_count = sp.leaf ? (uint32_t)(sp.mid - begin) : 0u;
    n.left_or_prim_offset = sp.leaf ? begin : left;
}

// Depth-first build of the subtree of `root` (a task whose node is nodes[root.ni]), children
// allocated in pairs in the order the tasks are taken: the left subtree is finished before the
// right one, so every subtree's nodes (below its root) are one contiguous run of the array.
// Ranges of at most `defer_max` primitives are not built but listed in `deferred` together with
// the number of nodes allocated before them.
struct Deferred {
    Task task;
    uint32_t at; // nodes.size() when the task was taken
};

int build_dfs(const Prims &P, Task root, std::vector<BVHNode> &nodes, unsigned threads, uint32_t defer_max,
              std::vector<Deferred> *deferred)
{
    int max_depth = 0;
    std::vector<Task> stack;
    stack.push_back(root);
    while (!stack.empty()) {
        const Task t = stack.back();
        stack.pop_back();
        if (deferred && t.end - t.begin <= defer_max && t.end - t.begin > 2u) {
            deferred->push_back({t, (uint32_t)nodes.size()});
            continue;
        }
        max_depth = std::max(max_depth, t.depth);
        const Split sp = split_node(P, t, threads);
        const uint32_t left = (uint32_t)nodes.size();
        set_node(nodes[t.ni], sp, t.begin, left);
        if (sp.leaf)
            continue;
        nodes.push_back(BVHNode{});
        nodes.push_back(BVHNode{});
        // right first on the stack so that the left subtree is finished first
        stack.push_back({left + 1u, sp.mid, t.end, t.depth + 1});
        stack.push_back({left, t.begin, sp.mid, t.depth + 1});
    }
    return max_depth;
}

// Builder threads: NBVH_BUILD_THREADS if set, else the host's hardware threads; one for small meshes.
unsigned build_threads(uint32_t n_prims)
{
    if (n_prims < 65536u)
        return 1u;
    unsigned t = std::thread::hardware_concurrency();
    if (const char *e = std::getenv("NBVH_BUILD_THREADS")) {
        const long v = std::strtol(e, nullptr, 10);
        if (v > 0)
            t = (unsigned)v;
    }
    return std::min(std::max(t, 1u), 64u);
}

// The whole tree: the top part depth-first on this thread (large ranges bounded and binned in
// parallel), the subtrees of at most defer_max primitives built concurrently into their own arrays,
// then every node placed where the single-threaded depth-first build puts it. The result is
// identical for any number of threads: each subtree works on its own range of `prims`, and a
// subtree's nodes form one run that the sequential build would allocate at the moment it took the
// subtree's root, after the runs of the subtrees taken before it.
int build_tree(const Prims &P, uint32_t n, std::vector<BVHNode> &nodes)
{
    const unsigned threads = build_threads(n);
    const uint32_t defer_max = threads > 1u ? std::max<uint32_t>(4096u, n / (4u * threads)) : 0u;
    nodes.clear();
    nodes.reserve(2u * (size_t)n);
    nodes.push_back(BVHNode{});
    std::vector<Deferred> deferred;
    int max_depth = build_dfs(P, Task{0u, 0u, n, 0}, nodes, threads, defer_max, threads > 1u ? &deferred : nullptr);
    if (deferred.empty())
        return max_depth;
    std::vector<std::vector<BVHNode>> sub(deferred.size());
    std::vector<int> sub_depth(deferred.size(), 0);
    parallel_for((uint32_t)deferred.size(), threads, [&](uint32_t i) {
        std::vector<BVHNode> &local = sub[i];
        local.reserve(2u * (size_t)(deferred[i].task.end - deferred[i].task.begin));
        local.push_back(BVHNode{});
        Task root = deferred[i].task;
        root.ni = 0u;
        sub_depth[i] = build_dfs(P, root, local, 1u, 0u, nullptr);
    });
    // final position of top node s: s plus the nodes of the subtrees taken before it was allocated;
    // of subtree i's node j >= 1: deferred[i].at + (nodes of subtrees 0..i-1) + j - 1
    std::vector<uint64_t> before(deferred.size() + 1u, 0u);
    for (size_t i = 0; i < deferred.size(); i++) {
        before[i + 1u] = before[i] + (sub[i].size() - 1u);
        max_depth = std::max(max_depth, sub_depth[i]);
    }
    const size_t total = nodes.size() + (size_t)before.back();
    std::vector<uint32_t> top_pos(nodes.size());
    for (size_t s = 0, i = 0; s < nodes.size(); s++) {
        while (i < deferred.size() && deferred[i].at <= s)
            i++;
        top_pos[s] = (uint32_t)(s + before[i]);
    }
    auto sub_pos = [&](size_t i, uint32_t j) { return (uint32_t)(deferred[i].at + before[i] + j - 1u); };
    std::vector<BVHNode> out(total);
    for (size_t s = 0; s < nodes.size(); s++) {
        BVHNode nd = nodes[s];
        if (nd.prim_count == 0u)
            nd.left_or_prim_offset = top_pos[nd.left_or_prim_offset];
        out[top_pos[s]] = nd;
    }
    for (size_t i = 0; i < deferred.size(); i++) {
        const std::vector<BVHNode> &local = sub[i];
        for (uint32_t j = 0; j < (uint32_t)local.size(); j++) {
            BVHNode nd = local[j];
            if (nd.prim_count == 0u)
                nd.left_or_prim_offset = sub_pos(i, nd.left_or_prim_offset);
            out[j == 0u ? top_pos[deferred[i].task.ni] : sub_pos(i, j)] = nd;
        }
    }
    nodes.swap(out);
    return max_depth;
}

} // namespace

bool build_bvh2(const std::vector<float> &vertices, const std::vector<uint32_t> &indices, std::vector<BVHNode> &nodes,
                std::vector<uint32_t> &prim_indices, std::string &err)
{
    const uint32_t nt = (uint32_t)(indices.size() / 3u);
    if (nt == 0) {
        err = "mesh has no triangles";
        return false;
    }
    std::vector<Box> boxes(nt);
    std::vector<float> centroids(3u * (size_t)nt);
    for (uint32_t p = 0; p < nt; p++) {
        Box b;
        b.reset();
        for (int k = 0; k < 3; k++)
            b.grow(&vertices[3u * (size_t)indices[3u * (size_t)p + k]]);
        boxes[p] = b;
        for (int k = 0; k < 3; k++)
            centroids[3u * (size_t)p + k] = 0.5f * (b.mn[k] + b.mx[k]);
    }
    prim_indices.resize(nt);
    for (uint32_t p = 0; p < nt; p++)
        prim_indices[p] = p;
    const Prims P{boxes, centroids, prim_indices};
    if (build_tree(P, nt, nodes) > kMaxDepth) {
        err = "BVH deeper than the 32-entry traversal stack";
        return false;
    }
    // flat-box regularisation, src/cuda/cuda_backend.cpp:212-223
    for (auto &n : nodes)
        for (int k = 0; k < 3; k++)
            if (n.max[k] - n.min[k] <= kBoxRegularisation) {
                n.min[k] -= kBoxRegularisation * 0.5f;
                n.max[k] += kBoxRegularisation * 0.5f;
            }
    return true;
}

// traverse_and_build_neural_bvh, src/cuda/neural/neural_bvh_renderer_accel.cpp:25-88: copy the
// classic BVH down to max_depth; leaves become LEAF_FINAL (1) when they are classic leaves and
// LEAF_LOD(6) (= 8, the coarsest LoD, assigned first when building the cut) otherwise.
void build_neural_cut(const std::vector<BVHNode> &nodes, uint32_t max_depth, std::vector<BVHNode> &neural,
                      std::vector<uint32_t> *node_map, std::vector<uint32_t> *depth)
{
    constexpr uint32_t kLeafLod6 = kLeafLodBase + kNumBvhLods - 1u;
    neural.assign(1, BVHNode{});
    if (node_map)
        node_map->assign(1, 0u);
    if (depth)
        depth->assign(1, 0u);
    struct Task {
        uint32_t bvh_idx, neural_idx, depth;
    };
    // recursion order of the reference: a node's two children are allocated, then the left
    // subtree is built completely before the right one
    std::vector<Task> stack;
    stack.push_back({0u, 0u, 0u});
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        const BVHNode &src = nodes[t.bvh_idx];
        BVHNode &dst = neural[t.neural_idx];
        if (node_map)
            (*node_map)[t.neural_idx] = t.bvh_idx;
        if (depth)
            (*depth)[t.neural_idx] = t.depth;
        std::memcpy(dst.min, src.min, sizeof(dst.min));
        std::memcpy(dst.max, src.max, sizeof(dst.max));
        if (src.prim_count > 0u || t.depth == max_depth) {
            dst.prim_count = src.prim_count > 0u ? kLeafFinal : kLeafLod6;
            dst.left_or_prim_offset = kNoNeuralChild;
            continue;
        }
        const uint32_t left = (uint32_t)neural.size();
        neural.push_back(BVHNode{});
        neural.push_back(BVHNode{});
        if (node_map)
            node_map->resize(neural.size(), 0u);
        if (depth)
            depth->resize(neural.size(), 0u);
        BVHNode &d2 = neural[t.neural_idx];
        d2.prim_count = 0u;
        d2.left_or_prim_offset = left;
        stack.push_back({src.left_or_prim_offset + 1u, left + 1u, t.depth + 1u});
        stack.push_back({src.left_or_prim_offset, left, t.depth + 1u});
    }
}

uint32_t build_sort_keys(const std::vector<BVHNode> &neural, uint32_t max_bins, std::vector<uint32_t> &keys)
{
    const size_t n = neural.size();
    keys.assign(n, 0u);
    std::vector<uint32_t> order;
    std::vector<uint32_t> stack{0u};
    while (!stack.empty()) {
        const uint32_t i = stack.back();
        stack.pop_back();
        const uint32_t pc = neural[i].prim_count;
        if ((pc > 0u && pc <= kLeafLodBase) || neural[i].left_or_prim_offset == kNoNeuralChild) {
            order.push_back(i);
            continue;
        }
        stack.push_back(neural[i].left_or_prim_offset + 1u);
        stack.push_back(neural[i].left_or_prim_offset);
    }
    const uint64_t leaves = order.size();
    const uint32_t bins = (uint32_t)std::min<uint64_t>(max_bins, leaves);
    for (uint64_t r = 0; r < leaves; r++)
        keys[order[r]] = (uint32_t)(r * bins / leaves);
    return bins;
}

bool coords_in_fast_div_domain(const float *c, size_t n)
{
    for (size_t i = 0; i < n; i++) {
        uint32_t bits;
        std::memcpy(&bits, &c[i], 4);
        if (bits == 0u)
            continue; // +0
        const float a = std::fabs(c[i]);
        if (!(a >= 0x1p-60f && a <= 0x1p11f))
            return false; // -0, tiny, huge, inf or nan
    }
    return true;
}

bool nodes_in_fast_div_domain(const std::vector<BVHNode> &nodes)
{
    for (const BVHNode &n : nodes)
        if (!coords_in_fast_div_domain(n.min, 3) || !coords_in_fast_div_domain(n.max, 3))
            return false;
    return true;
}

// Inference copy of the neural cut: every node box dilated once by `dil` with the FP32 operations
// of intersect_primitive_min_max / intersect_traversal_bbox (include/cuda/neural/accel/
// neural_bvh2.cuh:80-86, 101-107; centre = min + extent * 0.5, extent * (1 + dil)), and per node the
// union of the dilated boxes of the leaves below it (the traversal culls a subtree whose union is
// entirely behind the origin or beyond the current closest hit; such a subtree holds no leaf the
// reference would accept, so the accepted segments and their order are unchanged).
void build_inference_nodes(const std::vector<BVHNode> &neural, float dil, std::vector<BVHNode> &dilated,
                           std::vector<float> &bounds)
{
    const size_t n = neural.size();
    dilated = neural;
    if (dil != 0.0f) {
        const float scale = 1.0f + dil;
        for (size_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                const float mn = neural[i].min[k], mx = neural[i].max[k];
                const float ext = mx - mn;
                const float center = mn + ext * 0.5f;
                const float next = ext * scale;
                dilated[i].min[k] = center - next * 0.5f;
                dilated[i].max[k] = center + next * 0.5f;
            }
    }
    bounds.assign(8u * n, 0.0f);
    // children are allocated after their parent: a reverse sweep sees children first
    for (size_t ii = n; ii-- > 0;) {
        float *b = &bounds[8u * ii];
        const BVHNode &d = dilated[ii];
        // a leaf at the rendered LoD (0): a final or LoD-0 leaf, or a node without a neural child
        const uint32_t pc = neural[ii].prim_count;
        const bool leaf = (pc > 0u && pc <= kLeafLodBase) || neural[ii].left_or_prim_offset == kNoNeuralChild;
        if (leaf) {
            for (int k = 0; k < 3; k++) {
                b[k] = d.min[k];
                b[4 + k] = d.max[k];
            }
        } else {
            const float *l = &bounds[8u * neural[ii].left_or_prim_offset];
            const float *r = &bounds[8u * (neural[ii].left_or_prim_offset + 1u)];
            for (int k = 0; k < 3; k++) {
                b[k] = std::min(l[k], r[k]);
                b[4 + k] = std::max(l[4 + k], r[4 + k]);
            }
        }
    }
}

} // namespace nbvh
