// k_query.cu -- the neural closest-hit / visibility query as a device-resident wavefront.
//
// Reference path: NeuralPathModule::neural_bvh_traversal (src/cuda/neural/path/path_module.cu:
// 54-137) runs, per traversal step, an encode kernel, tcnn inference, a process kernel and a
// compaction kernel, then copies the active count to the host and synchronises. Here:
//
//   k_wave_first   one thread per ray: the first entered leaf (K2). Rays that enter none are
//                  answered at once; the others are appended (warp-aggregated) to state list 0.
//   then per step, over the rays listed by the previous step:
//   k_wave_encode  K3: segment points and hash-grid features, one thread per (ray, point, level),
//                  FP16 rows written in the layout the tensor-core MLP loads by TMA;
//   k_mlp_tc       K4: the fused MLP on tcgen05 tensor cores (k_mlp_tc.cu), 128-row tiles;
//   k_wave_decode  K2: LocalT decode and closest-hit update, then the next entered leaf for the
//                  rays that continue, appended to the other list.
//
// Splitting the step lets each phase run at the occupancy it needs: the gathers of K3 with 48
// warps per SM, the MLP with its accumulators in tensor memory, the divergent traversal with the
// cut read through L1 (or staged in shared memory: StepResources::stage_cut). Every kernel reads the list length from device memory, so the host
// checks it only once per batch of steps (one 16-byte copy).
#include <type_traits>

#include "device_math.cuh"
#include "net_device.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kEncodeThreads = 256;
constexpr uint32_t kFirstThreads = 256;
constexpr uint32_t kSortThreads = 1024;
// Lists shorter than this are walked in list order: the sort would cost more than the locality it buys.
constexpr uint32_t kSortMinRows = 1u << 16;
// Rows with at least this many (point, level) pairs to encode are sorted by octant within a leaf.
constexpr uint32_t kSubBinMinPointLevels = 32;
// node visits of a traversal between lane refills (measured on GB300, 2^22 uniform rays: 4 -> 3.29,
// 8 -> 3.25, 12 -> 3.24, 16 -> 3.24 ms per query)
constexpr uint32_t kDefaultVisitsPerRound = 12;
// Encoder blocks of 256 threads per SM: the launch bound (up to 64 registers a thread; the paired
// corner gathers use 56 and spill at the 40 of a 6-block bound) and the default launch. Every launch uses at
// most this many per SM, so each block's contiguous range of rows runs in a single wave; fewer
// blocks than fit an SM make each block's range of the sorted rows longer, so that an SM's L1
// serves fewer leaf regions at a time (measured on GB300 with the rows sorted by leaf and octant,
// 2^22 rays, at a 40-register bound: 6 blocks 3.25, 5 3.25, 4 3.21, 3 3.27, 2 3.44 ms per query;
// the 64-register bound with paired gathers then took 4 blocks from 3.22 to 3.17-3.19 ms).
constexpr uint32_t kEncodeBlocksPerSm = 4;
// From step tail_step() on, the rays still listed are finished by one persistent kernel
// (k_wave_tail) instead of one short wavefront step after another: the lists are short by then and
// each step would cost about the same fixed 60-80 us whatever its length. The switch depends only
// on the step (how many segments a ray has evaluated) and on the cut, so a ray's record does not
// depend on the other rays of its batch. Measured on GB300: cuts up to kMaxSortNodes nodes (their
// later steps still fill the GPU) gain most from step 5 on, larger learned cuts (long runs of
// small leaves, lists that stay short for 20-30 steps) from step 3 on.
__host__ __device__ constexpr uint32_t tail_step(uint32_t n_cut_nodes)
{
    return n_cut_nodes <= kMaxSortNodes ? 5u : 3u;
}
constexpr uint32_t kTailWarps = 8;
constexpr uint32_t kTailThreads = kTailWarps * 32;
// decode: the shared-memory cut variant runs one 768-thread block per SM, the global-memory
// variant two 384-thread blocks; both leave 85 registers per thread (the traversal stack stays in
// registers and local memory without spilling)
constexpr uint32_t decode_threads(bool smem_cut) { return smem_cut ? 768u : 384u; }

struct WaveArgs {
    GridParams grid;
    NeuralConsts nc;
    const float4 *nodes;  // pre-dilated inference copy of the cut
    const float4 *bounds; // union of dilated leaf boxes per node
    const uint8_t *non_neural;
    const uint32_t *table;
    const __half *weights; // 16-bit network matrices (network-first parameter layout)
    const nbvh_ray *rays;
    nbvh_neural_hit *hits;
    QueryCounters *counters;
    uint32_t *fallback_list;
    WaveList lists[2];
    uint32_t *wave_counts; // 3 rotating list counters + the MLP's error word
    __half *features;      // [capacity][n_inputs] FP16 rows of the current step
    float *outputs;        // [capacity][8] network outputs of the current step
    uint32_t *perm;        // list rows in leaf-node order (nullptr: rows in list order)
    const uint32_t *ray_order; // the first pass's order of the rays (nullptr: batch order)
    uint32_t *node_bins;   // [2][n_sort_nodes] rows per leaf node of the current / next list
    uint32_t *node_cursor; // [2][n_sort_nodes] placement cursors of the sort
    const uint32_t *sort_key; // sort bin of each leaf (cuts above kMaxSortNodes nodes); NULL: the node
    uint32_t n_sort_nodes;    // sort bins
    uint32_t sub_bins;        // 1: each leaf's rows in 8 bins by the octant of their segment midpoint
    uint16_t *row_keys;       // [capacity] sort bin of each listed row, written as it is appended
                              // (nullptr: the sort recomputes it from the row's state)
    uint32_t n_hidden_layers;
    uint32_t n;
    uint32_t n_cut_nodes;
    uint32_t bf16;   // MLP inputs in BF16 (else FP16)
    uint32_t prec;   // nbvh_precision of the MLP (FP8: hidden-matrix inputs rounded to E4M3)
    uint32_t visits; // node visits per traversal round between lane refills
    // rays finishing in step late_from or later are listed (the early copy of the records to the
    // host was taken before them); late_from = ~0 lists nothing
    uint32_t *late_list;
    uint32_t *late_count;
    uint32_t late_from;
};

__device__ __forceinline__ void write_hit(nbvh_neural_hit *hits, uint32_t id, float t, V3 nrm, V3 alb, float vis,
                                          uint32_t flags, uint32_t segments)
{
    float4 *out = reinterpret_cast<float4 *>(hits + id);
    out[0] = make_float4(t, nrm.x, nrm.y, nrm.z);
    out[1] = make_float4(alb.x, alb.y, alb.z, vis);
    out[2] = make_float4(__uint_as_float(flags), __uint_as_float(segments), __uint_as_float(kInvalid), 0.f);
}

// The record of a ray that finishes in decode step `it`, plus its id on the late list when the
// early host copy of the records was already taken.
__device__ __forceinline__ void finish_hit(const WaveArgs &a, uint32_t it, uint32_t id, float t, V3 nrm, V3 alb,
                                           float vis, uint32_t flags, uint32_t segments)
{
    write_hit(a.hits, id, t, nrm, alb, vis, flags, segments);
    if (it >= a.late_from) {
        const uint32_t k = atomicAdd(a.late_count, 1u);
        if (k < a.n)
            a.late_list[k] = id;
    }
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

// Sort bin of a leaf: the leaf itself, or for large cuts its bin among runs of leaves in
// depth-first order (neighbouring leaves in space).
__device__ __forceinline__ uint32_t sort_bin(const WaveArgs &a, uint32_t node)
{
    return a.sort_key ? a.sort_key[node] : node;
}

// Sort bin of a listed row: its leaf's bin, and with sub-bins the octant of the leaf box that holds
// the midpoint of the row's segment, so that the encoder meets the rows of a leaf region by region.
// The first pass and the decode (counting the rows they append) and the sort (placing them)
// evaluate it on the same stored values.
__device__ __forceinline__ uint32_t row_bin(const WaveArgs &a, uint32_t node, V3 o, V3 d, float mint, float maxt)
{
    const uint32_t b = sort_bin(a, node);
    if (!a.sub_bins)
        return b;
    // explicit roundings: every call site must get the same bits, whatever the compiler contracts
    const float tm = __fmul_rn(0.5f, __fadd_rn(mint, maxt));
    const float4 lo = __ldg(a.nodes + 2u * node), hi = __ldg(a.nodes + 2u * node + 1u);
    const uint32_t oct = (__fmaf_rn(d.x, tm, o.x) > __fmul_rn(0.5f, __fadd_rn(lo.x, hi.x)) ? 1u : 0u) |
                         (__fmaf_rn(d.y, tm, o.y) > __fmul_rn(0.5f, __fadd_rn(lo.y, hi.y)) ? 2u : 0u) |
                         (__fmaf_rn(d.z, tm, o.z) > __fmul_rn(0.5f, __fadd_rn(lo.z, hi.z)) ? 4u : 0u);
    return kSubBins * b + oct;
}

__device__ __forceinline__ uint32_t listed_row_bin(const WaveArgs &a, const WaveList &in, uint32_t r)
{
    if (a.row_keys)
        return a.row_keys[r];
    if (!a.sub_bins)
        return sort_bin(a, in.meta[r].y);
    const float4 od0 = in.od0[r], od1 = in.od1[r];
    const uint4 m = in.meta[r];
    return row_bin(a, m.y, mk3(od0.x, od0.y, od0.z), mk3(od1.x, od1.y, od1.z), od1.w, __uint_as_float(m.x));
}

// Counts the rows a warp appends per sort bin (one atomic per distinct bin in the warp); all 32
// lanes take part.
__device__ __forceinline__ void count_nodes(uint32_t *bins, bool want, uint32_t node)
{
    const unsigned m = __ballot_sync(kFull, want);
    if (!want)
        return;
    const unsigned same = __match_any_sync(m, node);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(same) - 1))
        atomicAdd(&bins[node], (uint32_t)__popc(same));
}

// Coherence bin of a ray: its direction class (octant and dominant axis: 24 classes) above the
// Morton code of its origin's cell in an 8 x 8 x 8 grid over the scene box grown by half its size
// on every side (origins outside are clamped to the border cells). Measured on GB300 against the
// octant alone (4,096 bins): classic 1.097 -> 1.060 ms, neural 3.285 -> 3.275 ms per 2^22 rays;
// a finer direction grid (cube faces x 4 x 4) with 4 x 4 x 4 origin cells was slower (1.114, 3.303).
__device__ __forceinline__ uint32_t ray_bin(const nbvh_ray *rays, uint32_t i, V3 lo, V3 scale)
{
    const float4 *r = reinterpret_cast<const float4 *>(rays + i);
    const float4 ra = __ldg(r), rb = __ldg(r + 1);
    const uint32_t oct = (rb.x > 0.0f ? 1u : 0u) | (rb.y > 0.0f ? 2u : 0u) | (rb.z > 0.0f ? 4u : 0u);
    const float ax = fabsf(rb.x), ay = fabsf(rb.y), az = fabsf(rb.z);
    const uint32_t dom = (ax >= ay && ax >= az) ? 0u : (ay >= az ? 1u : 2u); // NaN -> 2
    auto cell = [](float x, float l, float s) {
        const float c = (x - l) * s;
        return c >= 7.0f ? 7u : (c > 0.0f ? (uint32_t)c : 0u); // NaN -> 0
    };
    const uint32_t cx = cell(ra.x, lo.x, scale.x), cy = cell(ra.y, lo.y, scale.y), cz = cell(ra.z, lo.z, scale.z);
    uint32_t m = 0;
#pragma unroll
    for (int b = 0; b < 3; b++)
        m |= (((cx >> b) & 1u) << (3 * b)) | (((cy >> b) & 1u) << (3 * b + 1)) | (((cz >> b) & 1u) << (3 * b + 2));
    return (oct * 3u + dom) * 512u + m; // < 24 x 512 = kRayBins
}

struct RayBinArgs {
    const nbvh_ray *rays;
    uint32_t n;
    V3 lo, scale;
    uint16_t *keys;
    uint32_t *bins;  // kRayBins counts (zeroed before), then the cursors
    uint32_t *order; // n ray ids, bin by bin
};

// Counts the rays per bin and keeps every ray's bin. Each block takes one contiguous chunk of the
// batch and adds its shared-memory counts to the global ones (one atomic per non-empty bin).
constexpr uint32_t kRayBinThreads = 1024;

__device__ __forceinline__ void ray_chunk(uint32_t n, uint32_t &r0, uint32_t &r1)
{
    const uint32_t per = (n + gridDim.x - 1u) / gridDim.x;
    r0 = min(n, blockIdx.x * per);
    r1 = min(n, r0 + per);
}

__global__ void __launch_bounds__(kRayBinThreads) k_ray_bins(const __grid_constant__ RayBinArgs a)
{
    __shared__ uint32_t cnt[kRayBins];
    for (uint32_t b = threadIdx.x; b < kRayBins; b += blockDim.x)
        cnt[b] = 0u;
    __syncthreads();
    uint32_t r0, r1;
    ray_chunk(a.n, r0, r1);
    for (uint32_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const uint32_t b = ray_bin(a.rays, i, a.lo, a.scale);
        a.keys[i] = (uint16_t)b;
        atomicAdd(&cnt[b], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kRayBins; b += blockDim.x)
        if (cnt[b])
            atomicAdd(&a.bins[b], cnt[b]);
}

// Exclusive scan of the bin counts into placement cursors (one block of 1,024 threads,
// kRayBins / 1,024 bins each).
constexpr uint32_t kRayBinsPerThread = kRayBins / 1024u;
static_assert(kRayBins % 1024u == 0u, "whole bins per scan thread");
__global__ void __launch_bounds__(1024) k_ray_bin_scan(uint32_t *bins)
{
    __shared__ uint32_t warp_sums[32];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    uint32_t v[kRayBinsPerThread], run = 0;
#pragma unroll
    for (uint32_t k = 0; k < kRayBinsPerThread; k++) {
        v[k] = bins[kRayBinsPerThread * t + k];
        run += v[k];
    }
    uint32_t incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t x = __shfl_up_sync(kFull, incl, off);
        if (lane >= (uint32_t)off)
            incl += x;
    }
    if (lane == 31u)
        warp_sums[warp] = incl;
    __syncthreads();
    uint32_t base = incl - run;
    for (uint32_t w = 0; w < warp; w++)
        base += warp_sums[w];
#pragma unroll
    for (uint32_t k = 0; k < kRayBinsPerThread; k++) {
        bins[kRayBinsPerThread * t + k] = base;
        base += v[k];
    }
}

// Places the ray ids bin by bin: each block takes the same chunk as k_ray_bins, counts it per bin
// again in shared memory, reserves one range per non-empty bin from the global cursors, then
// places its rays with shared-memory atomics (the order inside a bin does not matter).
__global__ void __launch_bounds__(kRayBinThreads) k_ray_bin_place(const __grid_constant__ RayBinArgs a)
{
    __shared__ uint32_t cnt[kRayBins];
    for (uint32_t b = threadIdx.x; b < kRayBins; b += blockDim.x)
        cnt[b] = 0u;
    __syncthreads();
    uint32_t r0, r1;
    ray_chunk(a.n, r0, r1);
    for (uint32_t i = r0 + threadIdx.x; i < r1; i += blockDim.x)
        atomicAdd(&cnt[a.keys[i]], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kRayBins; b += blockDim.x)
        if (cnt[b])
            cnt[b] = atomicAdd(&a.bins[b], cnt[b]); // now this block's next position in bin b
    __syncthreads();
    for (uint32_t i = r0 + threadIdx.x; i < r1; i += blockDim.x)
        a.order[atomicAdd(&cnt[a.keys[i]], 1u)] = i;
}

// K2 first pass: the first entered leaf of every ray (the first leaf is searched with an unbounded
// current_maxt, include/cuda/neural/neural_bvh_module_common.cuh:332-343). Rays that enter none
// are answered at once; the others are appended to state list 0. Persistent warps take rays from
// a work counter and refill lanes between rounds of a.visits node visits, as the decode
// kernel does, so the warp's lanes stay busy while the traversal lengths differ.
__global__ void __launch_bounds__(kFirstThreads, 4) k_wave_first(const __grid_constant__ WaveArgs a)
{
    const int lane = threadIdx.x & 31;
    uint32_t *head = &a.wave_counts[7];
    RayState s;
    uint32_t stack[kNeuralStackSize];
    RayDiv rdiv;
    bool cull_ok = false, active = false, exhausted = false;
    float tmax = 0.f;
    const GlobalCut cut{a.nodes, a.bounds};
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle != 0u && !exhausted) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(head, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            exhausted = base + (uint32_t)__popc(idle) >= a.n;
            const uint32_t i = base + __popc(idle & ((1u << lane) - 1u));
            if (!active && i < a.n) {
                const uint32_t ray = a.ray_order ? a.ray_order[i] : i;
                const float4 *r = reinterpret_cast<const float4 *>(a.rays + ray);
                const float4 ra = __ldg(r), rb = __ldg(r + 1);
                s.o = mk3(ra.x, ra.y, ra.z);
                s.d = mk3(rb.x, rb.y, rb.z);
                tmax = rb.w;
                cull_ok = s.d.x != 0.0f && s.d.y != 0.0f && s.d.z != 0.0f;
                rdiv = make_raydiv(s.o, s.d, a.nc.fast_div_ok != 0u);
                s.sp = 1;
                stack[0] = 0;
                s.ray_id = ray;
                active = true;
            }
        }
        if (!__any_sync(kFull, active)) {
            if (exhausted)
                break;
            continue;
        }
        bool listed = false;
        if (active) {
            const int res = neural_intersect_inference(cut, a.nc.bvh_lod, s.o, rdiv, cull_ok, stack, s.sp,
                                                       a.nc.inference_mint_epsilon, a.nc.inference_maxt_epsilon,
                                                       FLT_MAX, s.seg_mint, s.seg_maxt, s.seg_node, (int)a.visits);
            if (res != 2) {
                active = false;
                const uint32_t i = s.ray_id;
                if (res == 1) {
                    if (a.non_neural && a.non_neural[s.seg_node]) {
                        write_hit(a.hits, i, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, 0u, 0u);
                        const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                        a.fallback_list[slot] = i;
                        atomicAdd(&a.counters->fallback, 1u);
                    } else {
                        listed = true;
                        s.best_t = tmax; // the ray's tmax plays the role of the current closest hit
                        s.vis = 0.f;
                        s.nrm = mk3(0, 0, 0);
                        s.alb = mk3(0, 0, 0);
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
        }
        const uint32_t pos = warp_append(listed, &a.wave_counts[0]);
        const uint32_t bin = (a.perm && listed) ? row_bin(a, s.seg_node, s.o, s.d, s.seg_mint, s.seg_maxt) : 0u;
        if (listed) {
            store_state(a.lists[0], pos, s, stack);
            if (a.row_keys)
                a.row_keys[pos] = (uint16_t)bin;
        }
        if (a.perm)
            count_nodes(a.node_bins, listed, bin);
    }
}

// K3 of one step: the FP16 hash-grid features of every listed ray's current leaf segment, one
// thread per (ray, point) looping over the levels, written row-major to features[row][n_inputs]
// (point-major, then level, F features per level). Points follow encode_bvh_network_input_data
// (src/cuda/neural/neural_bvh_module_kernels.cu:266-303): the segment ends are swapped for a
// negative mint, then encoded into the dilated scene box. The point is computed once for all its
// levels, so the kernel's instructions go to the gathers and their interpolation; it holds no
// MLP state; its 4 blocks of 256 threads per SM keep many gathers in flight to hide their latency.

template <uint32_t F>
__global__ void __launch_bounds__(kEncodeThreads, kEncodeBlocksPerSm)
    k_wave_encode(const __grid_constant__ WaveArgs a, uint32_t it)
{
    __shared__ GridParams gp;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&a.grid);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&gp);
        for (uint32_t i = threadIdx.x; i < sizeof(GridParams) / 4u; i += blockDim.x)
            dst[i] = src[i];
    }
    __syncthreads();
    const uint32_t count_in = *reinterpret_cast<volatile const uint32_t *>(&a.wave_counts[it % 3u]);
    if (blockIdx.x == 0 && threadIdx.x == 0 && count_in)
        atomicAdd(&a.counters->encoded, count_in);
    const uint32_t L = gp.n_levels, P = gp.n_points;
    const WaveList &in = a.lists[it & 1u];
    const NeuralConsts &nc = a.nc;
    const V3 smin = mk3(nc.scene_min[0], nc.scene_min[1], nc.scene_min[2]);
    const V3 smax = mk3(nc.scene_max[0], nc.scene_max[1], nc.scene_max[2]);
    const float dilation = __fadd_rn(__fadd_rn(1.0f, nc.node_extent_dilation), nc.fixed_node_dilation);
    const V3 ext = scale3(sub3(smax, smin), dilation);
    const V3 center = scale3(add3(smax, smin), 0.5f);
    // levels whose features fill one 16-byte store: 4 (F = 2), 2 (F = 4), 1 (F = 8)
    constexpr uint32_t LPS = 8u / F;
    const bool vec_store = (L % LPS) == 0u; // each point's block of L * F halves starts 16-byte aligned
    const bool bf16 = a.bf16 != 0u;
    auto pack16 = [bf16](float lo, float hi) { return bf16 ? pack_bf162(lo, hi) : pack_half2(lo, hi); };
    uint32_t *feat = reinterpret_cast<uint32_t *>(a.features);
    const bool sorted = a.perm != nullptr && count_in >= kSortMinRows;
    const uint32_t total = count_in * P; // at most 2^22 rays x 16 points
    // Short lists (the tail of the query) split each point's levels over G threads, LPS levels
    // (one 16-byte store) each, so that a point's gathers are in flight together instead of one
    // level after another; long lists keep one thread per point (all levels), which the other
    // points' threads already hide.
    const uint32_t lanes = gridDim.x * blockDim.x;
    const uint32_t G = (vec_store && (size_t)total * (L / LPS) <= 2u * (size_t)lanes) ? (L / LPS) : 1u;
    const uint32_t LG = L / G;
    const uint32_t work = total * G;
    // each block takes one contiguous range of the (node-sorted) rows, so an SM's L1 serves the
    // grid cells of a few leaf regions at a time
    const uint32_t per_block = (work + gridDim.x - 1u) / gridDim.x;
    const uint32_t w_end = min(work, blockIdx.x * per_block + per_block);
    for (uint32_t w = blockIdx.x * per_block + threadIdx.x; w < w_end; w += blockDim.x) {
        const uint32_t g = w / G, lg = w - g * G;
        const uint32_t i = g / P, p = g - i * P;
        const uint32_t row = sorted ? a.perm[i] : i;
        const float4 od0 = in.od0[row], od1 = in.od1[row];
        const V3 o = mk3(od0.x, od0.y, od0.z), d = mk3(od1.x, od1.y, od1.z);
        float ta = od1.w, tb = __uint_as_float(in.meta[row].x);
        if (ta < 0.0f) { // swap for a negative mint (neural_bvh_module_kernels.cu:281-286)
            const float t = ta;
            ta = tb;
            tb = t;
        }
        const V3 epo = encode_world(ray_at(o, d, ta), center, ext);
        const V3 epi = encode_world(ray_at(o, d, tb), center, ext);
        float t;
        if (gp.segment_distribution == NBVH_SEGMENT_UNIFORM) {
            uint32_t rng = __float_as_uint(in.ar[row].w);
            for (uint32_t k = 0; k <= p; k++)
                t = lcg_randomf(rng);
        } else {
            uint32_t unused = 0;
            t = segment_t(p, P, gp.segment_distribution, unused);
        }
        const V3 pos = segment_point(epo, epi, t);
        uint32_t *dst = feat + (size_t)g * L * (F / 2u); // row * (P * L * F / 2) + p * L * F / 2 words
        if constexpr (F == 2u) {
            if (vec_store) {
                for (uint32_t l = lg * LG; l < lg * LG + LG; l += 4u) {
                    uint4 q;
                    float2 f = encode_level<true>(a.table, gp, l, pos);
                    q.x = pack16(f.x, f.y);
                    f = encode_level<true>(a.table, gp, l + 1u, pos);
                    q.y = pack16(f.x, f.y);
                    f = encode_level<true>(a.table, gp, l + 2u, pos);
                    q.z = pack16(f.x, f.y);
                    f = encode_level<true>(a.table, gp, l + 3u, pos);
                    q.w = pack16(f.x, f.y);
                    *reinterpret_cast<uint4 *>(dst + l) = q;
                }
            } else {
                for (uint32_t l = 0; l < L; l++) {
                    const float2 f = encode_level<true>(a.table, gp, l, pos);
                    dst[l] = pack16(f.x, f.y);
                }
            }
        } else {
            // F = 4: 8 bytes per level; F = 8: 16 bytes per level (always aligned to its size)
            for (uint32_t l = lg * LG; l < lg * LG + LG; l++) {
                float f[F];
                encode_level_wide<F>(a.table, gp, l, pos, f);
                if constexpr (F == 4u)
                    *reinterpret_cast<uint2 *>(dst + 2u * l) = make_uint2(pack16(f[0], f[1]), pack16(f[2], f[3]));
                else
                    *reinterpret_cast<uint4 *>(dst + 4u * l) = make_uint4(pack16(f[0], f[1]), pack16(f[2], f[3]),
                                                                          pack16(f[4], f[5]), pack16(f[6], f[7]));
            }
        }
    }
}

// Counting sort of the listed rays by their current leaf node (the per-node compaction of the
// segments). The per-node counts were gathered when the list was written. Each block takes one
// contiguous chunk of the list: it scans the counts in shared memory, counts its own rows per node
// with shared-memory atomics, reserves one range per non-empty node with a global atomic, then
// places its rows. The encoder, MLP and decoder then walk the list in node order, so rays of the
// same leaf region are encoded together and the grid cells of the coarser levels are served from
// L1. Also clears the next step's counts and cursors.
__global__ void __launch_bounds__(kSortThreads) k_wave_sort(const __grid_constant__ WaveArgs a, uint32_t it)
{
    extern __shared__ uint32_t sort_smem[];
    const uint32_t NB = a.n_sort_nodes;
    uint32_t *scan = sort_smem, *cnt = sort_smem + NB, *base = sort_smem + 2u * NB;
    const uint32_t *bins = a.node_bins + (it & 1u) * NB;
    uint32_t *cursor = a.node_cursor + (it & 1u) * NB;
    {
        uint32_t *next_bins = a.node_bins + ((it + 1u) & 1u) * NB;
        uint32_t *next_cursor = a.node_cursor + ((it + 1u) & 1u) * NB;
        for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < NB; k += gridDim.x * blockDim.x) {
            next_bins[k] = 0u;
            next_cursor[k] = 0u;
        }
    }
    const uint32_t count_in = *reinterpret_cast<volatile const uint32_t *>(&a.wave_counts[it % 3u]);
    const uint32_t per_block = (count_in + gridDim.x - 1u) / gridDim.x;
    const uint32_t r0 = blockIdx.x * per_block, r1 = min(count_in, r0 + per_block);
    if (count_in < kSortMinRows || r0 >= r1)
        return;
    // exclusive scan of the node counts: contiguous runs per thread, then a scan of the run sums
    const uint32_t per = (NB + blockDim.x - 1u) / blockDim.x;
    const uint32_t k0 = min(NB, threadIdx.x * per), k1 = min(NB, k0 + per);
    uint32_t run = 0;
    for (uint32_t k = k0; k < k1; k++) {
        run += bins[k];
        cnt[k] = 0u;
    }
    __shared__ uint32_t warp_sums[kSortThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, off);
        if (lane >= off)
            incl += v;
    }
    if (lane == 31)
        warp_sums[warp] = incl;
    __syncthreads();
    uint32_t acc = incl - run;
    for (int w = 0; w < warp; w++)
        acc += warp_sums[w];
    for (uint32_t k = k0; k < k1; k++) {
        scan[k] = acc;
        acc += bins[k];
    }
    const WaveList &in = a.lists[it & 1u];
    for (uint32_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
        atomicAdd(&cnt[listed_row_bin(a, in, r)], 1u);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < NB; k += blockDim.x) {
        const uint32_t c = cnt[k];
        base[k] = c ? atomicAdd(&cursor[k], c) : 0u;
        cnt[k] = 0u;
    }
    __syncthreads();
    for (uint32_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const uint32_t node = listed_row_bin(a, in, r);
        const uint32_t slot = scan[node] + base[node] + atomicAdd(&cnt[node], 1u);
        if (slot < count_in) // the counts match the list; the check only keeps a stray row in bounds
            a.perm[slot] = r;
    }
}

// K2 of one step: decode the network outputs of each listed ray's segment (process step,
// src/cuda/neural/path/path_inference_kernels.cu:61-131), keep the closest hit, then find the
// next entered leaf (process_bvh_network_output_and_intersect_neural_bvh,
// include/cuda/neural/neural_bvh_module_common.cuh:496-550) and append the ray to the next list,
// or write its final record. One thread per listed ray.
template <bool SMEM_CUT>
__global__ void __launch_bounds__(decode_threads(SMEM_CUT), SMEM_CUT ? 1 : 2) k_wave_decode(const __grid_constant__ WaveArgs a,
                                                                                   uint32_t it)
{
    const uint32_t count_in = *reinterpret_cast<volatile const uint32_t *>(&a.wave_counts[it % 3u]);
    uint32_t *count_out = &a.wave_counts[(it + 1u) % 3u];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.wave_counts[(it + 2u) % 3u] = 0u;      // output counter of the next step (last read a step ago)
        a.wave_counts[4u + (it + 1u) % 3u] = 0u; // work counter of the next step
    }
    if (blockIdx.x * blockDim.x >= count_in)
        return; // nothing for this block: skip staging the cut

    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *s_nodes = reinterpret_cast<float4 *>(smem_raw);
    float2 *s_bounds = reinterpret_cast<float2 *>(smem_raw + a.n_cut_nodes * 32u);
    if (SMEM_CUT) {
        for (uint32_t i = threadIdx.x; i < 2u * a.n_cut_nodes; i += blockDim.x)
            s_nodes[i] = __ldg(a.nodes + i);
        for (uint32_t i = threadIdx.x; i < a.n_cut_nodes; i += blockDim.x) {
            const float4 u = __ldg(a.bounds + 2u * i), v = __ldg(a.bounds + 2u * i + 1u);
            s_bounds[3u * i] = make_float2(u.x, u.y);
            s_bounds[3u * i + 1u] = make_float2(u.z, v.x);
            s_bounds[3u * i + 2u] = make_float2(v.y, v.z);
        }
        __syncthreads();
    }
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
    const float thr = nc.visibility_threshold;
    const uint32_t P = a.grid.n_points;
    const WaveList &in = a.lists[it & 1u];
    const WaveList &out = a.lists[(it + 1u) & 1u];
    const int lane = threadIdx.x & 31;
    uint32_t st_segments = 0, st_capped = 0, st_overflow = 0, st_fallback = 0;

    // Persistent warps with per-lane refill (after Aila and Laine, "Understanding the efficiency of
    // ray traversal on GPUs", HPG 2009): the next-leaf search takes a different number of node
    // visits per ray, so each round runs at most a.visits visits, after which lanes whose ray
    // is done take a new row from the step's work counter. Lanes stay busy instead of waiting for
    // the longest traversal of their warp. All lanes run every round (warp_append needs all 32).
    uint32_t *head = &a.wave_counts[4u + it % 3u];
    const bool sorted = a.perm != nullptr && count_in >= kSortMinRows;
    RayState s;
    uint32_t stack[kNeuralStackSize];
    RayDiv rdiv;
    bool cull_ok = false, active = false, exhausted = false;
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle != 0u && !exhausted) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(head, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            exhausted = base + (uint32_t)__popc(idle) >= count_in;
            const uint32_t i = base + __popc(idle & ((1u << lane) - 1u)); // position in node order
            if (!active && i < count_in) {
                load_state(in, sorted ? a.perm[i] : i, s, stack);
                bool traverse = false;
                if (s.segments > nc.max_traversal_steps) { // step cap (path_module.cu:68, last_inference)
                    s.flags |= NBVH_HIT_STEP_CAP;
                    st_capped++;
                    const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                    finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f,
                              s.flags, s.segments);
                } else {
                    if (a.grid.segment_distribution == NBVH_SEGMENT_UNIFORM)
                        for (uint32_t k = 0; k < P; k++) // the draws the encoder made for this segment
                            (void)lcg_randomf(s.rng);
                    const float4 *src = reinterpret_cast<const float4 *>(a.outputs + (size_t)i * 8u);
                    const float4 oa = src[0], ob = src[1];
                    const float o8[8] = {oa.x, oa.y, oa.z, oa.w, ob.x, ob.y, ob.z, ob.w};
                    s.segments++;
                    st_segments++;
                    if (nc.fallback_margin > 0.0f && fabsf(__fsub_rn(o8[0], thr)) < nc.fallback_margin) {
                        finish_hit(a, it, s.ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, s.flags & ~NBVH_HIT_VALID,
                                  s.segments);
                        const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                        a.fallback_list[slot] = s.ray_id;
                        st_fallback++;
                    } else {
                        // process_neural_bvh_traversal_step, path_inference_kernels.cu:61-131
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
                                        s.vis = o8[0];
                                        s.nrm = normalize3(mk3(__fsub_rn(__fmul_rn(o8[2], 2.0f), 1.0f),
                                                               __fsub_rn(__fmul_rn(o8[3], 2.0f), 1.0f),
                                                               __fsub_rn(__fmul_rn(o8[4], 2.0f), 1.0f)));
                                        s.alb = mk3(o8[5], o8[6], o8[7]);
                                    }
                                }
                            }
                        }
                        traverse = !stop && s.sp > 0;
                        if (!traverse) {
                            const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                            finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f,
                                      s.flags, s.segments);
                        }
                    }
                }
                if (traverse) {
                    active = true;
                    cull_ok = s.d.x != 0.0f && s.d.y != 0.0f && s.d.z != 0.0f;
                    rdiv = make_raydiv(s.o, s.d, nc.fast_div_ok != 0u);
                }
            }
        }
        if (!__any_sync(kFull, active)) {
            if (exhausted)
                break;
            continue;
        }
        bool keep = false;
        if (active) {
            // process_bvh_network_output_and_intersect_neural_bvh, common.cuh:496-550; the closest
            // hit so far (best_t) bounds the search
            const int res = neural_intersect_inference(cut, nc.bvh_lod, s.o, rdiv, cull_ok, stack, s.sp,
                                                       nc.inference_mint_epsilon, nc.inference_maxt_epsilon, s.best_t,
                                                       s.seg_mint, s.seg_maxt, s.seg_node, (int)a.visits);
            if (res != 2) {
                active = false;
                bool done = false;
                if (res == 1) {
                    if (a.non_neural && a.non_neural[s.seg_node]) {
                        finish_hit(a, it, s.ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, s.flags & ~NBVH_HIT_VALID,
                                  s.segments);
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
                if (!keep && !done) {
                    const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                    finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                              s.segments);
                }
            }
        }
        const uint32_t pos = warp_append(keep, count_out);
        const uint32_t bin = (a.perm && keep) ? row_bin(a, s.seg_node, s.o, s.d, s.seg_mint, s.seg_maxt) : 0u;
        if (keep) {
            store_state(out, pos, s, stack);
            if (a.row_keys) // the sort of this step ran before the encoder: the keys are free
                a.row_keys[pos] = (uint16_t)bin;
        }
        if (a.perm)
            count_nodes(a.node_bins + ((it + 1u) & 1u) * a.n_sort_nodes, keep, bin);
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

// Shared-memory layout of the tail kernel: [cut nodes + bounds when staged] [grid parameters]
// [network matrices] then per warp a 16-row feature tile, the 32 rows' segment end points, the 32
// rows' network outputs and each lane's enumerated segments.
constexpr uint32_t kTailMaxAhead = 8; // segments a lane may enumerate ahead of its decode

struct TailLayout {
    uint32_t cut_bytes, gp_off, w_off, warp_off, warp_bytes, fld, ends_off, outs_off, segs_off, total;
};

__host__ __device__ inline TailLayout tail_layout(uint32_t n_cut_nodes, bool smem_cut, uint32_t n_inputs,
                                                  uint32_t n_hidden_layers)
{
    TailLayout t;
    t.cut_bytes = smem_cut ? ((n_cut_nodes * 56u + 15u) & ~15u) : 0u;
    t.gp_off = t.cut_bytes;
    t.w_off = t.gp_off + (((uint32_t)sizeof(GridParams) + 15u) & ~15u);
    const SmemNetLayout SL = smem_net_layout(n_inputs, n_hidden_layers);
    t.warp_off = t.w_off + ((SL.total * 2u + 15u) & ~15u);
    t.fld = n_inputs + 8u;
    t.ends_off = (16u * t.fld * 2u + 15u) & ~15u;     // float4 [32][2]
    t.outs_off = t.ends_off + 32u * 32u;              // float [32][8]
    t.segs_off = t.outs_off + 32u * 32u;              // float2 [32 lanes][kTailMaxAhead]
    t.warp_bytes = t.segs_off + 32u * kTailMaxAhead * 8u;
    t.total = t.warp_off + kTailWarps * t.warp_bytes;
    return t;
}

// The rest of the query from step `it` on. Persistent warps own up to 32 rays each (one per lane,
// refilled from the step's list as rays finish). Per round, every lane lists the segments its ray
// evaluates next, the features of all listed segments are encoded into the warp's feature tile
// (up to two 16-row tiles), the MLP runs on them with mma.sync, and each lane decodes its outputs
// in order, exactly as k_wave_decode does one step at a time.
//
// While the list still has rays every lane lists one segment. Once it is exhausted and the warp
// thins out, a lane lists up to min(8, 32 / live lanes) segments ahead: the next leaves its
// traversal enters with the current closest hit as bound, keeping a copy of its stack after each.
// Decoding them in order is exact while no hit is accepted, since the bound and hence the
// traversal do not change; when one is accepted, the segments listed after it are dropped (not
// evaluated, not counted) and the stack goes back to its copy, so the traversal continues with
// the new bound exactly as the step-by-step query would. Rays with uniformly sampled segment
// points (whose random draws follow the evaluated segments) or with non-neural leaves list one
// segment at a time.
template <bool SMEM_CUT, bool BF16, bool FP8>
__global__ void __launch_bounds__(kTailThreads, SMEM_CUT ? 1 : 2) k_wave_tail(const __grid_constant__ WaveArgs a,
                                                                             uint32_t it)
{
    const uint32_t count_in = *reinterpret_cast<volatile const uint32_t *>(&a.wave_counts[it % 3u]);
    if (blockIdx.x * kTailThreads >= count_in)
        return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t n_in = a.grid.n_inputs, H = a.n_hidden_layers, P = a.grid.n_points;
    const TailLayout TL = tail_layout(a.n_cut_nodes, SMEM_CUT, n_in, H);
    float4 *s_nodes = reinterpret_cast<float4 *>(smem_raw);
    float2 *s_bounds = reinterpret_cast<float2 *>(smem_raw + a.n_cut_nodes * 32u);
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
    GridParams &gp = *reinterpret_cast<GridParams *>(smem_raw + TL.gp_off);
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&a.grid);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&gp);
        for (uint32_t i = threadIdx.x; i < sizeof(GridParams) / 4u; i += blockDim.x)
            dst[i] = src[i];
    }
    __half *sw = reinterpret_cast<__half *>(smem_raw + TL.w_off);
    load_weights_to_smem(a.weights, sw, n_in, H);
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
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, tig = lane & 3;
    unsigned char *wbase = smem_raw + TL.warp_off + (size_t)warp * TL.warp_bytes;
    __half *feat = reinterpret_cast<__half *>(wbase);
    float4 *ends = reinterpret_cast<float4 *>(wbase + TL.ends_off); // [row][2]
    float *outs = reinterpret_cast<float *>(wbase + TL.outs_off);   // [row][8]
    float2 *segs = reinterpret_cast<float2 *>(wbase + TL.segs_off) + lane * kTailMaxAhead; // this lane's

    const NeuralConsts &nc = a.nc;
    const float thr = nc.visibility_threshold;
    const V3 smin = mk3(nc.scene_min[0], nc.scene_min[1], nc.scene_min[2]);
    const V3 smax = mk3(nc.scene_max[0], nc.scene_max[1], nc.scene_max[2]);
    const float dilation = __fadd_rn(__fadd_rn(1.0f, nc.node_extent_dilation), nc.fixed_node_dilation);
    const V3 ext = scale3(sub3(smax, smin), dilation);
    const V3 center = scale3(add3(smax, smin), 0.5f);
    const WaveList &in = a.lists[it & 1u];
    uint32_t *head = &a.wave_counts[4u + it % 3u];
    const bool sorted = a.perm != nullptr && count_in >= kSortMinRows;
    const bool ahead_ok = a.grid.segment_distribution != NBVH_SEGMENT_UNIFORM && a.non_neural == nullptr;
    uint32_t st_segments = 0, st_capped = 0, st_overflow = 0, st_fallback = 0;

    // Rays that need many more segments cluster in space, and so in the node-sorted list: handing
    // out consecutive rows would leave a few warps with 32 long rays each. Rows are dealt in
    // transposed order instead (claim i -> row (i mod 32) * R + i / 32), so each warp gets rays
    // from 32 places of the list.
    const uint32_t deal_rows = (count_in + 31u) / 32u, deal_total = 32u * deal_rows;
    RayState s;
    uint32_t stack[kNeuralStackSize];
    uint32_t snap[kTailMaxAhead - 1u][kNeuralStackSize]; // stack after listing segment j (j < ahead - 1)
    int snap_sp[kTailMaxAhead - 1u];
    RayDiv rdiv;
    bool cull_ok = false, active = false, exhausted = false;
    uint32_t npend = 0;  // segments listed for this round (the loaded row brings one)
    for (;;) {
        // refill: lanes without a ray take the next rows of the list (node order when sorted)
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle != 0u && !exhausted) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(head, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            exhausted = base + (uint32_t)__popc(idle) >= deal_total;
            const uint32_t c = base + __popc(idle & ((1u << lane) - 1u));
            const uint32_t i = (c & 31u) * deal_rows + (c >> 5);
            if (!active && c < deal_total && i < count_in) {
                load_state(in, sorted ? a.perm[i] : i, s, stack);
                active = true;
                cull_ok = s.d.x != 0.0f && s.d.y != 0.0f && s.d.z != 0.0f;
                rdiv = make_raydiv(s.o, s.d, nc.fast_div_ok != 0u);
                segs[0] = make_float2(s.seg_mint, s.seg_maxt);
                npend = 1;
            }
        }
        const unsigned live0 = __ballot_sync(kFull, active);
        if (live0 == 0u) {
            if (exhausted)
                break;
            continue;
        }
        // list this round's segments: one, or more ahead once the warp thins out
        uint32_t want = 1u;
        if (ahead_ok && exhausted)
            want = min(kTailMaxAhead, 32u / (uint32_t)__popc(live0));
        bool trav_end = false; // the traversal found no further leaf (res = 0) or overflowed (res < 0)
        int trav_res = 1;
        while (active && npend < want && !trav_end && s.sp > 0) {
            if (npend > 0u) { // the stack as it was right after listing segment npend - 1
                for (int k = 0; k < s.sp; k++)
                    snap[npend - 1u][k] = stack[k];
                snap_sp[npend - 1u] = s.sp;
            }
            float mint, maxt;
            uint32_t node;
            const int res = neural_intersect_inference(cut, nc.bvh_lod, s.o, rdiv, cull_ok, stack, s.sp,
                                                       nc.inference_mint_epsilon, nc.inference_maxt_epsilon, s.best_t,
                                                       mint, maxt, node);
            if (res == 1) {
                if (a.non_neural && a.non_neural[node]) { // only with npend == 0 (no listing ahead)
                    finish_hit(a, it, s.ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, s.flags & ~NBVH_HIT_VALID,
                               s.segments);
                    const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                    a.fallback_list[slot] = s.ray_id;
                    st_fallback++;
                    active = false;
                    break;
                }
                segs[npend++] = make_float2(mint, maxt);
            } else {
                trav_end = true;
                trav_res = res;
            }
        }
        if (active && npend == 0u) { // nothing left to evaluate: the ray is answered
            if (trav_res < 0) {
                s.flags |= 0x8u;
                st_overflow++;
            }
            const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
            finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                       s.segments);
            active = false;
        }
        // rows of this round: each live lane's segments, consecutive
        const uint32_t mine = active ? npend : 0u;
        uint32_t row0 = mine;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, row0, off);
            if (lane >= off)
                row0 += v;
        }
        const uint32_t rows = __shfl_sync(kFull, row0, 31);
        row0 -= mine;
        if (rows == 0u)
            continue;
        for (uint32_t j = 0; j < mine; j++) {
            float ta = segs[j].x, tb = segs[j].y;
            if (ta < 0.0f) { // encode_bvh_network_input_data swaps for a negative mint
                const float t = ta;
                ta = tb;
                tb = t;
            }
            const V3 epo = encode_world(ray_at(s.o, s.d, ta), center, ext);
            const V3 epi = encode_world(ray_at(s.o, s.d, tb), center, ext);
            ends[2u * (row0 + j)] = make_float4(epo.x, epo.y, epo.z, __uint_as_float(s.rng));
            ends[2u * (row0 + j) + 1u] = make_float4(epi.x, epi.y, epi.z, 0.f);
        }
        __syncwarp();
        for (uint32_t tile = 0; tile * 16u < rows; tile++) {
            const uint32_t n_t = min(16u, rows - tile * 16u);
            const uint32_t mask = n_t >= 16u ? 0xFFFFu : ((1u << n_t) - 1u);
            auto pos = [&](uint32_t r, uint32_t p) -> V3 {
                const float4 e0 = ends[2u * (16u * tile + r)], e1 = ends[2u * (16u * tile + r) + 1u];
                float t;
                if (gp.segment_distribution == NBVH_SEGMENT_UNIFORM) {
                    uint32_t rng = __float_as_uint(e0.w);
                    for (uint32_t k = 0; k <= p; k++)
                        t = lcg_randomf(rng);
                } else {
                    uint32_t unused = 0;
                    t = segment_t(p, P, gp.segment_distribution, unused);
                }
                return segment_point(mk3(e0.x, e0.y, e0.z), mk3(e1.x, e1.y, e1.z), t);
            };
            encode_tile_any<BF16>(a.table, gp, pos, mask, feat, TL.fld);
            float o4[4];
            mlp_tile_from_smem<BF16, FP8>(sw, feat, TL.fld, n_in, H, o4);
            float *ob = outs + 16u * tile * 8u;
            ob[g * 8u + tig * 2u] = o4[0];
            ob[g * 8u + tig * 2u + 1u] = o4[1];
            ob[(g + 8u) * 8u + tig * 2u] = o4[2];
            ob[(g + 8u) * 8u + tig * 2u + 1u] = o4[3];
            __syncwarp();
        }
        // decode the listed segments in order
        bool finished = false, rewound = false;
        for (uint32_t j = 0; j < mine && !finished; j++) {
            const float mint = segs[j].x, maxt = segs[j].y;
            if (j > 0u && !(mint < s.best_t))
                continue; // beyond the closest hit accepted since it was listed: never entered
            if (s.segments > nc.max_traversal_steps) { // step cap (path_module.cu:68, last_inference)
                s.flags |= NBVH_HIT_STEP_CAP;
                st_capped++;
                const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                           s.segments);
                finished = true;
                break;
            }
            if (a.grid.segment_distribution == NBVH_SEGMENT_UNIFORM)
                for (uint32_t k = 0; k < P; k++) // the draws the encoder made for this segment
                    (void)lcg_randomf(s.rng);
            float o8[8];
#pragma unroll
            for (int c = 0; c < 8; c++)
                o8[c] = outs[(row0 + j) * 8u + (uint32_t)c];
            s.segments++;
            st_segments++;
            if (nc.fallback_margin > 0.0f && fabsf(__fsub_rn(o8[0], thr)) < nc.fallback_margin) {
                finish_hit(a, it, s.ray_id, FLT_MAX, mk3(0, 0, 0), mk3(0, 0, 0), 0.f, s.flags & ~NBVH_HIT_VALID,
                           s.segments);
                const uint32_t slot = atomicAdd(&a.counters->fallback_count, 1u);
                a.fallback_list[slot] = s.ray_id;
                st_fallback++;
                finished = true;
                break;
            }
            // process_neural_bvh_traversal_step, path_inference_kernels.cu:61-131
            bool stop = false;
            if (o8[0] > thr) {
                const bool inside = mint < 0.0f;
                if (nc.visibility_only && !inside) {
                    s.flags |= NBVH_HIT_VALID;
                    s.vis = o8[0];
                    stop = true;
                } else {
                    const float de =
                        decode_local_t(o8[1], mint, maxt, inside, nc.depth_epsilon, nc.fixed_depth_epsilon);
                    if (de != FLT_MAX) {
                        if (nc.visibility_only) {
                            s.flags |= NBVH_HIT_VALID;
                            s.vis = o8[0];
                            stop = true;
                        } else if (de < s.best_t) {
                            s.flags |= NBVH_HIT_VALID;
                            s.best_t = de;
                            s.vis = o8[0];
                            s.nrm = normalize3(mk3(__fsub_rn(__fmul_rn(o8[2], 2.0f), 1.0f),
                                                   __fsub_rn(__fmul_rn(o8[3], 2.0f), 1.0f),
                                                   __fsub_rn(__fmul_rn(o8[4], 2.0f), 1.0f)));
                            s.alb = mk3(o8[5], o8[6], o8[7]);
                            if (j + 1u < mine || (j + 1u == mine && trav_end && j < kTailMaxAhead - 1u &&
                                                  want > 1u)) {
                                // a traversal ran past this segment with the old bound: drop what it
                                // listed and resume from the stack as it was after this segment
                                for (int k = 0; k < snap_sp[j]; k++)
                                    stack[k] = snap[j][k];
                                s.sp = snap_sp[j];
                                trav_end = false;
                                trav_res = 1;
                                if (s.sp == 0) {
                                    const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                                    finish_hit(a, it, s.ray_id, s.best_t, s.nrm, s.alb, valid ? s.vis : 0.f,
                                               s.flags, s.segments);
                                    finished = true;
                                }
                                rewound = true;
                                break;
                            }
                        }
                    }
                }
            }
            if (stop || (j + 1u == mine && (trav_end || s.sp == 0))) {
                // answered: a visibility stop, or the last listed segment with no leaf after it
                if (!stop && trav_res < 0) {
                    s.flags |= 0x8u;
                    st_overflow++;
                }
                const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
                finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                           s.segments);
                finished = true;
            }
        }
        if (active && !finished && !rewound && mine > 0u && (trav_end || s.sp == 0)) {
            // every listed segment after the last one decoded lay beyond the closest hit, and the
            // traversal had already ended: the ray is answered
            if (trav_res < 0) {
                s.flags |= 0x8u;
                st_overflow++;
            }
            const bool valid = (s.flags & NBVH_HIT_VALID) != 0u;
            finish_hit(a, it, s.ray_id, valid ? s.best_t : FLT_MAX, s.nrm, s.alb, valid ? s.vis : 0.f, s.flags,
                       s.segments);
            finished = true;
        }
        if (finished)
            active = false;
        npend = 0;
        __syncwarp();
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

constexpr size_t kSmemLimit = (size_t)kMaxDynamicSmem;
constexpr uint32_t kStepsPerCheck = 4;

template <bool SMEM_CUT, bool BF16, bool FP8>
cudaError_t launch_tail_variant(const WaveArgs &a, uint32_t it, int num_sms, bool configure, size_t smem,
                                cudaStream_t s)
{
    if (configure) {
        cudaError_t e = allow_max_dynamic_smem(k_wave_tail<SMEM_CUT, BF16, FP8>);
        if (e != cudaSuccess)
            return e;
    }
    k_wave_tail<SMEM_CUT, BF16, FP8><<<(uint32_t)num_sms * (SMEM_CUT ? 1u : 2u), kTailThreads, smem, s>>>(a, it);
    return cudaGetLastError();
}

cudaError_t launch_tail(const WaveArgs &a, uint32_t it, int num_sms, bool configure, bool stage_cut,
                        cudaStream_t s)
{
    const TailLayout staged = tail_layout(a.n_cut_nodes, true, a.grid.n_inputs, a.n_hidden_layers);
    const TailLayout global = tail_layout(a.n_cut_nodes, false, a.grid.n_inputs, a.n_hidden_layers);
    const bool smem_cut = stage_cut && staged.total <= kMaxDynamicSmem;
    const size_t smem = smem_cut ? staged.total : global.total;
    if (a.bf16)
        return smem_cut ? launch_tail_variant<true, true, false>(a, it, num_sms, configure, smem, s)
                        : launch_tail_variant<false, true, false>(a, it, num_sms, configure, smem, s);
    if (a.prec == NBVH_PRECISION_FP8)
        return smem_cut ? launch_tail_variant<true, false, true>(a, it, num_sms, configure, smem, s)
                        : launch_tail_variant<false, false, true>(a, it, num_sms, configure, smem, s);
    return smem_cut ? launch_tail_variant<true, false, false>(a, it, num_sms, configure, smem, s)
                    : launch_tail_variant<false, false, false>(a, it, num_sms, configure, smem, s);
}

// The kernels of steps [it0, it1): sort, K3, K4, K2 per step, no host synchronisation.
template <bool SMEM_CUT>
cudaError_t enqueue_steps(const WaveArgs &a, const StepResources &r, size_t dec_smem, int num_sms, uint32_t it0,
                          uint32_t it1, cudaStream_t s, uint32_t &launches)
{
    cudaError_t e = cudaSuccess;
    const uint32_t F = a.grid.n_features;
    const uint32_t enc_per_sm = (r.encode_blocks_per_sm && r.encode_blocks_per_sm <= kEncodeBlocksPerSm)
                                    ? r.encode_blocks_per_sm
                                    : kEncodeBlocksPerSm;
    const uint32_t enc_blocks = (uint32_t)num_sms * enc_per_sm;
    const uint32_t dec_blocks = (uint32_t)num_sms * (SMEM_CUT ? 1u : 2u);
    for (uint32_t it = it0; it < it1; it++) {
        if (it == tail_step(a.n_cut_nodes)) {
            // the rest of the query in one launch; the list counters are cleared after it, so every
            // later check (or the counters a captured graph copies out) reads an empty list
            if (a.perm) {
                k_wave_sort<<<(uint32_t)num_sms, kSortThreads, 3u * a.n_sort_nodes * 4u, s>>>(a, it);
                e = cudaGetLastError();
                if (e != cudaSuccess)
                    return e;
                launches++;
            }
            e = launch_tail(a, it, num_sms, !r.capture_only, r.stage_cut, s);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(a.wave_counts, 0, 3u * sizeof(uint32_t), s);
            if (e != cudaSuccess)
                return e;
            launches++;
            return cudaSuccess;
        }
        if (a.perm) {
            k_wave_sort<<<(uint32_t)num_sms, kSortThreads, 3u * a.n_sort_nodes * 4u, s>>>(a, it);
            e = cudaGetLastError();
            if (e != cudaSuccess)
                return e;
            launches++;
        }
        const bool prof = r.prof && !r.capture_only && r.prof->used + 2u <= 2u * kMaxProfiledLaunches;
        if (prof && (e = cudaEventRecord(r.prof->ev[r.prof->used], s)) != cudaSuccess)
            return e;
        if (F == 4u)
            k_wave_encode<4><<<enc_blocks, kEncodeThreads, 0, s>>>(a, it);
        else if (F == 8u)
            k_wave_encode<8><<<enc_blocks, kEncodeThreads, 0, s>>>(a, it);
        else
            k_wave_encode<2><<<enc_blocks, kEncodeThreads, 0, s>>>(a, it);
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        if (prof) {
            if ((e = cudaEventRecord(r.prof->ev[r.prof->used + 1u], s)) != cudaSuccess)
                return e;
            r.prof->used += 2u;
        }
        e = launch_mlp_tc(r.feature_map, r.wpacked, a.grid.n_inputs, a.n_hidden_layers, a.lists[0].capacity,
                          &a.wave_counts[it % 3u], a.outputs, &a.wave_counts[3], a.prec, num_sms, s,
                          !r.capture_only, r.wait_ns, r.stall);
        if (e != cudaSuccess)
            return e;
        k_wave_decode<SMEM_CUT><<<dec_blocks, decode_threads(SMEM_CUT), dec_smem, s>>>(a, it);
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        launches += 3u;
        if (r.drain_host && it == r.drain_step) {
            // early copy of every record to the host on the copy stream, overlapping the later
            // steps; the rays finishing after this point are listed and rewritten at the end
            e = cudaEventRecord(r.drain_snap, s);
            if (e == cudaSuccess)
                e = cudaStreamWaitEvent(r.drain_stream, r.drain_snap, 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(r.drain_host, a.hits, (size_t)a.n * sizeof(nbvh_neural_hit), cudaMemcpyDefault,
                                    r.drain_stream);
            if (e == cudaSuccess)
                e = cudaEventRecord(r.drain_done, r.drain_stream);
            if (e != cudaSuccess)
                return e;
            *r.drain_taken = true;
        }
    }
    return cudaSuccess;
}

// Copies the wave counters to the host words and waits for them; 1 if the list of step `it` is
// empty (the query is done), 0 if not, or an error (cudaErrorTimeout if the MLP's bounded wait
// gave up).
cudaError_t check_done(const WaveArgs &a, const StepResources &r, uint32_t it, cudaStream_t s, bool &done)
{
    cudaError_t e = cudaMemcpyAsync(r.h_words, a.wave_counts, 4u * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess)
        return e;
    if (r.ev) {
        e = cudaEventRecord(r.ev, s);
        if (e == cudaSuccess)
            e = cudaEventSynchronize(r.ev);
    } else {
        e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess)
        return e;
    if (r.h_words[3] != 0u)
        return cudaErrorTimeout;
    done = r.h_words[it % 3u] == 0u;
    return cudaSuccess;
}

// The step loop from step `from` (after `unchecked` steps launched without a host check when from
// is 0): batches of kStepsPerCheck steps, the host reading the list length after each batch. The
// loop ends when a list comes out empty or at the step cap (each ray at most
// max_traversal_steps + 1 segments) plus the final capping step. With capture_only the unchecked
// steps and the copy of the counters are only enqueued (for stream capture) and nothing waits.
template <bool SMEM_CUT>
cudaError_t run_steps(const WaveArgs &a, const StepResources &r, size_t dec_smem, int num_sms, uint32_t max_steps,
                      uint32_t from, cudaStream_t s, uint32_t &launches)
{
    cudaError_t e = cudaSuccess;
    if (!r.capture_only) { // kernel attributes are set outside stream capture (an earlier run set them)
        e = allow_max_dynamic_smem(k_wave_decode<SMEM_CUT>);
        if (e == cudaSuccess && a.perm)
            e = allow_max_dynamic_smem(k_wave_sort);
        if (e != cudaSuccess)
            return e;
    }
    const uint32_t limit = max_steps + 2u;
    uint32_t it = from;
    if (from == 0u && r.unchecked_steps > 0u) {
        const uint32_t u = r.unchecked_steps < limit ? r.unchecked_steps : limit;
        e = enqueue_steps<SMEM_CUT>(a, r, dec_smem, num_sms, 0u, u, s, launches);
        if (e != cudaSuccess)
            return e;
        it = u;
        if (r.capture_only)
            return cudaMemcpyAsync(r.h_words, a.wave_counts, 4u * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        bool done = false;
        e = check_done(a, r, it, s, done);
        if (e != cudaSuccess || done)
            return e;
    }
    while (it < limit) {
        const uint32_t batch = (limit - it) < kStepsPerCheck ? (limit - it) : kStepsPerCheck;
        e = enqueue_steps<SMEM_CUT>(a, r, dec_smem, num_sms, it, it + batch, s, launches);
        if (e != cudaSuccess)
            return e;
        it += batch;
        bool done = false;
        e = check_done(a, r, it, s, done);
        if (e != cudaSuccess || done)
            return e;
    }
    return cudaSuccess;
}

} // namespace

cudaError_t launch_ray_order(const nbvh_ray *rays, uint32_t n, const float scene_min[3], const float scene_max[3],
                             uint16_t *keys, uint32_t *bins, uint32_t *order, int num_sms, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    RayBinArgs rb;
    rb.rays = rays;
    rb.n = n;
    float lo[3], sc[3];
    for (int k = 0; k < 3; k++) {
        const float ext = scene_max[k] - scene_min[k];
        lo[k] = scene_min[k] - 0.5f * ext;
        sc[k] = ext > 0.f ? 4.0f / ext : 0.f; // 8 cells over twice the extent
    }
    rb.lo.x = lo[0], rb.lo.y = lo[1], rb.lo.z = lo[2];
    rb.scale.x = sc[0], rb.scale.y = sc[1], rb.scale.z = sc[2];
    rb.keys = keys;
    rb.bins = bins;
    rb.order = order;
    const uint32_t blocks = (uint32_t)num_sms;
    cudaError_t e = cudaMemsetAsync(bins, 0, kRayBins * sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return e;
    k_ray_bins<<<blocks, kRayBinThreads, 0, s>>>(rb);
    k_ray_bin_scan<<<1, 1024, 0, s>>>(bins);
    k_ray_bin_place<<<blocks, kRayBinThreads, 0, s>>>(rb);
    return cudaGetLastError();
}

cudaError_t configure_query_kernels()
{
    const cudaError_t es[] = {
        allow_max_dynamic_smem(k_wave_decode<true>),          allow_max_dynamic_smem(k_wave_decode<false>),
        allow_max_dynamic_smem(k_wave_tail<true, false, false>), allow_max_dynamic_smem(k_wave_tail<false, false, false>),
        allow_max_dynamic_smem(k_wave_tail<true, true, false>),  allow_max_dynamic_smem(k_wave_tail<false, true, false>),
        allow_max_dynamic_smem(k_wave_tail<true, false, true>),  allow_max_dynamic_smem(k_wave_tail<false, false, true>),
        allow_max_dynamic_smem(k_wave_sort), configure_mlp_tc()};
    for (cudaError_t e : es)
        if (e != cudaSuccess)
            return e;
    return cudaSuccess;
}

cudaError_t launch_wave_query(const float4 *dilated_nodes, const float4 *bounds, uint32_t n_cut_nodes,
                              const uint8_t *non_neural, const __half *params_h, const GridParams &grid,
                              const NeuralConsts &nc, uint32_t n_hidden_layers, const nbvh_ray *rays, uint32_t n,
                              nbvh_neural_hit *hits, QueryCounters *counters, uint32_t *fallback_list,
                              const WaveList lists[2], uint32_t *wave_counts, const StepResources &res, uint32_t prec,
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
    a.features = res.features;
    a.outputs = res.outputs;
    const bool keyed = res.sort_key != nullptr && res.n_sort_bins > 0u;
    const uint32_t n_bins = keyed ? res.n_sort_bins : n_cut_nodes;
    a.sort_key = keyed ? res.sort_key : nullptr;
    // octant sub-bins where the caller sized the count buffers for them, the sort's three
    // shared-memory arrays of 8 x n_bins words fit, and each row has enough point-levels to gather
    // for the encoder's better locality to outweigh the sort's extra reads (measured on GB300: 4
    // points x 16 levels 3.35 -> 3.31 ms per 2^22-ray query; 3 points x 8 levels 2.32 -> 2.37 ms)
    a.sub_bins = (res.sub_bins && (size_t)3u * 4u * kSubBins * n_bins <= (size_t)kMaxDynamicSmem &&
                  grid.n_points * grid.n_levels >= kSubBinMinPointLevels)
                     ? 1u
                     : 0u;
    a.n_sort_nodes = a.sub_bins ? kSubBins * n_bins : n_bins;
    a.bf16 = prec == NBVH_PRECISION_BF16 ? 1u : 0u;
    a.prec = prec;
    const bool sort = res.perm != nullptr && n_bins <= kMaxSortNodes;
    a.perm = sort ? res.perm : nullptr;
    a.row_keys = (sort && a.n_sort_nodes <= 65536u) ? res.row_keys : nullptr;
    a.ray_order = nullptr;
    a.node_bins = res.node_bins;
    a.node_cursor = res.node_cursor;
    a.n_hidden_layers = n_hidden_layers;
    a.n = n;
    a.n_cut_nodes = n_cut_nodes;
    a.visits = res.visits_per_round ? res.visits_per_round : kDefaultVisitsPerRound;
    a.late_list = res.late_list;
    a.late_count = res.late_count;
    a.late_from = res.drain_host ? res.drain_step + 1u : 0xFFFFFFFFu;
    const size_t smem_cut = (size_t)n_cut_nodes * 56u;
    const bool use_smem_cut = res.stage_cut && smem_cut <= kSmemLimit;
    if (res.resume_from > 0u) // continue a query whose first steps ran from a captured graph
        return use_smem_cut
                   ? run_steps<true>(a, res, smem_cut, num_sms, nc.max_traversal_steps, res.resume_from, s, *launches)
                   : run_steps<false>(a, res, 0, num_sms, nc.max_traversal_steps, res.resume_from, s, *launches);
    // words 0-2: rotating list lengths; 3: the MLP's error word; 4-6: rotating work counters of
    // the decode kernel; 7: work counter of the first pass
    cudaError_t e = cudaMemsetAsync(wave_counts, 0, 8u * sizeof(uint32_t), s);
    if (e == cudaSuccess && res.drain_host)
        e = cudaMemsetAsync(res.late_count, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return e;
    if (sort) {
        e = cudaMemsetAsync(res.node_bins, 0, 2u * a.n_sort_nodes * sizeof(uint32_t), s);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(res.node_cursor, 0, 2u * a.n_sort_nodes * sizeof(uint32_t), s);
        if (e != cudaSuccess)
            return e;
    }
    e = launch_pack_weights(params_h, grid.n_inputs, n_hidden_layers, res.wpacked, s);
    if (e != cudaSuccess)
        return e;
    *launches = 2;
    if (res.ray_keys && res.ray_bins && res.perm && n >= kRaySortMin) {
        // the first pass takes the rays bin by bin (its list rows are re-sorted by node afterwards,
        // so the buffer of the node order holds the ray order until then)
        e = launch_ray_order(rays, n, nc.scene_min, nc.scene_max, res.ray_keys, res.ray_bins, res.perm, num_sms, s);
        if (e != cudaSuccess)
            return e;
        a.ray_order = res.perm;
        *launches += 3u;
    }
    uint32_t first_blocks = (n + kFirstThreads - 1u) / kFirstThreads;
    const uint32_t first_cap = (uint32_t)num_sms * 4u; // resident blocks (64 registers a thread)
    if (first_blocks > first_cap)
        first_blocks = first_cap;
    k_wave_first<<<first_blocks, kFirstThreads, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    if (use_smem_cut)
        return run_steps<true>(a, res, smem_cut, num_sms, nc.max_traversal_steps, 0u, s, *launches);
    return run_steps<false>(a, res, 0, num_sms, nc.max_traversal_steps, 0u, s, *launches);
}

namespace {

// The records of the rays listed as finishing after the early host copy, copied to the host. All
// records are final in src by now, so the whole 64-byte lines a listed record touches are copied:
// four threads write one line with 16-byte stores, and the host link receives full lines instead
// of the 48-byte partial writes of single records (several times slower on the link).
__global__ void __launch_bounds__(256) k_copy_late(const uint32_t *__restrict__ late, const uint32_t *late_count,
                                                   uint32_t n, const nbvh_neural_hit *__restrict__ src,
                                                   nbvh_neural_hit *dst)
{
    const uint32_t count = min(*late_count, n);
    const size_t total = (size_t)n * sizeof(nbvh_neural_hit);
    const unsigned char *in = reinterpret_cast<const unsigned char *>(src);
    unsigned char *out = reinterpret_cast<unsigned char *>(dst);
    for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < (size_t)count * 8u;
         w += (size_t)gridDim.x * blockDim.x) {
        const uint32_t id = late[w >> 3], sub = (uint32_t)(w & 7u);
        const size_t first = (size_t)id * sizeof(nbvh_neural_hit);
        const size_t line = (first >> 6) + (sub >> 2);
        if (line > ((first + sizeof(nbvh_neural_hit) - 1u) >> 6))
            continue;
        const size_t off = line * 64u + (sub & 3u) * 16u;
        if (off + 16u <= total)
            *reinterpret_cast<float4 *>(out + off) = *reinterpret_cast<const float4 *>(in + off);
    }
}

} // namespace

cudaError_t launch_copy_late(const uint32_t *late, const uint32_t *late_count, uint32_t n, const nbvh_neural_hit *src,
                             nbvh_neural_hit *dst, int num_sms, cudaStream_t s)
{
    k_copy_late<<<(uint32_t)num_sms * 4u, 256, 0, s>>>(late, late_count, n, src, dst);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Fixed scratch of the allocation-free query: a file-scope device array, so the CUDA runtime
// creates one copy per device when it loads this module and no call allocates it.
// ---------------------------------------------------------------------------------------------

namespace {
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];
} // namespace

// The buffer on `device`, which the caller has made current. Its address is looked up on every
// call (the lookup allocates nothing): a module that the runtime loads again after a device reset
// places the buffer anew, and a handle created after the reset must not use the old address.
cudaError_t noalloc_scratch(int device, NoallocScratch *out)
{
    if (device < 0)
        return cudaErrorInvalidDevice;
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess)
        return e;
    unsigned char *p = static_cast<unsigned char *>(addr);
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
    out->features = reinterpret_cast<__half *>(p);
    p += kNoallocFeatureBytes;
    out->outputs = reinterpret_cast<float *>(p);
    p += kNoallocOutputBytes;
    out->wpacked = reinterpret_cast<__half *>(p);
    p += kNoallocWeightBytes;
    out->perm = reinterpret_cast<uint32_t *>(p);
    out->node_bins = out->perm + n;
    out->node_cursor = out->node_bins + 2u * kMaxSortNodes;
    p += kNoallocSortBytes;
    out->fallback_list = reinterpret_cast<uint32_t *>(p);
    p += n * 4u;
    out->counters = reinterpret_cast<QueryCounters *>(p);
    p += 256u;
    out->wave_counts = reinterpret_cast<uint32_t *>(p);
    return cudaSuccess;
}

} // namespace nbvh
