// k_tree_cut.cu -- learned tree cut on the device: per-node loss accounting, the per-step
// heuristic maximum that drives node survival, the top-k selection of the leaves to split and the
// split itself, and the LoD assignment of the current leaves.
//
// Reference: the tree-cut part of NeuralBVHRenderer::render (src/cuda/neural/neural_bvh_renderer.cu:
// 196-282) -- update_neural_tree_cut_loss and k + 1 launches of update_neural_tree_cut_decisions
// (src/cuda/neural/neural_bvh_renderer_kernels.cu:202-287), a device-to-host copy of the selection,
// then split_neural_bvh_at / assign_lod_to_current_neural_leaf_nodes on the host with uploads
// (src/cuda/neural/neural_bvh_renderer_accel.cpp:256-441). Here the selection is one radix select
// in a single block and the split is done in the same kernel, so a training step with a split
// needs no host round trip: the node count lives on the device and every kernel reads it there.
#include <cfloat>

#include "device_math.cuh"
#include "nbvh_internal.h"

namespace nbvh {

namespace {

constexpr uint32_t kSplitThreads = 1024;
constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t node_prim(const float4 *nodes, uint32_t i)
{
    return __float_as_uint(nodes[2u * i].w);
}

__device__ __forceinline__ uint32_t node_left(const float4 *nodes, uint32_t i)
{
    return __float_as_uint(nodes[2u * i + 1u].w);
}

// Key of a split candidate: the heuristic's bits when it is positive (positive floats order as
// unsigned integers), 0 for everything that cannot be split (interior nodes, final leaves, nodes
// whose classic node is a leaf).
__device__ __forceinline__ uint32_t split_key(const TreeCutArgs &a, const uint4 *stats, uint32_t i)
{
    if (node_left(a.nodes, i) != kNoNeuralChild || node_prim(a.nodes, i) == kLeafFinal)
        return 0u;
    if (__float_as_uint(a.classic[2u * a.node_map[i]].w) != 0u)
        return 0u;
    const uint4 st = stats[i];
    const float hval = tree_cut_heuristic(__uint_as_float(st.x), st.y, st.w);
    return hval > 0.0f ? __float_as_uint(hval) : 0u;
}

// Exclusive prefix sum over the block (1024 threads); *total receives the block sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_tmp, uint32_t *total)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, off);
        if (lane >= (uint32_t)off)
            x += y;
    }
    if (lane == 31u)
        warp_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tmp[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, w, off);
            if (lane >= (uint32_t)off)
                w += y;
        }
        warp_tmp[lane] = w; // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = warp == 0 ? 0u : warp_tmp[warp - 1u];
    *total = warp_tmp[31];
    __syncthreads(); // warp_tmp is reused by the next call
    return before + x - v;
}

// update_neural_tree_cut_loss: the sample's loss (the sum of its output channels' loss values) and
// `dims` samples go to the node the sample was drawn from.
__global__ void __launch_bounds__(256) k_cut_accumulate(const float *__restrict__ sample_loss,
                                                        const uint32_t *__restrict__ sample_nodes, uint32_t n,
                                                        uint32_t dims, uint32_t *stats)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t node = sample_nodes[i];
    atomicAdd(reinterpret_cast<float *>(stats + 4u * node), sample_loss[i]);
    atomicAdd(stats + 4u * node + 3u, dims);
}

// Launch 0 of update_neural_tree_cut_decisions for every leaf: iter_alive + 1; and the maximum
// heuristic of the splittable leaves (floored at 0) into words[slot].
__global__ void __launch_bounds__(256) k_cut_alive_max(const __grid_constant__ TreeCutArgs a, uint32_t slot)
{
    const uint32_t count = *reinterpret_cast<volatile const uint32_t *>(a.words + kCutCount);
    uint32_t best = 0u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        if (node_left(a.nodes, i) != kNoNeuralChild)
            continue;
        uint4 st = reinterpret_cast<uint4 *>(a.stats)[i];
        st.y += 1u;
        a.stats[4u * i + 1u] = st.y;
        if (node_prim(a.nodes, i) == kLeafFinal)
            continue;
        const float hval = tree_cut_heuristic(__uint_as_float(st.x), st.y, st.w);
        if (hval > 0.0f)
            best = max(best, __float_as_uint(hval));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        best = max(best, __shfl_xor_sync(kFull, best, off));
    if ((threadIdx.x & 31u) == 0u && best != 0u)
        atomicMax(a.words + slot, best);
}

// Selection and split in one block. The k splittable leaves with the largest heuristics (ties:
// lower node index first) are found by a radix select over the keys (4 passes of 8 bits), then
// split in ascending node order: the j-th selected node gets children count + 2j and count + 2j + 1
// whose boxes, leaf kinds and classic indices come from the classic BVH (split_neural_bvh_at).
__global__ void __launch_bounds__(kSplitThreads) k_cut_split(const __grid_constant__ TreeCutArgs a, uint32_t k,
                                                             uint32_t lod)
{
    __shared__ uint32_t hist[256];
    __shared__ uint32_t warp_tmp[32];
    __shared__ uint32_t s_prefix, s_remaining;
    const uint32_t tid = threadIdx.x;
    const uint32_t count = a.words[kCutCount];
    const uint4 *stats4 = reinterpret_cast<const uint4 *>(a.stats);
    for (uint32_t b = tid; b < 256u; b += kSplitThreads)
        hist[b] = 0u;
    __syncthreads();
    uint32_t eligible_local = 0;
    for (uint32_t i = tid; i < count; i += kSplitThreads) {
        const uint32_t key = split_key(a, stats4, i);
        a.keys[i] = key;
        if (key != 0u) {
            eligible_local++;
            atomicAdd(&hist[key >> 24], 1u);
        }
    }
    uint32_t eligible;
    (void)block_exclusive_scan(eligible_local, warp_tmp, &eligible);

    // threshold: every key above `thresh` is taken, plus the first `need_eq` keys equal to it
    uint32_t thresh = 0u, need_eq = 0u;
    if (eligible > k) {
        if (tid == 0) {
            s_prefix = 0u;
            s_remaining = k;
        }
        for (int d = 3; d >= 0; d--) {
            const uint32_t shift = 8u * (uint32_t)d;
            if (d < 3) {
                __syncthreads();
                for (uint32_t b = tid; b < 256u; b += kSplitThreads)
                    hist[b] = 0u;
                __syncthreads();
                const uint32_t prefix = s_prefix, hi = shift + 8u;
                for (uint32_t i = tid; i < count; i += kSplitThreads) {
                    const uint32_t key = a.keys[i];
                    if (key != 0u && (key >> hi) == (prefix >> hi))
                        atomicAdd(&hist[(key >> shift) & 255u], 1u);
                }
            }
            __syncthreads();
            if (tid == 0) {
                uint32_t above = 0u;
                for (int b = 255; b >= 0; b--) {
                    if (above + hist[b] >= s_remaining) {
                        s_prefix |= (uint32_t)b << shift;
                        s_remaining -= above;
                        break;
                    }
                    above += hist[b];
                }
            }
            __syncthreads();
        }
        thresh = s_prefix;
        need_eq = s_remaining;
    }
    const uint32_t m = eligible > k ? k : eligible;
    if (m == 0u)
        return;
    if (count + 2u * m > a.capacity) {
        if (tid == 0)
            a.words[kCutError] = 1u;
        return;
    }

    uint32_t eq_base = 0u, sel_base = 0u;
    for (uint32_t c0 = 0; c0 < count; c0 += kSplitThreads) {
        const uint32_t i = c0 + tid;
        const uint32_t key = i < count ? a.keys[i] : 0u;
        const uint32_t is_eq = (need_eq != 0u && key != 0u && key == thresh) ? 1u : 0u;
        uint32_t eq_total;
        const uint32_t eq_rank = eq_base + block_exclusive_scan(is_eq, warp_tmp, &eq_total);
        const bool sel = key != 0u && (key > thresh || (is_eq && eq_rank < need_eq));
        uint32_t sel_total;
        const uint32_t rank = sel_base + block_exclusive_scan(sel ? 1u : 0u, warp_tmp, &sel_total);
        if (sel) {
            const uint32_t left = count + 2u * rank;
            const uint32_t c = a.node_map[i];
            const float4 p0 = a.classic[2u * c], p1 = a.classic[2u * c + 1u];
            const uint32_t cl = __float_as_uint(p1.w);
            const uint32_t depth = a.stats[4u * i + 2u] + 1u;
            for (uint32_t j = 0; j < 2u; j++) {
                const uint32_t nj = left + j, cj = cl + j;
                const float4 c0v = a.classic[2u * cj], c1v = a.classic[2u * cj + 1u];
                const uint32_t prim = __float_as_uint(c0v.w) > 0u ? kLeafFinal : kLeafLodBase + lod;
                a.nodes[2u * nj] = make_float4(c0v.x, c0v.y, c0v.z, __uint_as_float(prim));
                a.nodes[2u * nj + 1u] = make_float4(c1v.x, c1v.y, c1v.z, __uint_as_float(kNoNeuralChild));
                reinterpret_cast<uint4 *>(a.stats)[nj] = make_uint4(0u, 1u, depth, 0u);
                a.node_map[nj] = cj;
            }
            uint32_t prim = node_prim(a.nodes, i);
            if (prim == kLeafLodBase + lod)
                prim = 0u;
            a.nodes[2u * i] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(prim));
            a.nodes[2u * i + 1u] = make_float4(p1.x, p1.y, p1.z, __uint_as_float(left));
            atomicMax(a.words + kCutMaxDepth, depth);
        }
        eq_base += eq_total;
        sel_base += sel_total;
    }
    if (tid == 0) {
        a.words[kCutCount] = count + 2u * sel_base;
        a.words[kCutSplits] += sel_base;
    }
}

// assign_lod_to_current_neural_leaf_nodes: every node without a neural child becomes a leaf of
// LoD `lod` unless it is a final leaf (nothing changes when lod is the coarsest LoD).
__global__ void __launch_bounds__(256) k_cut_assign_lod(const __grid_constant__ TreeCutArgs a, uint32_t lod)
{
    const uint32_t count = a.words[kCutCount];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        if (node_left(a.nodes, i) != kNoNeuralChild)
            continue;
        const uint32_t prim = node_prim(a.nodes, i) == kLeafFinal ? kLeafFinal : kLeafLodBase + lod;
        a.nodes[2u * i].w = __uint_as_float(prim);
    }
}

} // namespace

cudaError_t launch_cut_accumulate(const float *sample_loss, const uint32_t *sample_nodes, uint32_t n, uint32_t dims,
                                  uint32_t *stats, cudaStream_t s)
{
    if (n == 0)
        return cudaSuccess;
    k_cut_accumulate<<<(n + 255u) / 256u, 256, 0, s>>>(sample_loss, sample_nodes, n, dims, stats);
    return cudaGetLastError();
}

cudaError_t launch_cut_alive_max(const TreeCutArgs &a, uint32_t slot, int num_sms, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(a.words + slot, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return e;
    uint32_t blocks = (a.capacity + 255u) / 256u;
    const uint32_t cap = (uint32_t)num_sms * 4u;
    if (blocks > cap)
        blocks = cap;
    k_cut_alive_max<<<blocks > 0 ? blocks : 1u, 256, 0, s>>>(a, slot);
    return cudaGetLastError();
}

cudaError_t launch_cut_split(const TreeCutArgs &a, uint32_t k, uint32_t lod, cudaStream_t s)
{
    if (k == 0)
        return cudaSuccess;
    k_cut_split<<<1, kSplitThreads, 0, s>>>(a, k, lod);
    return cudaGetLastError();
}

cudaError_t launch_cut_assign_lod(const TreeCutArgs &a, uint32_t lod, int num_sms, cudaStream_t s)
{
    uint32_t blocks = (a.capacity + 255u) / 256u;
    const uint32_t cap = (uint32_t)num_sms * 4u;
    if (blocks > cap)
        blocks = cap;
    k_cut_assign_lod<<<blocks > 0 ? blocks : 1u, 256, 0, s>>>(a, lod);
    return cudaGetLastError();
}

} // namespace nbvh
