// k_mlp_tc.cu -- the fully fused MLP (K4 forward) on the 5th-generation tensor cores.
//
// tcnn's FullyFusedMLP (configured at src/cuda/neural/neural_bvh_module.cu:232-238: 64 neurons,
// ReLU hidden layers, Sigmoid output, no biases, output padded to 16) evaluated on 128-row tiles:
//
//   TMA        one 2-D tensor copy per 8-column slice moves the tile's FP16 inputs from HBM into
//              shared memory, already in the tensor core's K-major core-matrix layout;
//   tcgen05    one thread issues each layer as M=128 x N=64 (N=16 for the output layer) MMAs over
//              K in steps of 16; the FP32 accumulator lives in tensor memory (columns 0-63);
//   epilogue   each of the 4 warps reads its 32 TMEM lanes (= its 32 rows), applies ReLU, rounds to
//              FP16 and writes the next layer's A operand into tensor memory (columns 64-95, two
//              values per column), from where the next MMAs read it; after the output layer it
//              applies the sigmoid and stores 8 FP32 outputs per row.
//
// Only layer 0 reads the input tile in shared memory, so the next tile's copy starts as soon as
// layer 0's MMAs have completed and arrives under the remaining layers. One CTA per SM runs up to
// five such tile pipelines (4 warps, 96 TMEM columns and one input buffer each) side by side, so
// one pipeline's epilogue overlaps the others' MMAs. The weights (about 42 KB) are packed once per
// call into the operand layout and copied to shared memory once per CTA.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "nbvh_internal.h"
#include "net_device.cuh"
#include "tc_device.cuh"

namespace nbvh {

namespace {

constexpr uint32_t kTileRows = 128;
constexpr uint32_t kGroupThreads = 128; // one tile pipeline: 4 warps, one TMEM lane (= tile row) each
constexpr uint32_t kMaxGroups = 5;      // 5 x 96 TMEM columns fit the SM's 512
constexpr uint32_t kGroupCols = 96;     // a group's accumulator in columns [0, 64), activations in [64, 96)
constexpr uint32_t kActCol = 64;
// Shared memory of an SM and the part the runtime reserves per CTA (sm_100 family).
constexpr size_t kSmPerSm = 228u * 1024u;
constexpr size_t kSmemReservedPerCta = 1024u;

// TMEM columns a CTA of `groups` allocates (a power of two, at least 32)
__host__ __device__ constexpr uint32_t tmem_alloc_cols(uint32_t groups)
{
    return groups * kGroupCols <= 128u ? 128u : (groups * kGroupCols <= 256u ? 256u : 512u);
}

// The input tiles follow the weights on a 1,024-byte boundary (the swizzle atoms of the tiles).
__host__ __device__ constexpr uint32_t tile_offset(uint32_t wbytes) { return (wbytes + 1023u) & ~1023u; }

// Feature rows of a multiple of 64 values are copied in 128-byte swizzled boxes (one TMA request
// per 128-byte row segment); other widths in 16-byte boxes (eight times the requests).
__host__ __device__ constexpr bool feature_map_swizzled(uint32_t n_inputs) { return n_inputs % 64u == 0u; }

__host__ __device__ inline uint32_t w0_bytes(uint32_t n_inputs) { return kNeurons * n_inputs * 2u; }
__host__ __device__ inline uint32_t hidden_w_bytes() { return kNeurons * kNeurons * 2u; }
__host__ __device__ inline uint32_t out_w_bytes() { return kOutputsPadded * kNeurons * 2u; }

// FP16 network matrices (network-first parameter order, each [rows][cols] row-major) -> the
// K-major core-matrix operand layout, matrices back to back.
__global__ void k_pack_weights(const __half *__restrict__ w, uint32_t n_inputs, uint32_t n_hidden_layers,
                               __half *__restrict__ packed)
{
    const uint32_t n0 = kNeurons * n_inputs, nh = (n_hidden_layers - 1u) * kNeurons * kNeurons;
    const uint32_t total = n0 + nh + kOutputsPadded * kNeurons;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        uint32_t byte;
        if (i < n0) {
            byte = tc::operand_offset(i / n_inputs, i % n_inputs, kNeurons);
        } else if (i < n0 + nh) {
            const uint32_t j = i - n0, m = j / (kNeurons * kNeurons), e = j % (kNeurons * kNeurons);
            byte = w0_bytes(n_inputs) + m * hidden_w_bytes() + tc::operand_offset(e / kNeurons, e % kNeurons, kNeurons);
        } else {
            const uint32_t e = i - n0 - nh;
            byte = w0_bytes(n_inputs) + (n_hidden_layers - 1u) * hidden_w_bytes() +
                   tc::operand_offset(e / kNeurons, e % kNeurons, kOutputsPadded);
        }
        packed[byte / 2u] = w[i];
    }
}

struct MlpTcArgs {
    const __half *wpacked;
    uint32_t wbytes;
    uint32_t n_inputs;
    uint32_t n_hidden_layers;
    uint32_t n;              // rows of the tensor map
    const uint32_t *d_count; // optional row count produced on the device (min with n)
    float *outputs;
    uint32_t *status;
    uint32_t fp8;    // inputs of the hidden matrices rounded to FP8-E4M3
    uint32_t groups; // tile pipelines per CTA (blockDim.x / 128)
    uint64_t wait_ns; // time limit of the phase waits
    uint32_t stall;   // failure-path test: wait on an mbarrier nothing arrives at (it runs out)
};

// D = A * W^T for the 128-row tile: A (128 x K) at a_addr, W (N x K) at w_addr, both in the
// operand layout; one MMA per 16 values of K.
__device__ __forceinline__ void issue_layer(uint32_t tmem, uint32_t a_addr, uint32_t w_addr, uint32_t k_dim,
                                            uint32_t n_dim, uint32_t idesc)
{
    const uint32_t a_lbo = kTileRows * 16u, b_lbo = n_dim * 16u;
    for (uint32_t k = 0; k < k_dim / 16u; k++) {
        const uint64_t ad = tc::smem_desc(a_addr + 2u * k * a_lbo, a_lbo, 128u);
        const uint64_t bd = tc::smem_desc(w_addr + 2u * k * b_lbo, b_lbo, 128u);
        tc::mma_f16(tmem, ad, bd, idesc, k > 0u ? 1u : 0u);
    }
}

// Layer 0 from an input tile in the 128-byte swizzled layout (inputs a multiple of 64): A (128 x K)
// as K / 64 column blocks of 16 KB, W (N x K) in the unswizzled operand layout.
__device__ __forceinline__ void issue_layer_sw128(uint32_t tmem, uint32_t a_addr, uint32_t w_addr, uint32_t k_dim,
                                                  uint32_t n_dim, uint32_t idesc)
{
    const uint32_t b_lbo = n_dim * 16u;
    for (uint32_t k = 0; k < k_dim / 16u; k++) {
        const uint64_t ad = tc::smem_desc_sw128(a_addr + (k >> 2) * (kTileRows * 128u) + (k & 3u) * 32u);
        const uint64_t bd = tc::smem_desc(w_addr + 2u * k * b_lbo, b_lbo, 128u);
        tc::mma_f16(tmem, ad, bd, idesc, k > 0u ? 1u : 0u);
    }
}

// D = A * W^T with A (128 x K) in tensor memory at column a_col (K / 2 columns), W (N x K) in
// shared memory in the operand layout; one MMA per 16 values of K (8 columns of A).
__device__ __forceinline__ void issue_layer_ta(uint32_t tmem, uint32_t a_col, uint32_t w_addr, uint32_t k_dim,
                                               uint32_t n_dim, uint32_t idesc)
{
    const uint32_t b_lbo = n_dim * 16u;
    for (uint32_t k = 0; k < k_dim / 16u; k++) {
        const uint64_t bd = tc::smem_desc(w_addr + 2u * k * b_lbo, b_lbo, 128u);
        tc::mma_f16_ta(tmem, tmem + a_col + 8u * k, bd, idesc, k > 0u ? 1u : 0u);
    }
}

// Hidden-layer epilogue for this thread's row: 64 accumulator columns -> ReLU -> 16-bit (FP16 or
// BF16) -> the next layer's A operand, 32 columns of this row's lane from column kActCol on.
template <bool BF16, bool FP8>
__device__ __forceinline__ void epilogue_hidden(uint32_t tmem_row, bool quant)
{
    static_assert(!(FP8 && BF16), "FP8 hidden layers run on the FP16 tensor-core path");
    uint32_t v[4][16];
#pragma unroll
    for (int q = 0; q < 4; q++)
        tc::tmem_ld16(tmem_row + 16u * q, v[q]);
    tc::tmem_wait_ld();
    uint32_t packed[32];
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const uint32_t lo = v[j >> 3][(2 * j) & 15], hi = v[j >> 3][(2 * j + 1) & 15];
        if (FP8 && quant) // FP8 mode: the input of a hidden matrix is an E4M3 value (exact in FP16)
            packed[j] = fp8_act_relu_half2(__uint_as_float(lo), __uint_as_float(hi));
        else // ReLU and rounding in one conversion: max(x, 0) rounded to nearest even
            packed[j] = pack_relu<BF16>(__uint_as_float(lo), __uint_as_float(hi));
    }
    tc::tmem_st32(tmem_row + kActCol, packed);
    tc::tmem_wait_st();
}

// Output-layer epilogue: sigmoid of the 8 used output columns of this thread's row.
__device__ __forceinline__ void epilogue_out(uint32_t tmem_row, float (&o)[8])
{
    uint32_t v[8];
    tc::tmem_ld8(tmem_row, v);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 8; i++)
        o[i] = 1.0f / (1.0f + expf(-__uint_as_float(v[i])));
}

// Barrier `id` of the 128 threads of one tile group; the AND of `v` over them.
__device__ __forceinline__ bool group_sync_and(uint32_t id, bool v)
{
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.and.pred q, %2, 128, p;\n"
                 " selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r)
                 : "r"(v ? 1u : 0u), "r"(id)
                 : "memory");
    return r != 0u;
}
__device__ __forceinline__ void group_sync(uint32_t id)
{
    asm volatile("barrier.cta.sync %0, 128;\n" ::"r"(id) : "memory");
}

// One CTA per SM, `groups` independent tile pipelines of 128 threads (4 warps) each. A group owns
// an input tile buffer, 96 TMEM columns, two mbarriers and one issuing thread, and runs its tiles
// layer after layer; the groups interleave on the SM, so one group's epilogue overlaps the others'
// MMAs and copies. The weights are in shared memory once for all groups.
template <bool BF16, bool FP8>
__global__ void __launch_bounds__(kMaxGroups * kGroupThreads, 1) k_mlp_tc(const __grid_constant__ CUtensorMap fmap,
                                                                          const MlpTcArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t K = a.n_inputs, H = a.n_hidden_layers, G = a.groups;
    uint32_t n = a.n;
    if (a.d_count) {
        const uint32_t c = *reinterpret_cast<volatile const uint32_t *>(a.d_count);
        n = c < n ? c : n;
    }
    const uint32_t n_tiles = (n + kTileRows - 1u) / kTileRows;
    if (blockIdx.x >= n_tiles)
        return; // no tile for this CTA: skip TMEM and the weight copy
    const uint32_t tile_bytes = kTileRows * K * 2u;
    const bool sw128 = feature_map_swizzled(K);
    if ((tc::smem_addr(smem) & 1023u) != 0u) { // the swizzled tiles need 1,024-byte aligned atoms
        if (threadIdx.x == 0)
            atomicOr(a.status, 2u);
        return;
    }
    const uint32_t tid = threadIdx.x, gid = tid / kGroupThreads, gtid = tid % kGroupThreads;
    const uint32_t warp = gtid >> 5, row = gtid;
    // the group's issuing thread: lane 0 of warp (gid mod 4), so that the groups' issuers sit on
    // different schedulers; it alone waits on the group's mbarriers, the other warps sleep in the
    // group barrier meanwhile
    const bool issuer = gtid == 32u * (gid & 3u);
    unsigned char *tile = smem + tile_offset(a.wbytes) + gid * tile_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + tile_offset(a.wbytes) + G * tile_bytes);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2u * G + 2u);
    const uint32_t bar_w = tc::smem_addr(&bars[2u * G]);
    const uint32_t bar_load = tc::smem_addr(&bars[2u * gid]), bar_mma = tc::smem_addr(&bars[2u * gid + 1u]);
    const uint32_t w_addr = tc::smem_addr(smem), t_addr = tc::smem_addr(tile);
    const uint32_t gbar = 1u + gid; // named barrier of the group (0 is __syncthreads)

    if (tid < 32u) {
        tc::tmem_alloc(tc::smem_addr(slot), tmem_alloc_cols(G));
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (uint32_t b = 0; b < 2u * G + 2u; b++) // the last one is the failure-path test's
            tc::mbar_init(tc::smem_addr(&bars[b]), 1u);
        tc::mbar_init_fence();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem_all = *slot;
    const uint32_t tmem = tmem_all + gid * kGroupCols;
    const uint32_t tmem_row = tmem + ((32u * warp) << 16);

    auto load_tile = [&](uint32_t t) {
        tc::mbar_expect_tx(bar_load, tile_bytes);
        if (sw128) { // boxes of 64 values (128-byte rows), swizzled
            for (uint32_t c = 0; c < K / 64u; c++)
                tc::tma_load_2d(t_addr + c * kTileRows * 128u, &fmap, (int32_t)(64u * c), (int32_t)(t * kTileRows),
                                bar_load);
        } else { // boxes of 8 values (16-byte rows)
            for (uint32_t c = 0; c < K / 8u; c++)
                tc::tma_load_2d(t_addr + c * kTileRows * 16u, &fmap, (int32_t)(8u * c), (int32_t)(t * kTileRows),
                                bar_load);
        }
    };
    uint32_t ph_load = 0, ph_mma = 0;
    bool load_pending = false, mma_pending = false;
    uint32_t t = blockIdx.x + gid * gridDim.x;
    const uint32_t stride = G * gridDim.x;
    // the group's first tile is on its way while the weights arrive
    if (issuer && t < n_tiles)
        load_tile(t);
    load_pending = t < n_tiles;
    if (tid == 0) {
        tc::mbar_expect_tx(bar_w, a.wbytes);
        for (uint32_t o = 0; o < a.wbytes; o += 16384u)
            tc::bulk_load(w_addr + o, reinterpret_cast<const unsigned char *>(a.wpacked) + o,
                          a.wbytes - o < 16384u ? a.wbytes - o : 16384u, bar_w);
    }
    bool ok = tc::mbar_wait(bar_w, 0u, a.wait_ns);
    if (a.stall && tid == 0) // nothing ever arrives at this barrier: the wait runs out
        ok = ok && tc::mbar_wait(tc::smem_addr(&bars[2u * G + 1u]), 0u, a.wait_ns);
    ok = __syncthreads_and(ok);
    const uint32_t id_hidden = tc::idesc_f16(kTileRows, kNeurons, BF16);
    const uint32_t id_out = tc::idesc_f16(kTileRows, kOutputsPadded, BF16);
    for (; ok && t < n_tiles; t += stride) {
        ok = issuer ? tc::mbar_wait(bar_load, ph_load, a.wait_ns) : true;
        ok = group_sync_and(gbar, ok);
        if (!ok)
            break;
        ph_load ^= 1u;
        load_pending = false;
        for (uint32_t layer = 0; layer <= H; layer++) {
            if (issuer) {
                tc::fence_after_sync();
                if (layer == 0 && sw128)
                    issue_layer_sw128(tmem, t_addr, w_addr, K, kNeurons, id_hidden);
                else if (layer == 0)
                    issue_layer(tmem, t_addr, w_addr, K, kNeurons, id_hidden);
                else if (layer < H)
                    issue_layer_ta(tmem, kActCol, w_addr + w0_bytes(K) + (layer - 1u) * hidden_w_bytes(), kNeurons,
                                   kNeurons, id_hidden);
                else
                    issue_layer_ta(tmem, kActCol, w_addr + w0_bytes(K) + (H - 1u) * hidden_w_bytes(), kNeurons,
                                   kOutputsPadded, id_out);
                tc::mma_commit(bar_mma);
            }
            mma_pending = true;
            ok = issuer ? tc::mbar_wait(bar_mma, ph_mma, a.wait_ns) : true;
            ok = group_sync_and(gbar, ok);
            if (!ok)
                break;
            ph_mma ^= 1u;
            mma_pending = false;
            tc::fence_after_sync();
            if (layer == 0) {
                // layer 0 was the input tile's only reader: start the group's next copy under the
                // remaining layers
                if (issuer && t + stride < n_tiles)
                    load_tile(t + stride);
                load_pending = t + stride < n_tiles;
            }
            if (layer < H) {
                epilogue_hidden<BF16, FP8>(tmem_row, layer + 1u < H);
            } else {
                float o[8];
                epilogue_out(tmem_row, o);
                const uint32_t r = t * kTileRows + row;
                if (r < n) {
                    float4 *dst = reinterpret_cast<float4 *>(a.outputs + (size_t)r * 8u);
                    dst[0] = make_float4(o[0], o[1], o[2], o[3]);
                    dst[1] = make_float4(o[4], o[5], o[6], o[7]);
                }
            }
            tc::fence_before_sync();
            group_sync(gbar);
        }
    }
    if (!ok) {
        // a wait ran out: record it, give copies and MMAs still in flight one more bounded wait
        if (issuer) {
            atomicOr(a.status, 1u);
            if (load_pending)
                tc::mbar_wait(bar_load, ph_load);
            if (mma_pending)
                tc::mbar_wait(bar_mma, ph_mma);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < 32u) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem_all, tmem_alloc_cols(G));
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

} // namespace

cudaError_t configure_mlp_tc()
{
    cudaError_t e = allow_max_dynamic_smem(k_mlp_tc<false, false>);
    if (e == cudaSuccess)
        e = allow_max_dynamic_smem(k_mlp_tc<true, false>);
    if (e == cudaSuccess)
        e = allow_max_dynamic_smem(k_mlp_tc<false, true>);
    return e;
}

uint32_t packed_weight_bytes(uint32_t n_inputs, uint32_t n_hidden_layers)
{
    return w0_bytes(n_inputs) + (n_hidden_layers - 1u) * hidden_w_bytes() + out_w_bytes();
}

cudaError_t launch_pack_weights(const __half *params_h, uint32_t n_inputs, uint32_t n_hidden_layers, __half *packed,
                                cudaStream_t s)
{
    const uint32_t total = packed_weight_bytes(n_inputs, n_hidden_layers) / 2u;
    k_pack_weights<<<(total + 255u) / 256u, 256, 0, s>>>(params_h, n_inputs, n_hidden_layers, packed);
    return cudaGetLastError();
}

cudaError_t make_feature_map(const __half *features, uint32_t n_inputs, uint32_t rows, TensorMapBytes *out,
                             bool allow_swizzle)
{
    static_assert(sizeof(CUtensorMap) == sizeof(TensorMapBytes), "tensor map size");
    if ((reinterpret_cast<uintptr_t>(features) & 15u) != 0u || n_inputs % 16u != 0u || n_inputs > 128u || rows == 0u)
        return cudaErrorInvalidValue;
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode)
        return cudaErrorNotSupported;
    CUtensorMap fmap;
    const cuuint64_t dims[2] = {n_inputs, rows};
    const cuuint64_t strides[1] = {(cuuint64_t)n_inputs * 2u};
    // 64 values x 128 rows, 128-byte swizzle (one atom column of the K-major swizzled layout), or
    // 8 values x 128 rows unswizzled (one K column of core matrices)
    const bool sw = allow_swizzle && feature_map_swizzled(n_inputs);
    const cuuint32_t box[2] = {sw ? 64u : 8u, kTileRows};
    const cuuint32_t estr[2] = {1u, 1u};
    // 16-bit rows; the element type of the map only sizes the copy (FP16 and BF16 move the same bits)
    if (encode(&fmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half *>(features), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, sw ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    memcpy(out->bytes, &fmap, sizeof(fmap));
    return cudaSuccess;
}

cudaError_t launch_mlp_tc(const TensorMapBytes &feature_map, const __half *wpacked, uint32_t n_inputs,
                          uint32_t n_hidden_layers, uint32_t rows, const uint32_t *d_count, float *outputs,
                          uint32_t *status, uint32_t prec, int num_sms, cudaStream_t s, bool configure,
                          uint64_t wait_ns, bool stall)
{
    if (rows == 0)
        return cudaSuccess;
    const bool bf16 = prec == NBVH_PRECISION_BF16;
    CUtensorMap fmap;
    memcpy(&fmap, feature_map.bytes, sizeof(fmap));
    MlpTcArgs a;
    a.wpacked = wpacked;
    a.wbytes = packed_weight_bytes(n_inputs, n_hidden_layers);
    a.n_inputs = n_inputs;
    a.n_hidden_layers = n_hidden_layers;
    a.n = rows;
    a.d_count = d_count;
    a.outputs = outputs;
    a.status = status;
    a.fp8 = prec == NBVH_PRECISION_FP8 ? 1u : 0u;
    a.wait_ns = wait_ns ? wait_ns : tc::kWaitLimitNs;
    a.stall = stall ? 1u : 0u;
    // as many tile groups as shared memory holds (227 KB per CTA), at most kMaxGroups
    const size_t tile_bytes = (size_t)kTileRows * n_inputs * 2u;
    const size_t fixed = tile_offset(a.wbytes) + 8u * (2u * kMaxGroups + 2u) + 16u;
    const size_t room = 227u * 1024u;
    if (fixed + tile_bytes > room)
        return cudaErrorInvalidValue;
    uint32_t groups = (uint32_t)((room - fixed) / tile_bytes);
    groups = groups < kMaxGroups ? groups : kMaxGroups;
    // no more pipelines than the batch's tiles per SM: small batches (a serving slot's) leave
    // shared memory to the kernels of the other streams
    const uint32_t tiles_per_sm = (uint32_t)(((rows + kTileRows - 1u) / kTileRows + (uint32_t)num_sms - 1u) / (uint32_t)num_sms);
    groups = tiles_per_sm < groups ? (tiles_per_sm > 0u ? tiles_per_sm : 1u) : groups;
    a.groups = groups;
    size_t smem = tile_offset(a.wbytes) + groups * tile_bytes + 8u * (2u * groups + 2u) + 16u;
    // at most 512 / tmem_alloc_cols(groups) CTAs on an SM, so that their TMEM allocations always
    // fit: one CTA more must not fit the SM's 228 KB (each CTA also reserves 1 KB)
    const size_t max_ctas = 512u / tmem_alloc_cols(groups);
    const size_t smem_min = kSmPerSm / (max_ctas + 1u) - kSmemReservedPerCta + 128u;
    smem = smem < smem_min ? smem_min : smem;
    if (configure) {
        const cudaError_t e = bf16      ? allow_max_dynamic_smem(k_mlp_tc<true, false>)
                              : a.fp8 ? allow_max_dynamic_smem(k_mlp_tc<false, true>)
                                      : allow_max_dynamic_smem(k_mlp_tc<false, false>);
        if (e != cudaSuccess)
            return e;
    }
    const uint32_t tiles = (rows + kTileRows - 1u) / kTileRows;
    uint32_t blocks = (uint32_t)num_sms;
    if (blocks > tiles)
        blocks = tiles;
    const uint32_t threads = groups * kGroupThreads;
    if (bf16)
        k_mlp_tc<true, false><<<blocks, threads, smem, s>>>(fmap, a);
    else if (a.fp8)
        k_mlp_tc<false, true><<<blocks, threads, smem, s>>>(fmap, a);
    else
        k_mlp_tc<false, false><<<blocks, threads, smem, s>>>(fmap, a);
    return cudaGetLastError();
}

} // namespace nbvh
