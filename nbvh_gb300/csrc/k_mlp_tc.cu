// k_mlp_tc.cu -- the fully fused MLP (K4 forward) on the 5th-generation tensor cores.
//
// tcnn's FullyFusedMLP (configured at src/cuda/neural/neural_bvh_module.cu:232-238: 64 neurons,
// ReLU hidden layers, Sigmoid output, no biases, output padded to 16) evaluated on 128-row tiles:
//
//   TMA        one 2-D tensor copy per 8-column slice moves the tile's FP16 inputs from HBM into
//              shared memory, already in the tensor core's K-major core-matrix layout;
//   tcgen05    one thread issues each layer as M=128 x N=64 (N=16 for the output layer) MMAs over
//              K in steps of 16; the FP32 accumulator lives in tensor memory (64 columns);
//   epilogue   each of the 4 warps reads its 32 TMEM lanes (= its 32 rows), applies ReLU, rounds to
//              FP16 and writes the next layer's A operand back to shared memory (over the input
//              tile, which the finished MMA no longer needs); after the output layer it applies
//              the sigmoid and stores 8 FP32 outputs per row.
//
// The weights (about 42 KB) are packed once per call into the same operand layout and copied to
// shared memory with one bulk copy per CTA; three CTAs share an SM, so one CTA's epilogue overlaps
// another's MMAs and copies.
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
constexpr uint32_t kMlpThreads = 128;

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
    uint32_t fp8; // inputs of the hidden matrices rounded to FP8-E4M3
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

// Hidden-layer epilogue for this thread's row: 64 accumulator columns -> ReLU -> 16-bit (FP16 or
// BF16) -> the next layer's A operand (128 x 64) at act.
template <bool BF16, bool FP8>
__device__ __forceinline__ void epilogue_hidden(uint32_t tmem_row, unsigned char *act, uint32_t row, bool quant)
{
    using Pr = MlpPrec<BF16>;
    // FP8 mode: the input of a hidden matrix is an FP8-E4M3 value (exact in FP16)
    auto relu = [quant](uint32_t u) {
        return (FP8 && quant) ? fp8_act(fmaxf(__uint_as_float(u), 0.f)) : fmaxf(__uint_as_float(u), 0.f);
    };
    uint32_t v[4][16];
#pragma unroll
    for (int q = 0; q < 4; q++)
        tc::tmem_ld16(tmem_row + 16u * q, v[q]);
    tc::tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const uint32_t *s = &v[c >> 1][(c & 1) * 8];
        uint4 q;
        q.x = Pr::pack(relu(s[0]), relu(s[1]));
        q.y = Pr::pack(relu(s[2]), relu(s[3]));
        q.z = Pr::pack(relu(s[4]), relu(s[5]));
        q.w = Pr::pack(relu(s[6]), relu(s[7]));
        *reinterpret_cast<uint4 *>(act + tc::operand_offset(row, 8u * c, kTileRows)) = q;
    }
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

template <bool BF16, bool FP8>
__global__ void __launch_bounds__(kMlpThreads, 3) k_mlp_tc(const __grid_constant__ CUtensorMap fmap, const MlpTcArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t K = a.n_inputs, H = a.n_hidden_layers;
    uint32_t n = a.n;
    if (a.d_count) {
        const uint32_t c = *reinterpret_cast<volatile const uint32_t *>(a.d_count);
        n = c < n ? c : n;
    }
    const uint32_t n_tiles = (n + kTileRows - 1u) / kTileRows;
    if (blockIdx.x >= n_tiles)
        return; // no tile for this CTA: skip TMEM and the weight copy
    const uint32_t tile_off = (a.wbytes + 1023u) & ~1023u;
    unsigned char *tile = smem + tile_off;
    uint64_t *bars = reinterpret_cast<uint64_t *>(tile + kTileRows * K * 2u);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2);
    const uint32_t bar_load = tc::smem_addr(&bars[0]), bar_mma = tc::smem_addr(&bars[1]);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u, row = 32u * warp + lane;
    const uint32_t w_addr = tc::smem_addr(smem), t_addr = tc::smem_addr(tile);

    if (warp == 0) {
        tc::tmem_alloc(tc::smem_addr(slot), 64u);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(bar_load, 1u);
        tc::mbar_init(bar_mma, 1u);
        tc::mbar_init_fence();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t tmem_row = tmem + ((32u * warp) << 16);

    auto load_tile = [&](uint32_t t) {
        tc::mbar_expect_tx(bar_load, kTileRows * K * 2u);
        for (uint32_t c = 0; c < K / 8u; c++)
            tc::tma_load_2d(t_addr + c * kTileRows * 16u, &fmap, (int32_t)(8u * c), (int32_t)(t * kTileRows), bar_load);
    };
    uint32_t ph_load = 0, ph_mma = 0;
    bool load_pending = false, mma_pending = false;
    if (tid == 0) {
        tc::mbar_expect_tx(bar_load, a.wbytes);
        for (uint32_t o = 0; o < a.wbytes; o += 16384u)
            tc::bulk_load(w_addr + o, reinterpret_cast<const unsigned char *>(a.wpacked) + o,
                          a.wbytes - o < 16384u ? a.wbytes - o : 16384u, bar_load);
    }
    bool ok = tc::mbar_wait(bar_load, ph_load);
    ph_load ^= 1u;
    ok = __syncthreads_and(ok);
    uint32_t t = blockIdx.x;
    if (ok && t < n_tiles && tid == 0)
        load_tile(t);
    load_pending = ok && t < n_tiles;
    const uint32_t id_hidden = tc::idesc_f16(kTileRows, kNeurons, BF16);
    const uint32_t id_out = tc::idesc_f16(kTileRows, kOutputsPadded, BF16);
    for (; ok && t < n_tiles; t += gridDim.x) {
        ok = tc::mbar_wait(bar_load, ph_load);
        ok = __syncthreads_and(ok);
        if (!ok)
            break;
        ph_load ^= 1u;
        load_pending = false;
        for (uint32_t layer = 0; layer <= H; layer++) {
            if (tid == 0) {
                tc::fence_after_sync();
                if (layer == 0)
                    issue_layer(tmem, t_addr, w_addr, K, kNeurons, id_hidden);
                else if (layer < H)
                    issue_layer(tmem, t_addr, w_addr + w0_bytes(K) + (layer - 1u) * hidden_w_bytes(), kNeurons,
                                kNeurons, id_hidden);
                else
                    issue_layer(tmem, t_addr, w_addr + w0_bytes(K) + (H - 1u) * hidden_w_bytes(), kNeurons,
                                kOutputsPadded, id_out);
                tc::mma_commit(bar_mma);
            }
            mma_pending = true;
            ok = tc::mbar_wait(bar_mma, ph_mma);
            ok = __syncthreads_and(ok);
            if (!ok)
                break;
            ph_mma ^= 1u;
            mma_pending = false;
            tc::fence_after_sync();
            if (layer < H) {
                epilogue_hidden<BF16, FP8>(tmem_row, tile, row, layer + 1u < H);
                tc::fence_async_shared();
            } else {
                // the tile buffer is free: start the next tile's copy under this epilogue
                if (tid == 0 && t + gridDim.x < n_tiles)
                    load_tile(t + gridDim.x);
                load_pending = t + gridDim.x < n_tiles;
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
            __syncthreads();
        }
    }
    if (!ok) {
        // a wait ran out: record it, give copies and MMAs still in flight one more bounded wait
        if (tid == 0) {
            atomicOr(a.status, 1u);
            if (load_pending)
                tc::mbar_wait(bar_load, ph_load);
            if (mma_pending)
                tc::mbar_wait(bar_mma, ph_mma);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 64u);
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

cudaError_t make_feature_map(const __half *features, uint32_t n_inputs, uint32_t rows, TensorMapBytes *out)
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
    const cuuint32_t box[2] = {8u, kTileRows}; // 16 bytes x 128 rows: one K column of core matrices
    const cuuint32_t estr[2] = {1u, 1u};
    // 16-bit rows; the element type of the map only sizes the copy (FP16 and BF16 move the same bits)
    if (encode(&fmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half *>(features), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    memcpy(out->bytes, &fmap, sizeof(fmap));
    return cudaSuccess;
}

cudaError_t launch_mlp_tc(const TensorMapBytes &feature_map, const __half *wpacked, uint32_t n_inputs,
                          uint32_t n_hidden_layers, uint32_t rows, const uint32_t *d_count, float *outputs,
                          uint32_t *status, uint32_t prec, int num_sms, cudaStream_t s, bool configure)
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
    const size_t smem = ((a.wbytes + 1023u) & ~1023u) + kTileRows * n_inputs * 2u + 32u;
    if (configure) {
        const cudaError_t e = bf16      ? allow_max_dynamic_smem(k_mlp_tc<true, false>)
                              : a.fp8 ? allow_max_dynamic_smem(k_mlp_tc<false, true>)
                                      : allow_max_dynamic_smem(k_mlp_tc<false, false>);
        if (e != cudaSuccess)
            return e;
    }
    const uint32_t tiles = (rows + kTileRows - 1u) / kTileRows;
    uint32_t blocks = (uint32_t)num_sms * 3u;
    if (blocks > tiles)
        blocks = tiles;
    if (bf16)
        k_mlp_tc<true, false><<<blocks, kMlpThreads, smem, s>>>(fmap, a);
    else if (a.fp8)
        k_mlp_tc<false, true><<<blocks, kMlpThreads, smem, s>>>(fmap, a);
    else
        k_mlp_tc<false, false><<<blocks, kMlpThreads, smem, s>>>(fmap, a);
    return cudaGetLastError();
}

} // namespace nbvh
