// net_device.cuh -- multiresolution hash-grid encoding (used by every encoder: the wavefront and
// tail kernels of the query, the training rows, the stand-alone encode) and the warp-level MLP of
// the persistent tail kernel (the wavefront steps and training run the MLP on tcgen05 tensor
// cores: k_mlp_tc.cu, k_train.cu).
//
// The encoding follows the tcnn HashGrid behaviour the reference configures
// (src/cuda/neural/neural_bvh_module.cu:170-191): per level, position = x * scale + 0.5, trilinear
// weights over the 8 corners, dense indexing while res^3 fits the level, coherent prime hash
// (x * 1 ^ y * 2654435761 ^ z * 805459861) otherwise; one grid shared by all segment points
// (RepeatedComposite), features concatenated point-major then level-major.
//
// The MLP is tcnn's FullyFusedMLP shape (64 neurons, ReLU, Sigmoid output, no biases, output
// padded to 16). The tail kernel's warps each own 16-row tiles, too few rows for a tcgen05 MMA
// (M = 64 or 128 per CTA, issued by one thread for the whole CTA), so these are computed with
// mma.sync m16n8k16 (FP16 in, FP32 accumulate); hidden activations never leave registers: the FP32
// accumulator fragment of one layer, after ReLU and rounding to FP16, is exactly the A-operand
// fragment of the next layer.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "device_math.cuh"
#include "nbvh_internal.h"

namespace nbvh {

constexpr uint32_t kHiddenLd = kNeurons + 8; // padded smem row stride (halves) of 64-wide matrices

// offsets (in halves) of the network matrices inside the padded shared-memory copy
struct SmemNetLayout {
    uint32_t ld0;       // n_inputs + 8
    uint32_t hidden_off; // first 64x64 matrix
    uint32_t out_off;    // 16x64 output matrix
    uint32_t total;      // halves
};

__host__ __device__ inline SmemNetLayout smem_net_layout(uint32_t n_inputs, uint32_t n_hidden_layers)
{
    SmemNetLayout L;
    L.ld0 = n_inputs + 8u;
    L.hidden_off = kNeurons * L.ld0;
    L.out_off = L.hidden_off + (n_hidden_layers - 1u) * kNeurons * kHiddenLd;
    L.total = L.out_off + kOutputsPadded * kHiddenLd;
    return L;
}

// Copies the FP16 network matrices (packed [rows][cols], network-first parameter layout) into
// the padded shared-memory layout. Whole block participates.
__device__ __forceinline__ void load_weights_to_smem(const __half *__restrict__ w, __half *sw, uint32_t n_inputs,
                                                     uint32_t n_hidden_layers)
{
    SmemNetLayout L = smem_net_layout(n_inputs, n_hidden_layers);
    const uint32_t *w32 = reinterpret_cast<const uint32_t *>(w);
    // matrix 0: 64 x n_inputs
    uint32_t words0 = kNeurons * n_inputs / 2u;
    for (uint32_t i = threadIdx.x; i < words0; i += blockDim.x) {
        uint32_t r = (2u * i) / n_inputs, c = (2u * i) % n_inputs;
        *reinterpret_cast<uint32_t *>(sw + r * L.ld0 + c) = __ldg(w32 + i);
    }
    // hidden 64x64 matrices and the 16x64 output matrix
    uint32_t rows_rest = (n_hidden_layers - 1u) * kNeurons + kOutputsPadded;
    uint32_t words_rest = rows_rest * kNeurons / 2u;
    const uint32_t *wr = w32 + words0;
    for (uint32_t i = threadIdx.x; i < words_rest; i += blockDim.x) {
        uint32_t r = (2u * i) / kNeurons, c = (2u * i) % kNeurons;
        *reinterpret_cast<uint32_t *>(sw + L.hidden_off + r * kHiddenLd + c) = __ldg(wr + i);
    }
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_half2(float lo, float hi)
{
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ float2 unpack_half2(uint32_t u)
{
    __half2 h = *reinterpret_cast<__half2 *>(&u);
    return __half22float2(h);
}

__device__ __forceinline__ uint32_t pack_bf162(float lo, float hi)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

// Element type of the MLP operands (network weights, encoded inputs, hidden activations and the
// backward pass's activation gradients): FP16, the reference's network precision, or BF16. Both
// are 16-bit values multiplied on the tensor cores with FP32 accumulation; the hash-grid table
// itself stays FP16 in either case.
template <bool BF16>
struct MlpPrec;

template <>
struct MlpPrec<false> {
    __device__ static __forceinline__ uint32_t pack(float lo, float hi) { return pack_half2(lo, hi); }
    __device__ static __forceinline__ float2 unpack(uint32_t u) { return unpack_half2(u); }
    __device__ static __forceinline__ float round(float x) { return __half2float(__float2half_rn(x)); }
    __device__ static __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
    {
        mma16816(d, a, b0, b1);
    }
};

template <>
struct MlpPrec<true> {
    __device__ static __forceinline__ uint32_t pack(float lo, float hi) { return pack_bf162(lo, hi); }
    __device__ static __forceinline__ float2 unpack(uint32_t u)
    {
        return make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xFFFF0000u));
    }
    __device__ static __forceinline__ float round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
    __device__ static __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
    {
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};\n"
                     : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    }
};

// Table indices of the corners (x, y, z) and (x + 1, y, z) of one level.
__device__ __forceinline__ void level_x_pair_index(bool hashed, uint32_t res, uint32_t size, uint32_t x, uint32_t y,
                                                   uint32_t z, uint32_t &i0, uint32_t &i1)
{
    if (hashed) {
        const uint32_t h = (y * 2654435761u) ^ (z * 805459861u);
        i0 = (x ^ h) & (size - 1u);
        i1 = ((x + 1u) ^ h) & (size - 1u);
    } else {
        const uint32_t b = y * res + z * res * res;
        i0 = x + b;
        i1 = x + 1u + b;
        if (i0 >= size)
            i0 %= size;
        if (i1 >= size)
            i1 %= size;
    }
}

// Entries i0 and i1 of one level's table (`tab` = the level's first entry, 16-byte aligned: level
// offsets are multiples of 8 entries). When both fall in one aligned pair of entries -- always for
// an even x on a hashed level, whose hash takes x times 1, and for an even index on a dense level
// -- one load of the pair serves both corners; otherwise the second is a load of its own.
__device__ __forceinline__ void gather_x_pair(const uint32_t *__restrict__ tab, uint32_t i0, uint32_t i1,
                                              uint32_t &v0, uint32_t &v1)
{
    const uint2 pr = __ldg(reinterpret_cast<const uint2 *>(tab + (i0 & ~1u)));
    const bool odd = (i0 & 1u) != 0u;
    v0 = odd ? pr.y : pr.x;
    if ((i0 ^ i1) == 1u)
        v1 = odd ? pr.x : pr.y;
    else
        v1 = __ldg(tab + i1);
}

// Features of one point at one level: 2 values, FMA accumulation over corners c = 0..7 (bit d of
// c selects the upper corner along axis d), identical operation order to the CPU restatement.
// PAIRS gathers the x / x + 1 corners with gather_x_pair (the same values; measured on GB300 it
// pays in the wavefront and training encoders, 3.22 -> 3.17-3.19 ms per 2^22-ray query with the
// wider register bound, and not in the tail kernel's 16-row tiles, 3.17 -> 3.18 ms).
template <bool PAIRS>
__device__ __forceinline__ float2 encode_level(const uint32_t *__restrict__ table, const GridParams &gp, uint32_t l,
                                               V3 p)
{
    const float s = gp.scale[l];
    const float px = __fmaf_rn(p.x, s, 0.5f), py = __fmaf_rn(p.y, s, 0.5f), pz = __fmaf_rn(p.z, s, 0.5f);
    const float flx = floorf(px), fly = floorf(py), flz = floorf(pz);
    const uint32_t gx = (uint32_t)(int32_t)flx, gy = (uint32_t)(int32_t)fly, gz = (uint32_t)(int32_t)flz;
    const float rx = __fsub_rn(px, flx), ry = __fsub_rn(py, fly), rz = __fsub_rn(pz, flz);
    const uint32_t res = gp.res[l], size = gp.size[l], off = gp.offset[l];
    const bool hashed = gp.hashed[l] != 0u;
    uint32_t v[8];
    if constexpr (PAIRS) {
#pragma unroll
        for (uint32_t c = 0; c < 8; c += 2) {
            uint32_t i0, i1;
            level_x_pair_index(hashed, res, size, gx, gy + ((c >> 1) & 1u), gz + ((c >> 2) & 1u), i0, i1);
            gather_x_pair(table + off, i0, i1, v[c], v[c + 1]);
        }
    } else {
#pragma unroll
        for (uint32_t c = 0; c < 8; c++) {
            const uint32_t x = gx + (c & 1u), y = gy + ((c >> 1) & 1u), z = gz + ((c >> 2) & 1u);
            uint32_t idx;
            if (hashed) {
                idx = (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (size - 1u);
            } else {
                idx = x + y * res + z * res * res;
                if (idx >= size)
                    idx %= size;
            }
            v[c] = __ldg(table + off + idx);
        }
    }
    const float wx0 = __fsub_rn(1.0f, rx), wy0 = __fsub_rn(1.0f, ry), wz0 = __fsub_rn(1.0f, rz);
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
    for (uint32_t c = 0; c < 8; c++) {
        float w = __fmul_rn(__fmul_rn((c & 1u) ? rx : wx0, (c & 2u) ? ry : wy0), (c & 4u) ? rz : wz0);
        float2 f = unpack_half2(v[c]);
        a0 = __fmaf_rn(w, f.x, a0);
        a1 = __fmaf_rn(w, f.y, a1);
    }
    return make_float2(a0, a1);
}

// Table entry of F FP16 features: F = 4 one 8-byte word, F = 8 one 16-byte word (F = 2 is the
// 32-bit word encode_level reads).
template <uint32_t F>
struct GridEntry;
template <>
struct GridEntry<4> {
    using T = uint2;
    __device__ static __forceinline__ void halves(const T &v, uint32_t (&w)[2]) { w[0] = v.x, w[1] = v.y; }
};
template <>
struct GridEntry<8> {
    using T = uint4;
    __device__ static __forceinline__ void halves(const T &v, uint32_t (&w)[4])
    {
        w[0] = v.x, w[1] = v.y, w[2] = v.z, w[3] = v.w;
    }
};

// Features of one point at one level for F = 4 or 8 features per entry: the corners and weights of
// encode_level, feature k of corner c accumulated as acc_k = fma(w_c, entry_c[k], acc_k) in corner
// order (the CPU restatement's order). `table` is the grid's first entry (16-byte aligned).
template <uint32_t F>
__device__ __forceinline__ void encode_level_wide(const void *__restrict__ table, const GridParams &gp, uint32_t l,
                                                  V3 p, float (&acc)[F])
{
    using E = GridEntry<F>;
    const typename E::T *tab = reinterpret_cast<const typename E::T *>(table);
    const float s = gp.scale[l];
    const float px = __fmaf_rn(p.x, s, 0.5f), py = __fmaf_rn(p.y, s, 0.5f), pz = __fmaf_rn(p.z, s, 0.5f);
    const float flx = floorf(px), fly = floorf(py), flz = floorf(pz);
    const uint32_t gx = (uint32_t)(int32_t)flx, gy = (uint32_t)(int32_t)fly, gz = (uint32_t)(int32_t)flz;
    const float rx = __fsub_rn(px, flx), ry = __fsub_rn(py, fly), rz = __fsub_rn(pz, flz);
    const uint32_t res = gp.res[l], size = gp.size[l], off = gp.offset[l];
    const bool hashed = gp.hashed[l] != 0u;
    const float wx0 = __fsub_rn(1.0f, rx), wy0 = __fsub_rn(1.0f, ry), wz0 = __fsub_rn(1.0f, rz);
#pragma unroll
    for (uint32_t k = 0; k < F; k++)
        acc[k] = 0.0f;
    // corners in two groups of four, so that at most four wide gathers are live at once
#pragma unroll
    for (uint32_t c0 = 0; c0 < 8; c0 += 4) {
        typename E::T v[4];
#pragma unroll
        for (uint32_t cc = 0; cc < 4; cc++) {
            const uint32_t c = c0 + cc;
            const uint32_t x = gx + (c & 1u), y = gy + ((c >> 1) & 1u), z = gz + ((c >> 2) & 1u);
            uint32_t idx;
            if (hashed) {
                idx = (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (size - 1u);
            } else {
                idx = x + y * res + z * res * res;
                if (idx >= size)
                    idx %= size;
            }
            v[cc] = __ldg(tab + off + idx);
        }
#pragma unroll
        for (uint32_t cc = 0; cc < 4; cc++) {
            const uint32_t c = c0 + cc;
            const float w = __fmul_rn(__fmul_rn((c & 1u) ? rx : wx0, (c & 2u) ? ry : wy0), (c & 4u) ? rz : wz0);
            uint32_t h[F / 2];
            E::halves(v[cc], h);
#pragma unroll
            for (uint32_t k = 0; k < F / 2; k++) {
                const float2 f = unpack_half2(h[k]);
                acc[2 * k] = __fmaf_rn(w, f.x, acc[2 * k]);
                acc[2 * k + 1] = __fmaf_rn(w, f.y, acc[2 * k + 1]);
            }
        }
    }
}

// FP8 activations of a pair packed as FP16 (lo in the low half): e4m3(max(x, 0) * 2^7) / 2^7 per
// value, through the hardware conversions to and from E4M3 (nearest even, saturating at 448,
// subnormals on the 2^-9 grid: the rounding e4m3_round states); the 2^-7 scale is exact in FP16.
__device__ __forceinline__ uint32_t fp8_act_relu_half2(float lo, float hi)
{
    const float a = __fmul_rn(fmaxf(lo, 0.f), kFp8ActScale), b = __fmul_rn(fmaxf(hi, 0.f), kFp8ActScale);
    uint16_t e;
    asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;\n" : "=h"(e) : "f"(b), "f"(a));
    uint32_t h;
    asm("cvt.rn.f16x2.e4m3x2 %0, %1;\n" : "=r"(h) : "h"(e));
    __half2 v = *reinterpret_cast<const __half2 *>(&h);
    v = __hmul2(v, __float2half2_rn(1.0f / kFp8ActScale));
    return *reinterpret_cast<const uint32_t *>(&v);
}

// Two FP32 values -> ReLU -> 16-bit pair (lo in the low half), one cvt.rn.relu instruction.
template <bool BF16>
__device__ __forceinline__ uint32_t pack_relu(float lo, float hi)
{
    uint32_t r;
    if constexpr (BF16)
        asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(hi), "f"(lo));
    else
        asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// Rebuilds the 16-bit A fragments of the next layer from the FP32 accumulators (after ReLU).
// (FP8 and quant: the activations go through FP8-E4M3 first, the input format of the hidden
// matrices in FP8 mode; E4M3 values are exact in FP16. FP8 is a template argument so that the
// FP16 / BF16 kernels carry none of that code.)
template <bool BF16, bool FP8 = false>
__device__ __forceinline__ void relu_pack(const float (&acc)[8][4], uint32_t (&a)[4][4], bool quant = false)
{
    using Pr = MlpPrec<BF16>;
    static_assert(!(FP8 && BF16), "FP8 hidden layers run on the FP16 tensor-core path");
    if (FP8 && quant) {
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            a[kb][0] = fp8_act_relu_half2(acc[2 * kb][0], acc[2 * kb][1]);
            a[kb][1] = fp8_act_relu_half2(acc[2 * kb][2], acc[2 * kb][3]);
            a[kb][2] = fp8_act_relu_half2(acc[2 * kb + 1][0], acc[2 * kb + 1][1]);
            a[kb][3] = fp8_act_relu_half2(acc[2 * kb + 1][2], acc[2 * kb + 1][3]);
        }
        return;
    }
    auto act = [](float x) { return fmaxf(x, 0.f); };
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
        a[kb][0] = Pr::pack(act(acc[2 * kb][0]), act(acc[2 * kb][1]));
        a[kb][1] = Pr::pack(act(acc[2 * kb][2]), act(acc[2 * kb][3]));
        a[kb][2] = Pr::pack(act(acc[2 * kb + 1][0]), act(acc[2 * kb + 1][1]));
        a[kb][3] = Pr::pack(act(acc[2 * kb + 1][2]), act(acc[2 * kb + 1][3]));
    }
}

// Forward of one 16-row tile. make_a(kb, a) fills the layer-0 A fragment of k-block kb (16
// inputs). On return o[0..1] are the sigmoid outputs (row g, cols 2*tig, 2*tig+1) and o[2..3]
// those of row g + 8 (g = lane / 4, tig = lane % 4), for output columns 0..7.
template <bool BF16, bool FP8 = false, typename AMaker>
__device__ __forceinline__ void mlp_forward_tile(const __half *sw, uint32_t n_inputs, uint32_t n_hidden_layers,
                                                 AMaker &&make_a, float (&o)[4])
{
    using Pr = MlpPrec<BF16>;
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const SmemNetLayout L = smem_net_layout(n_inputs, n_hidden_layers);
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    const uint32_t nkb = n_inputs / 16u;
    for (uint32_t kb = 0; kb < nkb; kb++) {
        uint32_t a[4];
        make_a(kb, a);
        const __half *wrow = sw + g * L.ld0 + kb * 16u + tig * 2;
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            uint32_t b0 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * L.ld0);
            uint32_t b1 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * L.ld0 + 8);
            Pr::mma(acc[nt], a, b0, b1);
        }
    }
    const __half *wl = sw + L.hidden_off;
    for (uint32_t layer = 1; layer < n_hidden_layers; layer++) {
        uint32_t a[4][4];
        relu_pack<BF16, FP8>(acc, a, true);
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
            acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            const __half *wrow = wl + g * kHiddenLd + kb * 16 + tig * 2;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                uint32_t b0 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * kHiddenLd);
                uint32_t b1 = *reinterpret_cast<const uint32_t *>(wrow + nt * 8 * kHiddenLd + 8);
                Pr::mma(acc[nt], a[kb], b0, b1);
            }
        }
        wl += kNeurons * kHiddenLd;
    }
    uint32_t a[4][4];
    relu_pack<BF16>(acc, a);
    float oc[4] = {0.f, 0.f, 0.f, 0.f};
    const __half *wo = sw + L.out_off + g * kHiddenLd + tig * 2;
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
        uint32_t b0 = *reinterpret_cast<const uint32_t *>(wo + kb * 16);
        uint32_t b1 = *reinterpret_cast<const uint32_t *>(wo + kb * 16 + 8);
        Pr::mma(oc, a[kb], b0, b1);
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
        o[i] = 1.0f / (1.0f + expf(-oc[i]));
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// Encode phase of a 16-row tile: FP16 features of every (row, point, level) written to the warp's
// feature tile feat[16][ld] (ld = n_inputs + 8 halves); rows not in active_mask16 are zero. Lane j
// handles the (point, level) pairs j, j + 32, ... for all rows, four rows at a time: the four
// rows' points are formed first (an inactive row takes the cube centre, whose gathers are cheap L1
// hits) and then encoded without branches in between, so that the 32 gathers are in flight
// together; groups of four inactive rows are skipped. No MLP accumulator is live here.
template <bool BF16, typename PosFn>
__device__ __forceinline__ void encode_tile_to_smem(const uint32_t *__restrict__ table, const GridParams &gp,
                                                    PosFn &&pos, uint32_t active_mask16, __half *feat, uint32_t ld)
{
    const int lane = threadIdx.x & 31;
    const uint32_t L = gp.n_levels, PL = gp.n_points * gp.n_levels;
    for (uint32_t j = (uint32_t)lane; j < PL; j += 32u) {
        const uint32_t p = j / L, l = j - p * L;
        for (uint32_t r0 = 0; r0 < 16u; r0 += 4u) {
            const uint32_t m4 = (active_mask16 >> r0) & 0xFu;
            if (m4 == 0u) {
#pragma unroll
                for (uint32_t k = 0; k < 4u; k++)
                    *reinterpret_cast<uint32_t *>(feat + (r0 + k) * ld + 2u * j) = 0u;
                continue;
            }
            V3 q[4];
#pragma unroll
            for (uint32_t k = 0; k < 4u; k++)
                q[k] = ((m4 >> k) & 1u) ? pos(r0 + k, p) : mk3(0.5f, 0.5f, 0.5f);
            float2 f[4];
#pragma unroll
            for (uint32_t k = 0; k < 4u; k++)
                f[k] = encode_level<false>(table, gp, l, q[k]);
#pragma unroll
            for (uint32_t k = 0; k < 4u; k++)
                *reinterpret_cast<uint32_t *>(feat + (r0 + k) * ld + 2u * j) =
                    ((m4 >> k) & 1u) ? MlpPrec<BF16>::pack(f[k].x, f[k].y) : 0u;
        }
    }
    __syncwarp();
}

// encode_tile_to_smem for 4 or 8 features per level: lane j handles the (point, level) pairs
// j, j + 32, ... and writes their F features (one 8- or 16-byte store per row), 8 / F rows at a
// time so that the same number of gathered words is in flight as in the 2-feature form.
template <bool BF16, uint32_t F, typename PosFn>
__device__ __forceinline__ void encode_tile_to_smem_wide(const void *__restrict__ table, const GridParams &gp,
                                                         PosFn &&pos, uint32_t active_mask16, __half *feat,
                                                         uint32_t ld)
{
    constexpr uint32_t RB = 8u / F; // rows per batch
    const int lane = threadIdx.x & 31;
    const uint32_t L = gp.n_levels, PL = gp.n_points * gp.n_levels;
    for (uint32_t j = (uint32_t)lane; j < PL; j += 32u) {
        const uint32_t p = j / L, l = j - p * L;
        for (uint32_t r0 = 0; r0 < 16u; r0 += RB) {
            const uint32_t mb = (active_mask16 >> r0) & ((1u << RB) - 1u);
            uint32_t w[RB][F / 2];
            if (mb == 0u) {
#pragma unroll
                for (uint32_t k = 0; k < RB; k++)
#pragma unroll
                    for (uint32_t q = 0; q < F / 2; q++)
                        w[k][q] = 0u;
            } else {
                V3 qp[RB];
#pragma unroll
                for (uint32_t k = 0; k < RB; k++)
                    qp[k] = ((mb >> k) & 1u) ? pos(r0 + k, p) : mk3(0.5f, 0.5f, 0.5f);
#pragma unroll
                for (uint32_t k = 0; k < RB; k++) {
                    float f[F];
                    encode_level_wide<F>(table, gp, l, qp[k], f);
#pragma unroll
                    for (uint32_t q = 0; q < F / 2; q++)
                        w[k][q] = ((mb >> k) & 1u) ? MlpPrec<BF16>::pack(f[2 * q], f[2 * q + 1]) : 0u;
                }
            }
#pragma unroll
            for (uint32_t k = 0; k < RB; k++) {
                __half *dst = feat + (r0 + k) * ld + F * j;
                if constexpr (F == 4)
                    *reinterpret_cast<uint2 *>(dst) = make_uint2(w[k][0], w[k][1]);
                else
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(w[k][0], w[k][1], w[k][2], w[k][3]);
            }
        }
    }
    __syncwarp();
}

// The encode phase of a 16-row tile for the grid's features per level (2, 4 or 8).
template <bool BF16, typename PosFn>
__device__ __forceinline__ void encode_tile_any(const uint32_t *__restrict__ table, const GridParams &gp, PosFn &&pos,
                                                uint32_t active_mask16, __half *feat, uint32_t ld)
{
    if (gp.n_features == 4u)
        encode_tile_to_smem_wide<BF16, 4>(table, gp, pos, active_mask16, feat, ld);
    else if (gp.n_features == 8u)
        encode_tile_to_smem_wide<BF16, 8>(table, gp, pos, active_mask16, feat, ld);
    else
        encode_tile_to_smem<BF16>(table, gp, pos, active_mask16, feat, ld);
}

// MLP phase of a 16-row tile whose 16-bit features are in feat[16][ld]; outputs as mlp_forward_tile.
template <bool BF16, bool FP8 = false>
__device__ __forceinline__ void mlp_tile_from_smem(const __half *sw, const __half *feat, uint32_t ld,
                                                   uint32_t n_inputs, uint32_t n_hidden_layers, float (&o)[4])
{
    const int lane = threadIdx.x & 31;
    const __half *arow = feat + ((lane & 7) + ((lane >> 3) & 1) * 8) * ld + (lane >> 4) * 8;
    auto make_a = [&](uint32_t kb, uint32_t(&a)[4]) { ldsm_x4(a, arow + kb * 16u); };
    mlp_forward_tile<BF16, FP8>(sw, n_inputs, n_hidden_layers, make_a, o);
}

// Encoded segment points along [po, pi] (neural_bvh_module_kernels.cu:57-96).
__device__ __forceinline__ float segment_t(uint32_t k, uint32_t n_points, uint32_t distribution, uint32_t &rng)
{
    if (distribution == NBVH_SEGMENT_UNIFORM)
        return lcg_randomf(rng);
    float delta, offset;
    if (distribution == NBVH_SEGMENT_EQUIDISTANT_EXTERIOR) {
        delta = n_points == 1u ? 1.0f : __fdiv_rn(1.0f, (float)(n_points - 1u));
        offset = 0.0f;
    } else {
        delta = __fdiv_rn(1.0f, (float)n_points);
        offset = 0.5f;
    }
    return __fmul_rn(delta, __fadd_rn((float)k, offset));
}

__device__ __forceinline__ V3 segment_point(V3 epo, V3 epi, float t)
{
    return add3(scale3(epo, __fsub_rn(1.0f, t)), scale3(epi, t));
}

} // namespace nbvh
