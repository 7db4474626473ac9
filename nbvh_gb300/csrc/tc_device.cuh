// tc_device.cuh -- Blackwell (sm_103a) building blocks: tcgen05 tensor-core MMA with accumulators in
// tensor memory (TMEM), TMA bulk / tensor copies into shared memory, and mbarrier waits that give up
// after a time limit instead of spinning forever.
//
// Shared-memory operand layout used throughout (K-major, no swizzle): the matrix is cut into "core
// matrices" of 8 rows x 16 bytes (8 FP16 values), each stored as 128 contiguous bytes (row i of the
// core matrix at byte 16 * i). A descriptor gives two strides: LBO, the byte distance between core
// matrices adjacent along K, and SBO, the distance between core matrices adjacent along M (or N).
// Here every operand uses SBO = 128 (the 8-row groups of one K column of core matrices are
// contiguous) and LBO = rows * 16, so element (r, k) of an R-row operand lives at
//     (k / 8) * (R * 16) + r * 16 + (k % 8) * 2.
// This is also exactly what a 2-D TMA box of 8 values x R rows writes, so tiles arrive ready to use.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace nbvh {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in an R-row operand laid out as described above
__host__ __device__ constexpr uint32_t operand_offset(uint32_t r, uint32_t k, uint32_t rows)
{
    return (k >> 3) * (rows * 16u) + r * 16u + (k & 7u) * 2u;
}

// ---- mbarrier ----------------------------------------------------------------------------------

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0u;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// Time limit of every wait below: a phase that has not completed after this long never will (the
// work behind one phase takes microseconds), so the kernel records an error and winds down.
constexpr uint64_t kWaitLimitNs = 1000000000ull;

// Waits until the phase with the given parity has completed; false after limit_ns (a handle may
// set a shorter limit for its kernels' phase waits; the waits that drain copies and MMAs still in
// flight before a kernel exits always use kWaitLimitNs).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > limit_ns)
            return false;
    }
    return true;
}

// ---- TMA ---------------------------------------------------------------------------------------

// Plain bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Tiled 2-D tensor copy of one box at element coordinates (x, y); x * element size must be a
// multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void *tmap, int32_t x, int32_t y, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                 "[%4];\n" ::"r"(dst),
                 "l"(tmap), "r"(x), "r"(y), "r"(bar)
                 : "memory");
}

// ---- TMEM and tcgen05 ----------------------------------------------------------------------------

// Allocation and release are warp-wide (.sync.aligned); the column base is written to slot.
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Makes generic-proxy shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, both K-major; issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
                 "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

// D[tmem] (+)= A[tmem] * B[smem]^T: A read from tensor memory (row r in lane r, two 16-bit K values
// per 32-bit column, the lower K in the low half), B K-major in shared memory; issued by one thread.
__device__ __forceinline__ void mma_f16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                           uint32_t accumulate)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
                 "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

// The mbarrier receives one arrival when every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

// 16 (or 8) consecutive 32-bit columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                 "%14, %15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// 32 consecutive 32-bit columns of this thread's TMEM lane from registers (warp w writes lanes
// 32w..32w+31); complete once tmem_wait_st returns.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};\n"
                 ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
                 "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]),
                 "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]),
                 "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, no swizzle, base offset 0, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Shared-memory matrix descriptor of a K-major operand in the 128-byte swizzled layout: atoms of
// 8 rows x 128 bytes (64 16-bit values of K), rows 128 bytes apart with their 16-byte chunks XORed
// by the row index (what a TMA box of 64 values x R rows with SWIZZLE_128B writes), atoms along
// M/N 1,024 bytes apart. addr = atom-aligned base (1,024-byte aligned) + 32 bytes per 16 values of
// K inside the atom.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator, A and B both FP16 (or both BF16),
// both K-major, dense, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t m, uint32_t n, bool bf16)
{
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// The same with A and / or B MN-major (bits 15 and 16: the operand's M, resp. N, index is the one
// contiguous in memory). An MN-major operand without swizzle uses core matrices of 8 K-rows x 16
// bytes (8 values along M or N): the descriptor's LBO is then the byte distance between core
// matrices adjacent along K and SBO the distance between core matrices adjacent along M / N, the
// same roles as for a K-major operand. So a [rows][cols] buffer in the K-major layout above (core
// matrix = 8 rows x 8 columns, LBO = 16 * rows between column blocks, SBO = 128 between row
// blocks) is also the MN-major operand whose K index is the row: LBO = 128, SBO = 16 * rows.
__host__ __device__ constexpr uint32_t idesc_f16_major(uint32_t m, uint32_t n, bool bf16, bool a_mn, bool b_mn)
{
    return idesc_f16(m, n, bf16) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16);
}

} // namespace tc
} // namespace nbvh
