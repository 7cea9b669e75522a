// tc.cuh — fifth-generation tensor core (tcgen05) building blocks for the
// small BF16 MLP of the learned correction: TMEM allocation, shared-memory
// operand descriptors, MMA issue/commit, accumulator loads, mbarriers.
//
// Operand layout.  Every MMA operand lives in shared memory as a row-major
// R x K BF16 matrix ("K-major": K contiguous) in the canonical no-swizzle
// arrangement of 8-row x 16-byte core matrices:
//     byte offset of (r, k) = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (core matrices along K are adjacent) and SBO = K * 16 (one
// 8-row group of all K).  A is M x K (M = 128 rows = TMEM lanes), B is N x K
// (the nn.Linear weight layout [out][in]); D = A * B^T accumulates in FP32 in
// TMEM (lane = row of D, column = column of D).  A K step of 16 advances the
// start address of both descriptors by 2 * LBO.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace geon {
namespace tc {

constexpr uint32_t LBO = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: BF16 A and B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// The same with FP16 A and B (format code 0).
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- TMEM -----------------------------------------------------------------
// Executed by one full warp.  The allocated address is written to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes become visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA ------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accum) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :: "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)(accum ? 1 : 0)) : "memory");
}
// D[128 x N] (+)= A[128 x K] * B[N x K]^T, K a multiple of 16, A and B both
// BF16 (or both FP16 with f16 set).  Issued by one thread.
__device__ __forceinline__ void gemm(uint32_t d_tmem, const void* A, const void* B, int N, int K, bool accum,
                                     bool f16 = false) {
    const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
    const uint32_t sbo = (uint32_t)K * 16u;
    const uint32_t id = f16 ? idesc_f16(128, N) : idesc_bf16(128, N);
    for (int k = 0; k < K; k += 16) {
        const uint32_t step = (uint32_t)(k >> 3) * LBO;
        mma_bf16(d_tmem, make_desc(a0 + step, LBO, sbo), make_desc(b0 + step, LBO, sbo), id, accum || k > 0);
    }
}
// Arrives on the mbarrier once all previously issued MMAs of this thread complete.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(bar)) : "memory");
}

// ---- mbarrier ----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// Bounded wait: returns false if the phase did not complete within the limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = 1u << 22) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ---- TMEM -> registers --------------------------------------------------------
// Each warp of a 4-warp group reads its 32 lanes (rows 32w .. 32w+31) and 16
// consecutive FP32 columns starting at `col`.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ uint32_t tmem_addr(uint32_t base, int warp_in_group, int col) {
    return base + ((uint32_t)(warp_in_group * 32) << 16) + (uint32_t)col;
}

}  // namespace tc
}  // namespace geon
