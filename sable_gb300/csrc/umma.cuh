// tcgen05 (5th-generation tensor core) helpers for sm_103a: TMEM allocation,
// UMMA shared-memory and instruction descriptors, MMA issue / commit, TMEM
// loads and the fences that order them.  Inline PTX only.
//
// Operand layouts used by this library (no swizzle, checked bit for bit by an
// in-bounds single-CTA GEMM on the device):
//   K-major   element (r, k) of an operand block of 16 K columns lives at
//             byte (r & 7) * 16 + (r >> 3) * 256 + (k & 7) * 2 + (k >> 3) * 128:
//             core matrices of 8 rows x 16 bytes; descriptor LBO = 128 (the
//             stride between the two 8-column K halves), SBO = 256 (between
//             8-row groups).
//   MN-major  element (m, k) lives at byte (k & 7) * 16 + (m & 7) * 2 +
//             (m >> 3) * 128 + (k >> 3) * 2048 for a block of 128 M rows:
//             16-byte rows hold 8 consecutive m of one k; descriptor LBO = 2048
//             (between the 8-row K groups), SBO = 128 (between the 8-element
//             M groups).  (Measured: with the K groups 128 bytes apart and the
//             M groups 256 apart the descriptor is LBO = 128, SBO = 256, so
//             for this layout LBO is the K-group stride, SBO the M-group one.)
#pragma once
#include <stdint.h>

namespace {

constexpr uint32_t UMMA_KM_LBO = 128, UMMA_KM_SBO = 256;    // K-major blocks
constexpr uint32_t UMMA_MN_LBO = 2048, UMMA_MN_SBO = 128;   // MN-major blocks of 128 rows

__host__ __device__ constexpr int umma_kmajor_off(int r, int k) {
    return (r & 7) * 16 + (r >> 3) * 256 + (k & 7) * 2 + (k >> 3) * 128;
}
__host__ __device__ constexpr int umma_mnmajor_off(int m, int k) {
    return (k & 7) * 16 + (m & 7) * 2 + (m >> 3) * 128 + (k >> 3) * 2048;
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), LBO >> 4
// (16-29), SBO >> 4 (32-45), the fixed version bits 46-48 = 0b001, base
// offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16 with BF16 A and B and an FP32
// accumulator: D format bit 4, A / B format BF16 (bits 7, 10), A MN-major
// (bit 15) when a_mn, B K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N, bool a_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// TMEM columns to allocate for n accumulator columns (a power of two >= 32).
__host__ __device__ constexpr uint32_t umma_tmem_cols(int n) {
    return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : n <= 256 ? 256u : 512u;
}

// Whole warp: allocate `ncols` TMEM columns, address written to *dst (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t dst_saddr, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(dst_saddr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// Whole warp (the allocating one): free the columns.
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One thread: D[tmem] (+)= A * B, one M x N x 16 BF16 step.
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// One thread: arrive once on the mbarrier when the tcgen05 operations this
// thread issued since its previous commit have completed (an earlier commit
// already tracks the ones before).
__device__ __forceinline__ void umma_commit(uint32_t bar_saddr) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar_saddr)
                 : "memory");
}

// Whole warp: 16 consecutive accumulator columns of the warp's 32 TMEM lanes
// (lane i of the warp gets lane 32 (warp % 4) + i), then wait for the load.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace
