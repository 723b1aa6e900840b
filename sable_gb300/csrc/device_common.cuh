// Device helpers shared by the kernels of libsable (sm_103a): constants, the
// PTX wrappers for mbarriers, TMA bulk copies and cp.async, bounded waits,
// and small vector arithmetic.  Every wait here gives up after WAIT_NS.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "sable_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NWARP = SABLE_NWARP;
constexpr int RED_FLOATS = NWARP * SABLE_MAX_ROW_TILE;    // dense partials (CTA kernel)
constexpr int STAGE_OFF = 2 * RED_FLOATS * 4;             // + CSR partials, bytes
constexpr unsigned long long WAIT_NS = 2000000000ull;
constexpr int CTRL = SABLE_THREADS - 1;                    // control thread (CTA kernel)
constexpr int WCTRL = 31;                                  // control lane (warp kernel)
constexpr int ROWBUF_FLOATS = SABLE_MAX_ROW_TILE + 32;     // warp kernel: CSR row sums + dense temp

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
}

// An mbarrier whose phase completes after `count` arrivals.
__device__ __forceinline__ void mbar_init_count(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}

// One arrival (release at CTA scope: this thread's earlier writes, and those
// ordered before it, are visible to a thread whose wait sees the phase end).
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

// Wait for phase `parity` of an mbarrier, giving up after limit_ns.
__device__ __forceinline__ bool mbar_wait_for(unsigned bar, unsigned parity, unsigned long long limit_ns) {
    unsigned done = 0;
    const unsigned long long t0 = global_ns();
    while (true) {
        asm volatile(
            "{\n .reg .pred p;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(bar), "r"(parity), "r"(1000000u) : "memory");
        if (done) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// Wait for phase `parity` of an mbarrier, giving up after WAIT_NS.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) { return mbar_wait_for(bar, parity, WAIT_NS); }

// Release-acquire arrival on a split-tile counter (one thread, after the
// partial-sum stores of its CTA / warp are ordered before it).
__device__ __forceinline__ int arrive_acq_rel(int *cnt) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(cnt) : "memory");
    return old;
}

// One thread: expect `bytes` on `bar` and copy the record into `dst`.
__device__ __forceinline__ void tma_record(unsigned bar, void *dst, const unsigned char *src, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ void cp_async4(void *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory"); }

__device__ __forceinline__ float dot4(const float4 a, const float4 b, float acc) {
    acc = fmaf(a.x, b.x, acc);
    acc = fmaf(a.y, b.y, acc);
    acc = fmaf(a.z, b.z, acc);
    acc = fmaf(a.w, b.w, acc);
    return acc;
}

__device__ __forceinline__ float4 xquad(const int4 *xc, int q, const float *__restrict__ x) {
    const int4 c = xc[q];
    return make_float4(__ldg(x + c.x), __ldg(x + c.y), __ldg(x + c.z), __ldg(x + c.w));
}

__device__ __forceinline__ const MatIO &mat_of(const LaunchArgs &a, int mat) { return a.mats ? a.mats[mat] : a.mat0; }


__device__ __forceinline__ float4 fma4(float a, float4 b, float4 c) {
    c.x = fmaf(a, b.x, c.x);
    c.y = fmaf(a, b.y, c.y);
    c.z = fmaf(a, b.z, c.z);
    c.w = fmaf(a, b.w, c.w);
    return c;
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

}  // namespace
