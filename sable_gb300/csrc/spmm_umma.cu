// Split-BF16 SpMM on the tcgen05 tensor cores (TMEM accumulators): one CTA of
// UMMA_THREADS threads per (item, N-slice), body spmm_umma_item in spmm_umma.cuh; the plan's panel
// terms in the UMMA K-major layout come from build_umma_planes (exec.cpp).
#include <cuda_runtime.h>
#include <stdint.h>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"
#include "spmm_umma.cuh"

namespace {

// Panel ring of a launch: stages of TERMS * hp * 32 bytes for the plan's
// tallest tile, as many as fit (4..12) beside the X stages in the shared
// memory of one of three CTAs per SM.
template <int NT, int TERMS>
void umma_ring(int hp, int &bst, int &bstage) {
    using L = UmmaSmem<NT, TERMS>;
    bstage = TERMS * hp * 32;
    bst = (UMMA_SMEM_BUDGET - L::RST - L::OFF_B) / bstage;
    bst = bst < UMMA_BST_MIN ? UMMA_BST_MIN : bst > UMMA_BST_MAX ? UMMA_BST_MAX : bst;
}

template <int NT, int TERMS, bool TIMED>
__global__ void __launch_bounds__(UMMA_THREADS, 3)
spmm_umma_kernel(const LaunchArgs la, const int64_t part_stride, const int bst, const int bstage) {
    extern __shared__ __align__(1024) unsigned char smem[];
    long long t0 = 0;
    if (TIMED && threadIdx.x == 0) t0 = clock64();
    const int item = blockIdx.x, slice = blockIdx.y;
    const unsigned char *R = la.records + la.items[item].off;
    const MatIO &a = mat_of(la, reinterpret_cast<const ItemHeader *>(R)->mat);
    // a batch launches as many N-slices as its widest matrix needs; the CTAs
    // of a narrower matrix's missing slices leave (uniformly, before any barrier)
    if (slice * NT >= a.N) return;
    const int64_t po = la.umma_off[item];
    spmm_umma_item<NT, TERMS>(R, a, slice, la.mats ? a.part_stride : part_stride, smem, la.umma + (po > 0 ? po : 0),
                              la.error, bst, bstage);
    if (TIMED) {
        __syncthreads();
        if (threadIdx.x == 0) la.cycles[(int64_t)slice * la.n_items + item] = (int64_t)(clock64() - t0);
    }
}

template <int NT, int TERMS, bool TIMED>
int launch_u(const LaunchArgs &a, int N, int64_t part_stride, cudaStream_t s) {
    dim3 grid(a.n_items, (N + NT - 1) / NT);
    int bst, bstage;
    umma_ring<NT, TERMS>(a.umma_hp, bst, bstage);
    const int smem = UmmaSmem<NT, TERMS>::total(bst, bstage);
    cudaError_t e = cudaFuncSetAttribute(spmm_umma_kernel<NT, TERMS, TIMED>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
    spmm_umma_kernel<NT, TERMS, TIMED><<<grid, UMMA_THREADS, smem, s>>>(a, part_stride, bst, bstage);
    return (int)cudaGetLastError();
}

template <int NT>
int launch_nt(const LaunchArgs &a, int N, int terms, int64_t part_stride, bool timed, cudaStream_t s) {
    if (terms == 3) return timed ? launch_u<NT, 3, true>(a, N, part_stride, s) : launch_u<NT, 3, false>(a, N, part_stride, s);
    return timed ? launch_u<NT, 2, true>(a, N, part_stride, s) : launch_u<NT, 2, false>(a, N, part_stride, s);
}

}  // namespace

namespace sable {

int launch_spmm_umma(const LaunchArgs &a, int N, int nt, int terms, int64_t part_stride, bool timed, void *stream) {
    if (a.n_items <= 0 || N <= 0) return 0;
    if ((terms != 2 && terms != 3) || !a.umma || !a.umma_off || a.umma_hp < 16 || a.umma_hp > SABLE_MAX_ROW_TILE ||
        (a.umma_hp & 15))
        return (int)cudaErrorInvalidValue;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (nt) {
        case 32: return launch_nt<32>(a, N, terms, part_stride, timed, s);
        case 64: return launch_nt<64>(a, N, terms, part_stride, timed, s);
        case 128: return launch_nt<128>(a, N, terms, part_stride, timed, s);
        default: return (int)cudaErrorInvalidValue;
    }
}

}  // namespace sable
