// Split-BF16 tensor-core SpMM kernels (dense blocks of SpMM with N >= 32):
// one CTA per (item, N-slice), body spmm_tc_item in spmm_item.cuh.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"
#include "spmm_item.cuh"

namespace {

// PRE: the plan's pre-split A fragments (la.tcplanes, la.tcoff) feed the
// tensor cores; otherwise every warp splits its FP32 fragments per K step.
template <int NT, int TERMS, bool TIMED, bool PRE>
__global__ void __launch_bounds__(SABLE_THREADS)
spmm_tc_kernel(const LaunchArgs la, const int64_t part_stride) {
    extern __shared__ __align__(16) unsigned char smem[];
    long long t0 = 0;
    if (TIMED && threadIdx.x == 0) t0 = clock64();
    const int item = blockIdx.x, slice = blockIdx.y;
    const unsigned char *R = la.records + la.items[item].off;
    const MatIO &a = mat_of(la, reinterpret_cast<const ItemHeader *>(R)->mat);
    if (PRE)
        spmm_tc_item<NT, TERMS, true>(R, a, slice, part_stride, smem,
                                      static_cast<const uint4 *>(la.tcplanes) + la.tcoff[item]);
    else
        spmm_tc_item<NT, TERMS, false>(R, a, slice, part_stride, smem);
    if (TIMED) {
        __syncthreads();
        if (threadIdx.x == 0) la.cycles[(int64_t)slice * la.n_items + item] = (int64_t)(clock64() - t0);
    }
}

template <int NT, int TERMS, bool TIMED, bool PRE>
int launch_tc4(const LaunchArgs &a, int N, int64_t part_stride, cudaStream_t s) {
    dim3 grid(a.n_items, (N + NT - 1) / NT);
    const int smem = TcSmem<NT, PRE>::TOTAL;
    cudaFuncSetAttribute(spmm_tc_kernel<NT, TERMS, TIMED, PRE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    spmm_tc_kernel<NT, TERMS, TIMED, PRE><<<grid, SABLE_THREADS, smem, s>>>(a, part_stride);
    return (int)cudaGetLastError();
}

template <int NT, int TERMS, bool TIMED>
int launch_tc3(const LaunchArgs &a, int N, int64_t part_stride, cudaStream_t s) {
    return (a.tcplanes && a.tcoff) ? launch_tc4<NT, TERMS, TIMED, true>(a, N, part_stride, s)
                                   : launch_tc4<NT, TERMS, TIMED, false>(a, N, part_stride, s);
}

template <int NT>
int launch_tc(const LaunchArgs &a, int N, int terms, int64_t part_stride, bool timed, cudaStream_t s) {
    if (terms == 3) return timed ? launch_tc3<NT, 3, true>(a, N, part_stride, s) : launch_tc3<NT, 3, false>(a, N, part_stride, s);
    return timed ? launch_tc3<NT, 2, true>(a, N, part_stride, s) : launch_tc3<NT, 2, false>(a, N, part_stride, s);
}

}  // namespace

namespace sable {

int launch_spmm_tc(const LaunchArgs &a, int N, int nt, int terms, int64_t part_stride, bool timed, void *stream) {
    if (a.n_items <= 0 || N <= 0) return 0;
    if (terms != 2 && terms != 3) return (int)cudaErrorInvalidValue;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (nt) {
        case 32: return launch_tc<32>(a, N, terms, part_stride, timed, s);
        case 64: return launch_tc<64>(a, N, terms, part_stride, timed, s);
        case 128: return launch_tc<128>(a, N, terms, part_stride, timed, s);
        default: return (int)cudaErrorInvalidValue;
    }
}

void spmm_tc_free(sable_plan *p) {
    cudaFree(p->d_tcplanes);
    cudaFree(p->d_tcoff);
    p->d_tcplanes = nullptr;
    p->d_tcoff = nullptr;
}

}  // namespace sable
