// VBR SpMM kernels over item records: one CTA per (item, N-slice), bodies in
// spmm_item.cuh.  spmm_fp32_kernel is the plain FP32 form; the split-BF16
// tensor-core form is in spmm_tc.cu.
#include <cuda_runtime.h>
#include <stdint.h>
#include "sable_internal.h"
#include "spmm_item.cuh"

namespace {

template <int NT, bool TIMED>
__global__ void __launch_bounds__(SABLE_THREADS)
spmm_fp32_kernel(const LaunchArgs la, const int64_t part_stride) {
    extern __shared__ __align__(16) unsigned char smem[];
    long long t0 = 0;
    if (TIMED && threadIdx.x == 0) t0 = clock64();
    const int item = blockIdx.x, slice = blockIdx.y;
    const unsigned char *R = la.records + la.items[item].off;
    const MatIO &a = mat_of(la, reinterpret_cast<const ItemHeader *>(R)->mat);
    spmm_fp32_item<NT>(R, a, slice, part_stride, smem);
    if (TIMED) {
        __syncthreads();
        if (threadIdx.x == 0) la.cycles[(int64_t)slice * la.n_items + item] = (int64_t)(clock64() - t0);
    }
}

template <int NT>
int launch_nt(const LaunchArgs &a, int N, int64_t part_stride, bool timed, cudaStream_t s) {
    dim3 grid(a.n_items, (N + NT - 1) / NT);
    const int smem = SpmmSmem<NT>::TOTAL;
    if (timed) {
        cudaFuncSetAttribute(spmm_fp32_kernel<NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        spmm_fp32_kernel<NT, true><<<grid, SABLE_THREADS, smem, s>>>(a, part_stride);
    } else {
        cudaFuncSetAttribute(spmm_fp32_kernel<NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        spmm_fp32_kernel<NT, false><<<grid, SABLE_THREADS, smem, s>>>(a, part_stride);
    }
    return (int)cudaGetLastError();
}

}  // namespace

namespace sable {

int launch_spmm_fp32(const LaunchArgs &a, int N, int nt, int64_t part_stride, bool timed, void *stream) {
    if (a.n_items <= 0 || N <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (nt) {
        case 4: return launch_nt<4>(a, N, part_stride, timed, s);
        case 8: return launch_nt<8>(a, N, part_stride, timed, s);
        case 16: return launch_nt<16>(a, N, part_stride, timed, s);
        case 32: return launch_nt<32>(a, N, part_stride, timed, s);
        case 64: return launch_nt<64>(a, N, part_stride, timed, s);
        case 128: return launch_nt<128>(a, N, part_stride, timed, s);
        default: return (int)cudaErrorInvalidValue;
    }
}

}  // namespace sable
