// SpMM entry point that allocates no memory.
//
// sable_spmm keeps the partial sums of split tiles in a scratch buffer that it
// allocates with cudaMalloc the first time a plan is run at a given width.
// Some callers cannot let a library allocate device memory during a call:
// runtimes that hand all device memory to their own pool allocator up front
// and forbid later cudaMalloc (the allocation fails, or takes memory the pool
// counted on), and real-time or safety-critical loops that must not block on
// the driver's allocator.  sable_spmm_noalloc gives them the same SpMM kernels
// as sable_spmm (FP32, or split BF16 on the tensor cores when the plan has it
// and N >= 32) with the scratch in a fixed, file-scope device array instead.
//
// When the array is reserved: with CUDA's lazy module loading (the default),
// a device reserves the array when this library's device code is first
// loaded on it, which is at the latest the first sable_spmm_noalloc call on
// that device (its cudaGetSymbolAddress loads the module).  A caller whose
// pool allocator takes the whole device should make one call (any plan, any
// width) before the pool is created, so that the array is already reserved.
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace {

// Fixed scratch, held by every device that loads the library until exit:
// 2 Mi floats (8 MiB) of split-tile partial sums and 64 Ki arrival counters
// (256 KiB).
constexpr int64_t NOALLOC_PARTIAL_FLOATS = 2 << 20;
constexpr int64_t NOALLOC_COUNTERS = 64 << 10;
static __device__ __align__(256) float g_noalloc_partial[NOALLOC_PARTIAL_FLOATS];
static __device__ __align__(256) int g_noalloc_counters[NOALLOC_COUNTERS];

// Device addresses of the two arrays, looked up once per device.  In host
// code the array names are host-side stand-ins, not device addresses.
constexpr int MAX_DEVICES = 64;
struct ScratchAddr {
    bool ready = false;
    float *partial = nullptr;
    int *counters = nullptr;
};
ScratchAddr g_addr[MAX_DEVICES];
std::mutex g_addr_mutex;

int scratch_for_current_device(int dev, ScratchAddr *out) {
    if (dev < 0 || dev >= MAX_DEVICES) return sable::fail(SABLE_ERR_UNSUPPORTED, "device %d beyond %d", dev, MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    ScratchAddr &s = g_addr[dev];
    if (!s.ready) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
        if (e != cudaSuccess) return sable::cuda_fail(e, "cudaGetSymbolAddress(partial scratch)");
        s.partial = static_cast<float *>(p);
        e = cudaGetSymbolAddress(&p, g_noalloc_counters);
        if (e != cudaSuccess) return sable::cuda_fail(e, "cudaGetSymbolAddress(counter scratch)");
        s.counters = static_cast<int *>(p);
        s.ready = true;
    }
    *out = s;
    return SABLE_OK;
}

}  // namespace

using namespace sable;

extern "C" int sable_spmm_noalloc(sable_plan *p, const float *X_dev, int64_t ldx, float *Y_dev, int64_t ldy, int32_t N,
                                  void *stream) {
    if (!p || !X_dev || !Y_dev) return fail(SABLE_ERR_ARG, "null argument");
    if (N <= 0 || (N & 3) || (ldx & 3) || (ldy & 3) || ldx < N || ldy < N)
        return fail(SABLE_ERR_UNSUPPORTED, "SpMM needs N %% 4 == 0 and ld >= N, ld %% 4 == 0 (N=%d ldx=%lld ldy=%lld)", N,
                    (long long)ldx, (long long)ldy);
    if (((uintptr_t)X_dev & 15) || ((uintptr_t)Y_dev & 15))
        return fail(SABLE_ERR_UNSUPPORTED, "SpMM operands must be 16-byte aligned");
    if (p->compact) return fail(SABLE_ERR_UNSUPPORTED, "a plan of the per-warp SpMV executor (schedule 2) runs SpMV only");
    int rc = set_device(p->device);
    if (rc) return rc;
    const int nt = spmm_slice_width(N);
    const int n_slices = (N + nt - 1) / nt;
    const int64_t need_partial = p->n_partial * nt * n_slices;
    const int64_t need_counters = (int64_t)std::max<int32_t>(p->n_split_tiles, 1) * n_slices;
    if (need_partial > NOALLOC_PARTIAL_FLOATS || need_counters > NOALLOC_COUNTERS)
        return fail(SABLE_ERR_UNSUPPORTED,
                    "this plan at N=%d needs %lld partial floats and %lld counters; the fixed scratch of "
                    "sable_spmm_noalloc holds %lld and %lld (use sable_spmm, or larger work items)",
                    N, (long long)need_partial, (long long)need_counters, (long long)NOALLOC_PARTIAL_FLOATS,
                    (long long)NOALLOC_COUNTERS);
    ScratchAddr s;
    rc = scratch_for_current_device(p->device, &s);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The arrays keep the previous call's contents; the arrival counters must
    // start at zero (partial sums are written before they are read).
    cudaError_t e = cudaMemsetAsync(s.counters, 0, (size_t)need_counters * sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "clear counter scratch");
    LaunchArgs a;
    memset(&a, 0, sizeof a);
    a.records = p->d_records;
    a.items = p->d_items;
    a.mat0.x = X_dev;
    a.mat0.y = Y_dev;
    a.mat0.partial = s.partial;
    a.mat0.counters = s.counters;
    a.mat0.ldx = ldx;
    a.mat0.ldy = ldy;
    a.mat0.N = N;
    a.mat0.pad = std::max<int32_t>(p->n_split_tiles, 1);
    a.error = p->d_error;
    a.n_items = (int)p->n_items;
    a.stage_bytes = p->max_item_bytes;
    // the same kernel choice as sable_spmm (split BF16 on the tensor cores for
    // plans built with them at N >= 32, else FP32)
    const int err = launch_spmm_plan(p, a, N, nt, false, stream);
    if (err) return cuda_fail((cudaError_t)err, "spmm (fixed scratch) launch");
    return SABLE_OK;
}
