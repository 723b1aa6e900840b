// Self-test of the bounded waits every kernel of this library uses (no
// counterpart in the reference).  One thread initialises an mbarrier and
// waits for its first phase with a short limit; nothing arrives unless
// `arrive` asks the thread to arrive first.  Without the arrival the wait
// runs out, the kernel records that in a status word, and the host returns
// SABLE_ERR_TIMEOUT: the failure path of the kernels' waits, exercised with no
// fault, trap or endless loop, leaving the context usable.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"
#include "device_common.cuh"

namespace {

__global__ void wait_selftest_kernel(unsigned long long limit_ns, int arrive, unsigned long long *out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(smem_addr(&bar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_addr(&bar)) : "memory");
    const unsigned long long t0 = global_ns();
    const bool ok = mbar_wait_for(smem_addr(&bar), 0u, limit_ns);
    out[0] = ok ? 0ull : 1ull;
    out[1] = global_ns() - t0;
}

}  // namespace

using namespace sable;

extern "C" int sable_selftest_wait(int64_t limit_us, int32_t arrive, int64_t *elapsed_ns, void *stream) {
    if (limit_us < 1 || limit_us > 2000000) return fail(SABLE_ERR_ARG, "limit_us must be in 1..2000000");
    unsigned long long *d = nullptr;
    cudaError_t e = cudaMalloc((void **)&d, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "self-test buffer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    wait_selftest_kernel<<<1, 32, 0, s>>>((unsigned long long)limit_us * 1000ull, arrive ? 1 : 0, d);
    unsigned long long h[2] = {1ull, 0ull};
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "self-test wait kernel");
    if (elapsed_ns) *elapsed_ns = (int64_t)h[1];
    if (h[0]) return fail(SABLE_ERR_TIMEOUT, "self-test: the bounded wait ran out after %lld ns", (long long)h[1]);
    return SABLE_OK;
}
