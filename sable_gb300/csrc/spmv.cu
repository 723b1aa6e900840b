// VBR SpMV kernel for sm_103a: one CTA per work item (chunk) of a plan.
//
// Replaces the per-block call sequence of the generated executor
// (src/codegen.py:414-439: MKL CSR product with beta = 0, then one
// spmv_kernel call per dense block, src/codegen.py:263-291).
//
// Per work item:
//   1. the x values of the chunk's dense columns are gathered into shared
//      memory (xs), so that each 16-byte panel word meets its 4 x values in
//      one shared-memory load;
//   2. dense panel: 1024 virtual threads (4 per thread) each own one row of
//      the tile and walk the panel with stride h*floor(1024/h) words, so a
//      warp always reads 32 consecutive 16-byte words and accumulates in a
//      register with no atomics;
//   3. CSR entries: each warp reads 32 consecutive 8-byte entries, forms
//      value * x[col], and reduces equal rows with a shuffle segmented scan;
//      segment tails add into the warp's own row buffer;
//   4. per row, the dense partials and the 8 warp buffers are summed in a
//      fixed order, so results are bitwise reproducible run to run;
//   5. a tile split over several chunks publishes its partial row sums and
//      the last-arriving CTA adds them in chunk order.
#include <cuda_runtime.h>
#include <stdint.h>
#include "sable_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int RED_FLOATS = SABLE_THREADS * SABLE_VT;              // 1024
constexpr int YSW_FLOATS = (SABLE_THREADS / 32) * SABLE_MAX_ROW_TILE;  // 8 x 128
constexpr int RUNS_OFF = (RED_FLOATS + YSW_FLOATS) * 4;           // bytes
constexpr int XS_OFF = RUNS_OFF + SABLE_MAX_CHUNK_RUNS * 16;      // bytes

__device__ __forceinline__ float dot4(const float4 a, const float4 b, float acc) {
    acc = fmaf(a.x, b.x, acc);
    acc = fmaf(a.y, b.y, acc);
    acc = fmaf(a.z, b.z, acc);
    acc = fmaf(a.w, b.w, acc);
    return acc;
}

// Fill xs[0 .. 4*nq) from x through the chunk's run table (already in smem).
__device__ __forceinline__ void stage_x(float *xs, const int4 *runs, int nrun, int ncol,
                                        const float *__restrict__ x) {
    for (int k = threadIdx.x; k < ncol; k += SABLE_THREADS) {
        float v = 0.f;
        if (nrun > 0) {
            int lo = 0, hi = nrun - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (runs[mid].x <= k) lo = mid; else hi = mid - 1;
            }
            const int4 r = runs[lo];
            const int d = k - r.x;
            if (d >= 0 && d < r.z) v = __ldg(x + r.y + d);
        }
        xs[k] = v;
    }
}

template <bool TIMED>
__device__ __forceinline__ void spmv_one_chunk(const SpmvArgs &a, const int chunk_id, unsigned char *smem) {
    float *red = reinterpret_cast<float *>(smem);
    float *ysw = red + RED_FLOATS;
    int4 *runs = reinterpret_cast<int4 *>(smem + RUNS_OFF);
    float4 *xs4 = reinterpret_cast<float4 *>(smem + XS_OFF);
    __shared__ int s_last;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    long long t0 = 0;
    if (TIMED && tid == 0) t0 = clock64();

    const Chunk c = a.chunks[chunk_id];
    const int h = c.h;

    for (int r = tid; r < c.nrun; r += SABLE_THREADS) runs[r] = __ldg(a.runs + c.run0 + r);
    for (int i = tid; i < YSW_FLOATS; i += SABLE_THREADS) ysw[i] = 0.f;
    __syncthreads();
    if (c.nq > 0) stage_x(reinterpret_cast<float *>(xs4), runs, c.nrun, 4 * c.nq, a.x);
    __syncthreads();

    // ---- dense quad panel -------------------------------------------------
    int per = 0;  // quads advanced per sweep of the 1024 virtual threads
    if (c.nq > 0) {
        per = RED_FLOATS / h;
        const int tp = per * h;
        const float4 *__restrict__ P = a.panel + c.panel_f4;
        float acc[SABLE_VT];
        int vq[SABLE_VT], vr[SABLE_VT];
#pragma unroll
        for (int m = 0; m < SABLE_VT; ++m) {
            const int v = tid + SABLE_THREADS * m;
            acc[m] = 0.f;
            vq[m] = v < tp ? v / h : (1 << 29);
            vr[m] = v < tp ? v - (v / h) * h : 0;
        }
        const int nq = c.nq;
        for (int base = 0; base < nq; base += 2 * per) {
            float4 A0[SABLE_VT], A1[SABLE_VT];
#pragma unroll
            for (int m = 0; m < SABLE_VT; ++m) {
                const int q0 = vq[m] + base, q1 = q0 + per;
                A0[m] = q0 < nq ? __ldcs(P + (int64_t)q0 * h + vr[m]) : make_float4(0.f, 0.f, 0.f, 0.f);
                A1[m] = q1 < nq ? __ldcs(P + (int64_t)q1 * h + vr[m]) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int m = 0; m < SABLE_VT; ++m) {
                const int q0 = vq[m] + base, q1 = q0 + per;
                if (q0 < nq) acc[m] = dot4(A0[m], xs4[q0], acc[m]);
                if (q1 < nq) acc[m] = dot4(A1[m], xs4[q1], acc[m]);
            }
        }
#pragma unroll
        for (int m = 0; m < SABLE_VT; ++m) {
            const int v = tid + SABLE_THREADS * m;
            if (v < tp) red[v] = acc[m];
        }
    }

    // ---- CSR entries ------------------------------------------------------
    if (c.ns > 0) {
        const uint2 *__restrict__ E = a.sparse + c.sp0;
        float *myw = ysw + warp * SABLE_MAX_ROW_TILE;
        const int ns = c.ns;
        for (int g0 = warp * 32; g0 < ns; g0 += SABLE_THREADS * 4) {
            uint2 e[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int idx = g0 + u * SABLE_THREADS + lane;
                e[u] = idx < ns ? __ldcs(E + idx) : make_uint2(0u, 0u);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int idx = g0 + u * SABLE_THREADS + lane;
                const bool ok = idx < ns;
                const int key = ok ? int(e[u].y >> SABLE_COL_BITS) : -1;
                float s = ok ? __uint_as_float(e[u].x) * __ldg(a.x + (e[u].y & SABLE_COL_MASK)) : 0.f;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const float t = __shfl_up_sync(FULL, s, o);
                    const int kk = __shfl_up_sync(FULL, key, o);
                    if (lane >= o && kk == key) s += t;
                }
                const int knext = __shfl_down_sync(FULL, key, 1);
                const bool tail = (lane == 31) || (knext != key);
                if (tail && key >= 0) myw[key] += s;
            }
        }
    }
    __syncthreads();

    // ---- fixed-order row reduction and output ------------------------------
    const bool split = c.nchunk > 1;
    for (int i = warp; i < h; i += SABLE_THREADS / 32) {
        float s = 0.f;
        for (int k = lane; k < per; k += 32) s += red[k * h + i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) {
            float sp = 0.f;
#pragma unroll
            for (int w = 0; w < SABLE_THREADS / 32; ++w) sp += ysw[w * SABLE_MAX_ROW_TILE + i];
            const float tot = s + sp;
            if (!split) a.y[c.row0 + i] = tot;
            else a.partial[c.part_base + (int64_t)c.kidx * h + i] = tot;
        }
    }
    if (split) {
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = (atomicAdd(a.counters + c.tile, 1) == c.nchunk - 1);
        __syncthreads();
        if (s_last) {
            __threadfence();
            for (int i = tid; i < h; i += SABLE_THREADS) {
                float s = 0.f;
                for (int k = 0; k < c.nchunk; ++k) s += __ldcg(a.partial + c.part_base + (int64_t)k * h + i);
                a.y[c.row0 + i] = s;
            }
            if (tid == 0) a.counters[c.tile] = 0;  // ready for the next launch
        }
    }
    if (TIMED) {
        __syncthreads();
        if (tid == 0) a.ns_out[chunk_id] = (int64_t)(clock64() - t0);
    }
}

template <bool TIMED>
__global__ void __launch_bounds__(SABLE_THREADS)
spmv_chunk_kernel(const SpmvArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    spmv_one_chunk<TIMED>(a, blockIdx.x, smem);
}

}  // namespace

namespace sable {

int spmv_smem_bytes(int max_quads, int max_runs) {
    (void)max_runs;
    return XS_OFF + 16 * (max_quads > 0 ? max_quads : 1);
}

int launch_spmv(const SpmvArgs &a, int smem_bytes, bool timed, void *stream) {
    if (a.n_chunks <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (timed) {
        cudaFuncSetAttribute(spmv_chunk_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
        spmv_chunk_kernel<true><<<a.n_chunks, SABLE_THREADS, smem_bytes, s>>>(a);
    } else {
        cudaFuncSetAttribute(spmv_chunk_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
        spmv_chunk_kernel<false><<<a.n_chunks, SABLE_THREADS, smem_bytes, s>>>(a);
    }
    return (int)cudaGetLastError();
}

}  // namespace sable
