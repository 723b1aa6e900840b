// VBR SpMM, FP32 on the CUDA cores (the plain SpMM form) for sm_103a.
//
// Replaces gen_single_threaded_spmm (src/codegen.py:827-937): dense blocks
// through spmm_kernel (i-j-k loops, :851-859) and sparse blocks unrolled per
// nonzero (:906-922, DSL :150-163).  X and Y are row-major with width N
// (the reference fixes N = 512); one work item covers a chunk of a tile and
// an N-slice of width NT <= 128.
//
// Per work item (CTA of 256 threads):
//   dense   the item's panel columns are walked 16 at a time: their X rows
//           (gathered through the record's xcol table) and the 4 panel quads are
//           staged in shared memory; each thread owns RM rows x 4 columns of
//           the Y tile in registers (lanes span the N-slice, warps the rows).
//   sparse  each warp owns a contiguous row range holding about 1/8 of the
//           item's CSR entries (row pointers of the item) and walks it row by
//           row, lanes spanning the N-slice; the lane subgroups of a warp are
//           combined by xor shuffles once per row and the warp adds the row
//           into its own rows of the Y tile (fixed order, reproducible).
//   output  single-chunk tiles store Y directly; split tiles publish partial
//           tiles and the last-arriving CTA sums them in chunk order.
#include <cuda_runtime.h>
#include <stdint.h>
#include "sable_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int KSTEP = 16;  // panel columns per staging step

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

template <int NT>
struct SpmmSmem {
    static constexpr int CQ = NT / 4;
    static constexpr int YS = SABLE_MAX_ROW_TILE * NT * 4;         // Y tile
    static constexpr int BS = KSTEP * CQ * 16;                     // staged X rows
    static constexpr int AS = (KSTEP / 4) * SABLE_MAX_ROW_TILE * 16;  // staged quads
    static constexpr int RST = (SABLE_MAX_ROW_TILE + 8) * 4;
    static constexpr int OFF_BS = YS;
    static constexpr int OFF_AS = OFF_BS + BS;
    static constexpr int OFF_RST = OFF_AS + AS;
    static constexpr int TOTAL = OFF_RST + RST;
};

template <int NT, bool TIMED>
__global__ void __launch_bounds__(SABLE_THREADS)
spmm_fp32_kernel(const LaunchArgs la, const int64_t part_stride) {
    using L = SpmmSmem<NT>;
    constexpr int CQ = L::CQ;
    constexpr int RSUB = 32 / CQ;     // row (or entry) subgroups per warp
    constexpr int NRG = 8 * RSUB;     // row groups per CTA
    constexpr int RM = (SABLE_MAX_ROW_TILE + NRG - 1) / NRG;
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *ys4 = reinterpret_cast<float4 *>(smem);
    float4 *Bs = reinterpret_cast<float4 *>(smem + L::OFF_BS);
    float4 *As = reinterpret_cast<float4 *>(smem + L::OFF_AS);
    int *rst = reinterpret_cast<int *>(smem + L::OFF_RST);
    __shared__ int s_last;
    __shared__ int s_wrow[9];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cq = lane % CQ, rs = lane / CQ, rg = warp * RSUB + rs;
    const int chunk_id = blockIdx.x, slice = blockIdx.y;
    long long t0 = 0;
    if (TIMED && tid == 0) t0 = clock64();
    const ItemRef ref = la.items[chunk_id];
    const unsigned char *R = la.records + ref.off;
    const ItemHeader c = *reinterpret_cast<const ItemHeader *>(R);
    const MatIO &a = la.mats ? la.mats[c.mat] : la.mat0;
    const int h = c.h, nq = c.nq, ncol = 4 * nq;
    const int n0 = slice * NT;
    const bool col_ok = (n0 + 4 * cq) < a.N;
    const float *__restrict__ X = a.x;
    const int *colmap = reinterpret_cast<const int *>(R + c.xcol_off);   // panel column -> X row

    // ---- dense panel: register-blocked tile GEMM ---------------------------
    float4 acc[RM];
#pragma unroll
    for (int m = 0; m < RM; ++m) acc[m] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 *__restrict__ P = reinterpret_cast<const float4 *>(R + c.panel_off);
    for (int k0 = 0; k0 < ncol; k0 += KSTEP) {
        for (int t = tid; t < KSTEP * CQ; t += SABLE_THREADS) {
            const int kk = t / CQ, q = t - kk * CQ, k = k0 + kk, n = n0 + 4 * q;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < ncol && n < a.N) {
                const int col = __ldg(colmap + k);
                v = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)col * a.ldx + n));
            }
            Bs[t] = v;
        }
        const int qbase = k0 >> 2;
        for (int t = tid; t < (KSTEP / 4) * h; t += SABLE_THREADS) {
            const int qq = t / h, i = t - qq * h, q = qbase + qq;
            As[qq * SABLE_MAX_ROW_TILE + i] =
                q < nq ? __ldcs(P + (int64_t)q * h + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
#pragma unroll
        for (int qq = 0; qq < KSTEP / 4; ++qq) {
            const float4 b0 = Bs[(4 * qq + 0) * CQ + cq];
            const float4 b1 = Bs[(4 * qq + 1) * CQ + cq];
            const float4 b2 = Bs[(4 * qq + 2) * CQ + cq];
            const float4 b3 = Bs[(4 * qq + 3) * CQ + cq];
#pragma unroll
            for (int m = 0; m < RM; ++m) {
                const int i = rg + NRG * m;
                if (i < h) {
                    const float4 av = As[qq * SABLE_MAX_ROW_TILE + i];
                    acc[m] = fma4(av.x, b0, acc[m]);
                    acc[m] = fma4(av.y, b1, acc[m]);
                    acc[m] = fma4(av.z, b2, acc[m]);
                    acc[m] = fma4(av.w, b3, acc[m]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < RM; ++m) {
        const int i = rg + NRG * m;
        if (i < h) ys4[i * CQ + cq] = acc[m];
    }

    // ---- CSR entries: warps own row ranges of about ns/8 entries -------------
    if (c.ns > 0) {
        const uint2 *__restrict__ E = reinterpret_cast<const uint2 *>(R + c.csr_off);
        const int ns = c.ns;
        for (int i = tid; i <= h; i += SABLE_THREADS) rst[i] = __ldg(reinterpret_cast<const int *>(R + c.rp_off) + i);
        __syncthreads();
        if (warp == 0 && lane < 9) {
            const int target = (int)(((int64_t)ns * lane) / 8);
            int lo = 0, hi = h;  // first row r with rst[r] >= target
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (rst[mid] >= target) hi = mid; else lo = mid + 1;
            }
            s_wrow[lane] = lane == 8 ? h : lo;
        }
        __syncthreads();
        for (int r = s_wrow[warp]; r < s_wrow[warp + 1]; ++r) {
            const int b = rst[r], e = rst[r + 1];
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int base = b; base < e; base += RSUB * 4) {
                uint2 en[4];
                float4 xv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = base + u * RSUB + rs;
                    en[u] = i < e ? __ldg(E + i) : make_uint2(0u, 0u);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = base + u * RSUB + rs;
                    xv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (i < e && col_ok)
                        xv[u] = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)en[u].y * a.ldx + n0 + 4 * cq));
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) s = fma4(__uint_as_float(en[u].x), xv[u], s);
            }
#pragma unroll
            for (int o = CQ; o < 32; o <<= 1) {
                s.x += __shfl_xor_sync(FULL, s.x, o);
                s.y += __shfl_xor_sync(FULL, s.y, o);
                s.z += __shfl_xor_sync(FULL, s.z, o);
                s.w += __shfl_xor_sync(FULL, s.w, o);
            }
            if (rs == 0 && e > b) ys4[r * CQ + cq] = add4(ys4[r * CQ + cq], s);
        }
    }
    __syncthreads();

    // ---- output -------------------------------------------------------------
    const bool split = c.nitem > 1;
    const int64_t pbase = (int64_t)slice * part_stride + (c.part_base + (int64_t)c.kidx * h) * NT;
    for (int t = tid; t < h * CQ; t += SABLE_THREADS) {
        const int i = t / CQ, q = t - i * CQ, n = n0 + 4 * q;
        if (n >= a.N) continue;
        const float4 v = ys4[i * CQ + q];
        if (!split) *reinterpret_cast<float4 *>(a.y + (int64_t)(c.row0 + i) * a.ldy + n) = v;
        else *reinterpret_cast<float4 *>(a.partial + pbase + (int64_t)i * NT + 4 * q) = v;
    }
    if (split) {
        __threadfence();
        __syncthreads();
        int *cnt = a.counters + (int64_t)slice * a.pad + c.tile;   // a.pad: split tiles per N-slice
        if (tid == 0) s_last = (atomicAdd(cnt, 1) == c.nitem - 1);
        __syncthreads();
        if (s_last) {
            __threadfence();
            const int64_t tb = (int64_t)slice * part_stride + c.part_base * NT;
            for (int t = tid; t < h * CQ; t += SABLE_THREADS) {
                const int i = t / CQ, q = t - i * CQ, n = n0 + 4 * q;
                if (n >= a.N) continue;
                float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < c.nitem; ++k)
                    s = add4(s, __ldcg(reinterpret_cast<const float4 *>(a.partial + tb + ((int64_t)k * h + i) * NT + 4 * q)));
                *reinterpret_cast<float4 *>(a.y + (int64_t)(c.row0 + i) * a.ldy + n) = s;
            }
            if (tid == 0) *cnt = 0;
        }
    }
    if (TIMED) {
        __syncthreads();
        if (tid == 0) la.cycles[(int64_t)slice * la.n_items + chunk_id] = (int64_t)(clock64() - t0);
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
