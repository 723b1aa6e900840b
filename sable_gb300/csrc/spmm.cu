// VBR SpMM, FP32 on the CUDA cores (the plain SpMM form) for sm_103a.
//
// Replaces gen_single_threaded_spmm (src/codegen.py:827-937): dense blocks
// through spmm_kernel (i-j-k loops, :851-859) and sparse blocks unrolled per
// nonzero (:906-922, DSL :150-163).  X and Y are row-major with width N
// (the reference fixes N = 512); one work item covers a chunk of a tile and
// an N-slice of width NT <= 128.
//
// Per work item (CTA of 256 threads):
//   dense   the chunk's panel columns are walked 16 at a time: their X rows
//           (gathered through the run table) and the 4 panel quads are
//           staged in shared memory; each thread owns RM rows x 4 columns of
//           the Y tile in registers (lanes span the N-slice, warps the rows).
//   sparse  a row histogram of the chunk's CSR entries gives row starts; each
//           warp owns a contiguous row range with about 1/8 of the entries
//           and walks it with lanes spanning the N-slice, combining entries
//           of one row with a shuffle segmented scan; the warp adds segment
//           tails into its own rows of the Y tile (fixed order, reproducible).
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
    static constexpr int RUNS = SABLE_MAX_CHUNK_RUNS * 16;
    static constexpr int RST = (SABLE_MAX_ROW_TILE + 8) * 4;
    static constexpr int OFF_BS = YS;
    static constexpr int OFF_AS = OFF_BS + BS;
    static constexpr int OFF_RUNS = OFF_AS + AS;
    static constexpr int OFF_RST = OFF_RUNS + RUNS;
    static constexpr int OFF_COLMAP = OFF_RST + RST;  // int[4 * max_quads]
};

template <int NT, bool TIMED>
__global__ void __launch_bounds__(SABLE_THREADS)
spmm_fp32_kernel(const SpmmArgs a) {
    using L = SpmmSmem<NT>;
    constexpr int CQ = L::CQ;
    constexpr int RSUB = 32 / CQ;     // row (or entry) subgroups per warp
    constexpr int NRG = 8 * RSUB;     // row groups per CTA
    constexpr int RM = (SABLE_MAX_ROW_TILE + NRG - 1) / NRG;
    extern __shared__ __align__(16) unsigned char smem[];
    float4 *ys4 = reinterpret_cast<float4 *>(smem);
    float4 *Bs = reinterpret_cast<float4 *>(smem + L::OFF_BS);
    float4 *As = reinterpret_cast<float4 *>(smem + L::OFF_AS);
    int4 *runs = reinterpret_cast<int4 *>(smem + L::OFF_RUNS);
    int *rst = reinterpret_cast<int *>(smem + L::OFF_RST);
    int *colmap = reinterpret_cast<int *>(smem + L::OFF_COLMAP);
    __shared__ int s_last;
    __shared__ int s_wrow[9];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cq = lane % CQ, rs = lane / CQ, rg = warp * RSUB + rs;
    const int chunk_id = blockIdx.x, slice = blockIdx.y;
    long long t0 = 0;
    if (TIMED && tid == 0) t0 = clock64();
    const Chunk c = a.chunks[chunk_id];
    const int h = c.h, nq = c.nq, ncol = 4 * nq;
    const int n0 = slice * NT;
    const bool col_ok = (n0 + 4 * cq) < a.N;
    const float *__restrict__ X = a.X;

    for (int r = tid; r < c.nrun; r += SABLE_THREADS) runs[r] = __ldg(a.runs + c.run0 + r);
    __syncthreads();
    // column map of the chunk: panel column -> X row (-1 for padding)
    for (int k = tid; k < ncol; k += SABLE_THREADS) {
        int col = -1;
        if (c.nrun > 0) {
            int lo = 0, hi = c.nrun - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (runs[mid].x <= k) lo = mid; else hi = mid - 1;
            }
            const int4 r = runs[lo];
            const int d = k - r.x;
            if (d >= 0 && d < r.z) col = r.y + d;
        }
        colmap[k] = col;
    }
    __syncthreads();

    // ---- dense panel: register-blocked tile GEMM ---------------------------
    float4 acc[RM];
#pragma unroll
    for (int m = 0; m < RM; ++m) acc[m] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 *__restrict__ P = a.panel + c.panel_f4;
    for (int k0 = 0; k0 < ncol; k0 += KSTEP) {
        for (int t = tid; t < KSTEP * CQ; t += SABLE_THREADS) {
            const int kk = t / CQ, q = t - kk * CQ, k = k0 + kk, n = n0 + 4 * q;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < ncol && n < a.N) {
                const int col = colmap[k];
                if (col >= 0) v = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)col * a.ldx + n));
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

    // ---- CSR entries ------------------------------------------------------
    if (c.ns > 0) {
        const uint2 *__restrict__ E = a.sparse + c.sp0;
        const int ns = c.ns;
        for (int i = tid; i <= h; i += SABLE_THREADS) rst[i] = 0;
        __syncthreads();
        for (int e = tid; e < ns; e += SABLE_THREADS) atomicAdd(rst + 1 + int(__ldg(&E[e].y) >> SABLE_COL_BITS), 1);
        __syncthreads();
        if (warp == 0) {  // inclusive scan of rst[1..h] -> row starts
            int carry = 0;
            for (int b = 1; b <= h; b += 32) {
                int v = (b + lane <= h) ? rst[b + lane] : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(FULL, v, o);
                    if (lane >= o) v += t;
                }
                if (b + lane <= h) rst[b + lane] = v + carry;
                carry += __shfl_sync(FULL, v, 31);
            }
            // warp row ranges with about ns/8 entries each
            if (lane < 9) {
                const int target = (int)(((int64_t)ns * lane) / 8);
                int lo = 0, hi = h;  // first row r with rst[r] >= target
                while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (rst[mid] >= target) hi = mid; else lo = mid + 1;
                }
                s_wrow[lane] = lane == 8 ? h : lo;
            }
        }
        __syncthreads();
        const int e_lo = rst[s_wrow[warp]], e_hi = rst[s_wrow[warp + 1]];
        for (int base = e_lo; base < e_hi; base += RSUB * 4) {
            uint2 en[4];
            float4 xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = base + u * RSUB + rs;
                en[u] = e < e_hi ? __ldg(E + e) : make_uint2(0u, 0u);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = base + u * RSUB + rs;
                xv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (e < e_hi && col_ok)
                    xv[u] = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)(en[u].y & SABLE_COL_MASK) * a.ldx + n0 + 4 * cq));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = base + u * RSUB + rs;
                const bool ok = e < e_hi;
                const int key = ok ? int(en[u].y >> SABLE_COL_BITS) : -1;
                const float v = __uint_as_float(en[u].x);
                float4 s = ok ? make_float4(v * xv[u].x, v * xv[u].y, v * xv[u].z, v * xv[u].w)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int o = 1; o < RSUB; o <<= 1) {
                    const int src = lane - o * CQ;
                    float4 t;
                    t.x = __shfl_sync(FULL, s.x, src < 0 ? lane : src);
                    t.y = __shfl_sync(FULL, s.y, src < 0 ? lane : src);
                    t.z = __shfl_sync(FULL, s.z, src < 0 ? lane : src);
                    t.w = __shfl_sync(FULL, s.w, src < 0 ? lane : src);
                    const int kk = __shfl_sync(FULL, key, src < 0 ? lane : src);
                    if (rs >= o && kk == key) s = add4(s, t);
                }
                const int nx = lane + CQ;
                const int knext = __shfl_sync(FULL, key, nx < 32 ? nx : lane);
                const bool tail = (rs == RSUB - 1) || (knext != key);
                if (tail && key >= 0) ys4[key * CQ + cq] = add4(ys4[key * CQ + cq], s);
                __syncwarp();
            }
        }
    }
    __syncthreads();

    // ---- output -------------------------------------------------------------
    const bool split = c.nchunk > 1;
    const int64_t pbase = (int64_t)slice * a.part_stride + (c.part_base + (int64_t)c.kidx * h) * NT;
    for (int t = tid; t < h * CQ; t += SABLE_THREADS) {
        const int i = t / CQ, q = t - i * CQ, n = n0 + 4 * q;
        if (n >= a.N) continue;
        const float4 v = ys4[i * CQ + q];
        if (!split) *reinterpret_cast<float4 *>(a.Y + (int64_t)(c.row0 + i) * a.ldy + n) = v;
        else *reinterpret_cast<float4 *>(a.partial + pbase + (int64_t)i * NT + 4 * q) = v;
    }
    if (split) {
        __threadfence();
        __syncthreads();
        const int cidx = slice * 0 + c.tile;  // counters are laid out per slice below
        if (tid == 0) s_last = (atomicAdd(a.counters + (int64_t)slice * a.n_chunks + cidx, 1) == c.nchunk - 1);
        __syncthreads();
        if (s_last) {
            __threadfence();
            const int64_t tb = (int64_t)slice * a.part_stride + c.part_base * NT;
            for (int t = tid; t < h * CQ; t += SABLE_THREADS) {
                const int i = t / CQ, q = t - i * CQ, n = n0 + 4 * q;
                if (n >= a.N) continue;
                float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < c.nchunk; ++k)
                    s = add4(s, __ldcg(reinterpret_cast<const float4 *>(a.partial + tb + ((int64_t)k * h + i) * NT + 4 * q)));
                *reinterpret_cast<float4 *>(a.Y + (int64_t)(c.row0 + i) * a.ldy + n) = s;
            }
            if (tid == 0) a.counters[(int64_t)slice * a.n_chunks + cidx] = 0;
        }
    }
    if (TIMED) {
        __syncthreads();
        if (tid == 0) a.ns_out[(int64_t)slice * a.n_chunks + chunk_id] = (int64_t)(clock64() - t0);
    }
}

template <int NT>
int launch_nt(const SpmmArgs &a, int smem, bool timed, cudaStream_t s) {
    dim3 grid(a.n_chunks, a.n_slices);
    if (timed) {
        cudaFuncSetAttribute(spmm_fp32_kernel<NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        spmm_fp32_kernel<NT, true><<<grid, SABLE_THREADS, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(spmm_fp32_kernel<NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        spmm_fp32_kernel<NT, false><<<grid, SABLE_THREADS, smem, s>>>(a);
    }
    return (int)cudaGetLastError();
}

}  // namespace

namespace sable {

int spmm_smem_bytes(int nt, int max_quads, int max_runs, int row_tile) {
    (void)max_runs;
    (void)row_tile;
    int off = 0;
    switch (nt) {
        case 4: off = SpmmSmem<4>::OFF_COLMAP; break;
        case 8: off = SpmmSmem<8>::OFF_COLMAP; break;
        case 16: off = SpmmSmem<16>::OFF_COLMAP; break;
        case 32: off = SpmmSmem<32>::OFF_COLMAP; break;
        case 64: off = SpmmSmem<64>::OFF_COLMAP; break;
        default: off = SpmmSmem<128>::OFF_COLMAP; break;
    }
    return off + 4 * 4 * (max_quads > 0 ? max_quads : 1);
}

int launch_spmm_fp32(const SpmmArgs &a, int smem, bool timed, void *stream) {
    if (a.n_chunks <= 0 || a.n_slices <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (a.nt) {
        case 4: return launch_nt<4>(a, smem, timed, s);
        case 8: return launch_nt<8>(a, smem, timed, s);
        case 16: return launch_nt<16>(a, smem, timed, s);
        case 32: return launch_nt<32>(a, smem, timed, s);
        case 64: return launch_nt<64>(a, smem, timed, s);
        case 128: return launch_nt<128>(a, smem, timed, s);
        default: return (int)cudaErrorInvalidValue;
    }
}

}  // namespace sable
