// SpMM of one (item record, N-slice) work unit by one CTA of SABLE_THREADS
// threads: the bodies shared by the per-item kernels and the persistent batch
// kernel.  The caller passes the record (global memory), the matrix's MatIO,
// the slice and the dynamic shared memory (SpmmSmem<NT>::TOTAL or
// TcSmem<NT>::TOTAL bytes).
//
// FP32 form:
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
//
// Split-BF16 tensor-core form:
//
// Each FP32 value a of the dense panel and b of X is split into BF16 terms
// by repeated round-to-nearest: a_hi = bf16(a), a_mid = bf16(a - a_hi),
// a_lo = bf16(a - a_hi - a_mid).  Two precisions (Henry, Tang & Heinecke,
// "Leveraging the bfloat16 AI datatype for higher-precision computations",
// ARITH 2019):
//   TERMS = 2  a ~ a_hi + a_mid, three products hi*hi + hi*mid + mid*hi.
//              16 significant bits per operand: per product the error is at
//              most |a_mid b_mid| + |a r_b| + |r_a b| <= 3 * 2^-16 |a b|
//              (r = what the two terms leave out), ~1e-6 typical.
//   TERMS = 3  a ~ a_hi + a_mid + a_lo (24 bits, the whole FP32 significand),
//              six products hi*hi + hi*mid + mid*hi + hi*lo + lo*hi + mid*mid;
//              the dropped terms are below 2^-24 |a b|: FP32-level accuracy.
// The products run on the tensor cores as mma.sync m16n8k16 (BF16 in, FP32
// accumulate); the CSR entries of an item stay FP32 on the CUDA cores.
//
// Work item = (item record, N-slice of width NT <= 128), one CTA of 8 warps:
//   K loop over the item's panel columns, 16 at a time: the 16 X rows of the
//   panel columns (through the record's xcol table) are staged in shared
//   memory as FP32, and so are the A fragments: pre-split (PRE, the plan's
//   BF16 term fragments built once on the host, one 16-byte word per lane and
//   term) or the 4 FP32 panel quads, which every warp then splits per K step
//   (the batch kernel's form).  Every warp converts its B fragments (16 x 8)
//   to BF16 terms and issues 3 (TERMS = 2) or 6 (TERMS = 3) MMAs per 16 x 8
//   output tile.  Warps split the N-tiles first, then the M-tiles.
//   The accumulators go to the Y tile in shared memory, the CSR entries are
//   added by warp-owned row ranges (as in the FP32 kernel), and the tile is
//   stored (split tiles: partial tiles + last-arriving CTA, in item order).
#pragma once
#include <cuda_bf16.h>
#include "device_common.cuh"

namespace {

constexpr int KSTEP = 16;   // panel columns per staging step
constexpr int KSTAGES = 4;  // K steps in flight (cp.async pipeline depth)

// 16-byte asynchronous copy global -> shared; when !valid, nothing is read
// (src-size 0) and the 16 bytes are zero-filled.
__device__ __forceinline__ void cp16z(void *dst, const void *src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(valid ? 16 : 0) : "memory");
}

// Starts the copies of K step k0 into one stage: the KSTEP X rows of the
// step's panel columns (NT/4 float4 each, through colmap) and its KSTEP/4
// panel quads of every row.  Out-of-range parts are zero-filled.  The caller
// commits the group.
template <int NT>
__device__ __forceinline__ void stage_kstep(float4 *Bs, float4 *As, int k0, int ncol, const int *colmap,
                                            const float *X, int64_t ldx, int N, int n0, const float4 *P, int h,
                                            int nq) {
    constexpr int CQ = NT / 4;
    for (int t = threadIdx.x; t < KSTEP * CQ; t += SABLE_THREADS) {
        const int kk = t / CQ, q = t - kk * CQ, k = k0 + kk, n = n0 + 4 * q;
        const bool ok = k < ncol && n < N;
        const float *src = ok ? X + (int64_t)__ldg(colmap + k) * ldx + n : X;
        cp16z(&Bs[t], src, ok);
    }
    const int qbase = k0 >> 2;
    for (int t = threadIdx.x; t < (KSTEP / 4) * h; t += SABLE_THREADS) {
        const int qq = t / h, i = t - qq * h, q = qbase + qq;
        const bool ok = q < nq;
        cp16z(&As[qq * SABLE_MAX_ROW_TILE + i], ok ? P + (int64_t)q * h + i : P, ok);
    }
}

// Pre-split A fragments (built with the plan): for every K step ks and M
// tile mt of an item, TC_TERMS x 32 16-byte words in the order [ks][mt][term]
// [lane]; word (ks, mt, term, lane) holds the four packed BF16 pairs of
// lane's m16n8k16 A fragment of that term.
constexpr int TC_TERMS = 3;

// Starts the copies of the A fragments of K step ks (mtiles M tiles, all
// terms) into one stage; a step past the item's last is zero-filled.
__device__ __forceinline__ void stage_tc_planes(uint4 *Ap, const uint4 *planes, int ks, int nks, int mtiles) {
    const int n = mtiles * TC_TERMS * 32;
    const bool ok = ks < nks;
    const uint4 *src = planes + (int64_t)(ok ? ks : 0) * n;
    for (int t = threadIdx.x; t < n; t += SABLE_THREADS) cp16z(&Ap[t], ok ? src + t : planes, ok);
}

// Starts the copies of the KSTEP X rows of K step k0 only (pre-split A).
template <int NT>
__device__ __forceinline__ void stage_x_rows(float4 *Bs, int k0, int ncol, const int *colmap, const float *X,
                                             int64_t ldx, int N, int n0) {
    constexpr int CQ = NT / 4;
    for (int t = threadIdx.x; t < KSTEP * CQ; t += SABLE_THREADS) {
        const int kk = t / CQ, q = t - kk * CQ, k = k0 + kk, n = n0 + 4 * q;
        const bool ok = k < ncol && n < N;
        const float *src = ok ? X + (int64_t)__ldg(colmap + k) * ldx + n : X;
        cp16z(&Bs[t], src, ok);
    }
}

template <int NT>
struct SpmmSmem {
    static constexpr int CQ = NT / 4;
    static constexpr int YS = SABLE_MAX_ROW_TILE * NT * 4;         // Y tile
    static constexpr int BS = KSTEP * CQ * 16;                     // staged X rows
    static constexpr int AS = (KSTEP / 4) * SABLE_MAX_ROW_TILE * 16;  // staged quads
    static constexpr int RST = (SABLE_MAX_ROW_TILE + 8) * 4;
    // The K-loop stages share the space of the Y tile, which is only used
    // after the loop.
    static constexpr int OFF_BS = 0;                              // KSTAGES stages of X rows
    static constexpr int OFF_AS = OFF_BS + KSTAGES * BS;          // KSTAGES stages of quads
    static constexpr int LOOP = OFF_AS + KSTAGES * AS;
    static constexpr int OFF_RST = (YS > LOOP ? YS : LOOP);
    static constexpr int TOTAL = OFF_RST + RST;
};

template <int NT>
__device__ __forceinline__ void spmm_fp32_item(const unsigned char *R, const MatIO &a, int slice, int64_t part_stride,
                                               unsigned char *smem) {
    using L = SpmmSmem<NT>;
    constexpr int CQ = L::CQ;
    constexpr int RSUB = 32 / CQ;     // row (or entry) subgroups per warp
    constexpr int NRG = 8 * RSUB;     // row groups per CTA
    constexpr int RM = (SABLE_MAX_ROW_TILE + NRG - 1) / NRG;
    float4 *ys4 = reinterpret_cast<float4 *>(smem);
    float4 *Bs = reinterpret_cast<float4 *>(smem + L::OFF_BS);
    float4 *As = reinterpret_cast<float4 *>(smem + L::OFF_AS);
    int *rst = reinterpret_cast<int *>(smem + L::OFF_RST);
    __shared__ int s_last;
    __shared__ int s_wrow[9];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cq = lane % CQ, rs = lane / CQ, rg = warp * RSUB + rs;
    const ItemHeader c = *reinterpret_cast<const ItemHeader *>(R);
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
    // KSTAGES-deep pipeline: the copies of steps k+1 .. k+KSTAGES-1 are in
    // flight while step k is computed (one commit group per step, empty past
    // the end, so wait_group KSTAGES-1 always means "step k has landed")
    for (int st = 0; st < KSTAGES - 1; ++st) {
        if (st * KSTEP < ncol)
            stage_kstep<NT>(Bs + st * (KSTEP * CQ), As + st * ((KSTEP / 4) * SABLE_MAX_ROW_TILE), st * KSTEP, ncol,
                            colmap, X, a.ldx, a.N, n0, P, h, nq);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    int buf = 0;
    for (int k0 = 0; k0 < ncol; k0 += KSTEP, buf = (buf + 1) % KSTAGES) {
        const int nk = k0 + (KSTAGES - 1) * KSTEP, nb = (buf + KSTAGES - 1) % KSTAGES;
        if (nk < ncol)
            stage_kstep<NT>(Bs + nb * (KSTEP * CQ), As + nb * ((KSTEP / 4) * SABLE_MAX_ROW_TILE), nk, ncol, colmap, X,
                            a.ldx, a.N, n0, P, h, nq);
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group %0;" :: "n"(KSTAGES - 1) : "memory");
        __syncthreads();
        const float4 *Bsb = Bs + buf * (KSTEP * CQ);
        const float4 *Asb = As + buf * ((KSTEP / 4) * SABLE_MAX_ROW_TILE);
#pragma unroll
        for (int qq = 0; qq < KSTEP / 4; ++qq) {
            const float4 b0 = Bsb[(4 * qq + 0) * CQ + cq];
            const float4 b1 = Bsb[(4 * qq + 1) * CQ + cq];
            const float4 b2 = Bsb[(4 * qq + 2) * CQ + cq];
            const float4 b3 = Bsb[(4 * qq + 3) * CQ + cq];
#pragma unroll
            for (int m = 0; m < RM; ++m) {
                const int i = rg + NRG * m;
                if (i < h) {
                    const float4 av = Asb[qq * SABLE_MAX_ROW_TILE + i];
                    acc[m] = fma4(av.x, b0, acc[m]);
                    acc[m] = fma4(av.y, b1, acc[m]);
                    acc[m] = fma4(av.z, b2, acc[m]);
                    acc[m] = fma4(av.w, b3, acc[m]);
                }
            }
        }
        __syncthreads();
    }
    asm volatile("cp.async.wait_all;" ::: "memory");  // the Y tile reuses the stage space
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
        // split-K arrival as in cta_finish: barrier, one gpu-scope acq_rel
        // arrival, barrier; the last CTA reads the partials through L2
        __syncthreads();
        int *cnt = a.counters + (int64_t)slice * a.pad + c.tile;   // a.pad: split tiles per N-slice
        if (tid == 0) s_last = (arrive_acq_rel(cnt) == c.nitem - 1);
        __syncthreads();
        if (s_last) {
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
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// Split two FP32 values into TERMS packed BF16 pairs (low half = first value);
// t[0] is the leading term.  The differences are exact in FP32.
template <int TERMS>
__device__ __forceinline__ void split(float v0, float v1, uint32_t (&t)[TERMS]) {
#pragma unroll
    for (int k = 0; k < TERMS; ++k) {
        const __nv_bfloat16 a = __float2bfloat16_rn(v0), b = __float2bfloat16_rn(v1);
        t[k] = pack2(a, b);
        v0 -= __bfloat162float(a);
        v1 -= __bfloat162float(b);
    }
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int NT, bool PRE = false>
struct TcSmem {
    static constexpr int CQ = NT / 4;
    static constexpr int YS = SABLE_MAX_ROW_TILE * NT * 4;               // Y tile (FP32)
    static constexpr int BS = KSTEP * NT * 4;                            // staged X rows (FP32)
    static constexpr int AS = PRE ? (SABLE_MAX_ROW_TILE / 16) * TC_TERMS * 32 * 16  // staged A fragments
                                  : (KSTEP / 4) * SABLE_MAX_ROW_TILE * 16;         // staged quads
    static constexpr int RST = (SABLE_MAX_ROW_TILE + 8) * 4;
    // The K-loop stages share the space of the Y tile, which is only used
    // after the loop.
    static constexpr int OFF_BS = 0;                              // KSTAGES stages of X rows
    static constexpr int OFF_AS = OFF_BS + KSTAGES * BS;          // KSTAGES stages of quads
    static constexpr int LOOP = OFF_AS + KSTAGES * AS;
    static constexpr int OFF_RST = (YS > LOOP ? YS : LOOP);
    static constexpr int TOTAL = OFF_RST + RST;
};

// The end of a (tile item, N-slice) unit shared by the split-BF16 kernels:
// adds the item's CSR entries (FP32, CUDA cores; warps own row ranges of
// about ns/8 entries, lane subgroups combined by xor shuffles once per row)
// into the Y tile in shared memory, then stores the tile: directly for a
// single-item tile, else as a partial tile, the last-arriving CTA of the tile
// summing the partials in item order.  On entry every row < h of the Y tile
// (row-major h x NT floats at ys4) holds the dense part.
template <int NT>
__device__ __forceinline__ void spmm_tile_finish(const unsigned char *R, const ItemHeader &c, const MatIO &a,
                                                 int slice, int64_t part_stride, float4 *ys4, int *rst) {
    constexpr int CQ = NT / 4;
    constexpr int RSUB = 32 / CQ;
    __shared__ int s_last;
    __shared__ int s_wrow[9];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool act = tid < SABLE_THREADS;   // CTAs of more threads: the others only meet the barriers
    const int cq = lane % CQ, rs = lane / CQ;
    const int h = c.h, n0 = slice * NT;
    const float *__restrict__ X = a.x;
    // ---- CSR entries (FP32, CUDA cores) ----------------------------------------
    const bool col_ok = (n0 + 4 * cq) < a.N;
    __syncthreads();
    if (c.ns > 0) {
        const uint2 *__restrict__ E = reinterpret_cast<const uint2 *>(R + c.csr_off);
        const int ns = c.ns;
        if (act)
            for (int i = tid; i <= h; i += SABLE_THREADS) rst[i] = __ldg(reinterpret_cast<const int *>(R + c.rp_off) + i);
        __syncthreads();
        if (warp == 0 && lane < 9) {
            const int target = (int)(((int64_t)ns * lane) / 8);
            int lo = 0, hi = h;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (rst[mid] >= target) hi = mid; else lo = mid + 1;
            }
            s_wrow[lane] = lane == 8 ? h : lo;
        }
        __syncthreads();
        // A row's entries go 32 at a time: one coalesced load (an entry per
        // lane), then each row subgroup rs takes entries rs, rs + RSUB, ... of
        // the chunk by shuffle, CSR_U X rows in flight per lane, so no X load
        // waits for its entry's load.  Each lane adds its entries in
        // increasing order, as one entry at a time would.
        constexpr int CSR_U = 4;
        if constexpr (RSUB == 1) {
            // NT = 128: the 32 lanes are the 32 column quads, so a warp streams
            // the entries of all its rows as one sequence (rows are contiguous)
            // and adds a row's sum into the Y tile when the sequence leaves it:
            // the X loads of consecutive rows overlap instead of each row
            // paying its own load latencies.
            const int r_lo = act ? s_wrow[warp] : 0, r_hi = act ? s_wrow[warp + 1] : 0;
            if (r_lo < r_hi) {
                const int e_lo = rst[r_lo], e_hi = rst[r_hi];
                int r = r_lo, r_end = rst[r_lo + 1];
                float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int c0 = e_lo; c0 < e_hi; c0 += 32) {
                    const int cnt = min(32, e_hi - c0);
                    const uint2 mine = lane < cnt ? __ldg(E + c0 + lane) : make_uint2(0u, 0u);
                    for (int k0 = 0; k0 < cnt; k0 += CSR_U) {
                        float4 xv[CSR_U];
                        float vv[CSR_U];
#pragma unroll
                        for (int u = 0; u < CSR_U; ++u) {
                            const int k = k0 + u;
                            const int src = k < 32 ? k : 31;
                            vv[u] = __uint_as_float(__shfl_sync(FULL, mine.x, src));
                            const uint32_t col = __shfl_sync(FULL, mine.y, src);
                            xv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                            if (k < cnt && col_ok)
                                xv[u] = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)col * a.ldx + n0 + 4 * cq));
                        }
#pragma unroll
                        for (int u = 0; u < CSR_U; ++u) {
                            const int k = k0 + u;
                            if (k >= cnt) break;
                            while (c0 + k >= r_end) {   // row r is complete (warp-uniform)
                                if (r_end > rst[r]) ys4[r * CQ + cq] = add4(ys4[r * CQ + cq], s);
                                s = make_float4(0.f, 0.f, 0.f, 0.f);
                                ++r;
                                r_end = rst[r + 1];
                            }
                            if (col_ok) s = fma4(vv[u], xv[u], s);
                        }
                    }
                }
                if (e_hi > e_lo) ys4[r * CQ + cq] = add4(ys4[r * CQ + cq], s);   // the last entry's row
            }
        } else
        for (int r = act ? s_wrow[warp] : 0; r < (act ? s_wrow[warp + 1] : 0); ++r) {
            const int b = rst[r], e = rst[r + 1];
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int c0 = b; c0 < e; c0 += 32) {
                const int cnt = min(32, e - c0);
                const uint2 mine = lane < cnt ? __ldg(E + c0 + lane) : make_uint2(0u, 0u);
                for (int k0 = 0; k0 < cnt; k0 += CSR_U * RSUB) {
                    float4 xv[CSR_U];
                    float vv[CSR_U];
#pragma unroll
                    for (int u = 0; u < CSR_U; ++u) {
                        const int k = k0 + u * RSUB + rs;
                        const int src = k < 32 ? k : 31;
                        vv[u] = __uint_as_float(__shfl_sync(FULL, mine.x, src));
                        const uint32_t col = __shfl_sync(FULL, mine.y, src);
                        xv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (k < cnt && col_ok)
                            xv[u] = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)col * a.ldx + n0 + 4 * cq));
                    }
#pragma unroll
                    for (int u = 0; u < CSR_U; ++u)
                        if (k0 + u * RSUB + rs < cnt && col_ok) s = fma4(vv[u], xv[u], s);
                }
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

    // ---- output -------------------------------------------------------------------
    const bool split = c.nitem > 1;
    const int64_t pbase = (int64_t)slice * part_stride + (c.part_base + (int64_t)c.kidx * h) * NT;
    for (int e = tid; act && e < h * CQ; e += SABLE_THREADS) {
        const int i = e / CQ, q = e - i * CQ, n = n0 + 4 * q;
        if (n >= a.N) continue;
        const float4 v = ys4[i * CQ + q];
        if (!split) *reinterpret_cast<float4 *>(a.y + (int64_t)(c.row0 + i) * a.ldy + n) = v;
        else *reinterpret_cast<float4 *>(a.partial + pbase + (int64_t)i * NT + 4 * q) = v;
    }
    if (split) {
        // split-K arrival as in cta_finish: barrier, one gpu-scope acq_rel
        // arrival, barrier; the last CTA reads the partials through L2
        __syncthreads();
        int *cnt = a.counters + (int64_t)slice * a.pad + c.tile;
        if (tid == 0) s_last = (arrive_acq_rel(cnt) == c.nitem - 1);
        __syncthreads();
        if (s_last) {
            const int64_t tb = (int64_t)slice * part_stride + c.part_base * NT;
            for (int e = tid; act && e < h * CQ; e += SABLE_THREADS) {
                const int i = e / CQ, q = e - i * CQ, n = n0 + 4 * q;
                if (n >= a.N) continue;
                float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < c.nitem; ++k)
                    s = add4(s, __ldcg(reinterpret_cast<const float4 *>(a.partial + tb + ((int64_t)k * h + i) * NT + 4 * q)));
                *reinterpret_cast<float4 *>(a.y + (int64_t)(c.row0 + i) * a.ldy + n) = s;
            }
            if (tid == 0) *cnt = 0;
        }
    }
}

// PRE: the item's A fragments come pre-split (planes: the item's words, see
// stage_tc_planes) instead of being split from the FP32 panel on every step.
template <int NT, int TERMS, bool PRE = false>
__device__ __forceinline__ void spmm_tc_item(const unsigned char *R, const MatIO &a, int slice, int64_t part_stride,
                                             unsigned char *smem, const uint4 *planes = nullptr) {
    using L = TcSmem<NT, PRE>;
    constexpr int CQ = L::CQ;
    constexpr int NTILES = NT / 8;                        // 8-column MMA tiles of the slice
    constexpr int WN = NTILES < 4 ? NTILES : 4;           // warps along N (4 x 2 grid: each A fragment is
                                                          // split by 4 warps, not 8)
    constexpr int WM = 8 / WN;                            // warps along M
    constexpr int NPW = (NTILES + WN - 1) / WN;           // N-tiles per warp
    constexpr int MPW = (SABLE_MAX_ROW_TILE / 16 + WM - 1) / WM;  // M-tiles per warp (max)
    float *ys = reinterpret_cast<float *>(smem);
    float4 *ys4 = reinterpret_cast<float4 *>(smem);
    float *Bs = reinterpret_cast<float *>(smem + L::OFF_BS);
    float4 *As = reinterpret_cast<float4 *>(smem + L::OFF_AS);
    int *rst = reinterpret_cast<int *>(smem + L::OFF_RST);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;                 // MMA fragment coordinates
    const int wn = warp % WN, wm = warp / WN;
    const ItemHeader c = *reinterpret_cast<const ItemHeader *>(R);
    const int h = c.h, nq = c.nq, ncol = 4 * nq;
    const int mtiles = (h + 15) / 16;
    const int n0 = slice * NT;
    const float *__restrict__ X = a.x;
    const int *colmap = reinterpret_cast<const int *>(R + c.xcol_off);
    const float4 *__restrict__ P = reinterpret_cast<const float4 *>(R + c.panel_off);

    float acc[MPW][NPW][4];
#pragma unroll
    for (int i = 0; i < MPW; ++i)
#pragma unroll
        for (int j = 0; j < NPW; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;

    // KSTAGES-deep pipeline, as in spmm_fp32_item
    float4 *Bs4 = reinterpret_cast<float4 *>(Bs);
    constexpr int ASTAGE = L::AS / 16;  // float4 / uint4 words of one A stage
    uint4 *Ap = reinterpret_cast<uint4 *>(As);
    const int nks = (ncol + KSTEP - 1) / KSTEP;
    auto stage = [&](int k0, int sb) {
        if (PRE) {
            stage_x_rows<NT>(Bs4 + sb * (KSTEP * CQ), k0, ncol, colmap, X, a.ldx, a.N, n0);
            stage_tc_planes(Ap + sb * ASTAGE, planes, k0 / KSTEP, nks, mtiles);
        } else {
            stage_kstep<NT>(Bs4 + sb * (KSTEP * CQ), As + sb * ASTAGE, k0, ncol, colmap, X, a.ldx, a.N, n0, P, h, nq);
        }
    };
    for (int st = 0; st < KSTAGES - 1; ++st) {
        if (st * KSTEP < ncol) stage(st * KSTEP, st);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    int buf = 0;
    for (int k0 = 0; k0 < ncol; k0 += KSTEP, buf = (buf + 1) % KSTAGES) {
        const int nk = k0 + (KSTAGES - 1) * KSTEP, nb = (buf + KSTAGES - 1) % KSTAGES;
        if (nk < ncol) stage(nk, nb);
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group %0;" :: "n"(KSTAGES - 1) : "memory");
        __syncthreads();
        const float *Bsb = Bs + buf * (KSTEP * NT);
        const float *Af = reinterpret_cast<const float *>(As + buf * ASTAGE);
        const uint4 *Apb = Ap + buf * ASTAGE;
        // B fragments of this warp's N-tiles: bt[j][term][register]
        uint32_t bt[NPW][TERMS][2];
#pragma unroll
        for (int j = 0; j < NPW; ++j) {
            const int nt = wn + j * WN;
            const int col = nt * 8 + g;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
            if (nt < NTILES) {
                v0 = Bsb[(2 * t) * NT + col];
                v1 = Bsb[(2 * t + 1) * NT + col];
                v2 = Bsb[(2 * t + 8) * NT + col];
                v3 = Bsb[(2 * t + 9) * NT + col];
            }
            uint32_t s0[TERMS], s1[TERMS];
            split<TERMS>(v0, v1, s0);
            split<TERMS>(v2, v3, s1);
#pragma unroll
            for (int k = 0; k < TERMS; ++k) {
                bt[j][k][0] = s0[k];
                bt[j][k][1] = s1[k];
            }
        }
#pragma unroll
        for (int i = 0; i < MPW; ++i) {
            const int mt = wm + i * WM;
            if (mt >= mtiles) continue;
            // A fragment rows r0 = 16 mt + g, r1 = r0 + 8; columns 2t, 2t+1 (+8)
            uint32_t at[TERMS][4];
            if (PRE) {
#pragma unroll
                for (int k = 0; k < TERMS; ++k) {
                    const uint4 w = Apb[(mt * TC_TERMS + k) * 32 + lane];
                    at[k][0] = w.x;
                    at[k][1] = w.y;
                    at[k][2] = w.z;
                    at[k][3] = w.w;
                }
            } else {
                const int r0 = mt * 16 + g, r1 = r0 + 8;
                // column c of the K-step lives in quad c/4, component c%4: A(row, c) = Af[((c/4)*128 + row)*4 + c%4]
                auto ld2 = [&](int row, int col) {
                    if (row >= h) return make_float2(0.f, 0.f);
                    return *reinterpret_cast<const float2 *>(Af + ((col >> 2) * SABLE_MAX_ROW_TILE + row) * 4 + (col & 3));
                };
                const float2 a00 = ld2(r0, 2 * t), a10 = ld2(r1, 2 * t), a01 = ld2(r0, 2 * t + 8), a11 = ld2(r1, 2 * t + 8);
                uint32_t s00[TERMS], s10[TERMS], s01[TERMS], s11[TERMS];
                split<TERMS>(a00.x, a00.y, s00);
                split<TERMS>(a10.x, a10.y, s10);
                split<TERMS>(a01.x, a01.y, s01);
                split<TERMS>(a11.x, a11.y, s11);
#pragma unroll
                for (int k = 0; k < TERMS; ++k) {
                    at[k][0] = s00[k];
                    at[k][1] = s10[k];
                    at[k][2] = s01[k];
                    at[k][3] = s11[k];
                }
            }
            // products in the order (a-term, b-term), smallest terms first; the
            // N-tile loop inside, so consecutive MMAs go to independent
            // accumulators
            constexpr int NPROD = TERMS == 3 ? 6 : 3;
            constexpr int PA[6] = {1, 0, 2, 0, 1, 0}, PB[6] = {1, 2, 0, 1, 0, 0};
            constexpr int QA[3] = {0, 1, 0}, QB[3] = {1, 0, 0};
#pragma unroll
            for (int pr = 0; pr < NPROD; ++pr) {
                const int ta = TERMS == 3 ? PA[pr] : QA[pr], tb = TERMS == 3 ? PB[pr] : QB[pr];
#pragma unroll
                for (int j = 0; j < NPW; ++j) {
                    if (wn + j * WN >= NTILES) continue;
                    mma_bf16(acc[i][j], at[ta], bt[j][tb]);
                }
            }
        }
        __syncthreads();
    }
    // accumulators -> Y tile (rows >= h are not stored; all rows < h are written);
    // the Y tile reuses the stage space
    asm volatile("cp.async.wait_all;" ::: "memory");
    for (int e = tid; e < h * CQ; e += SABLE_THREADS) ys4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < MPW; ++i) {
        const int mt = wm + i * WM;
        if (mt >= mtiles) continue;
#pragma unroll
        for (int j = 0; j < NPW; ++j) {
            const int nt = wn + j * WN;
            if (nt >= NTILES) continue;
            const int r0 = mt * 16 + g, col = nt * 8 + 2 * t;
            if (r0 < h) {
                ys[r0 * NT + col] = acc[i][j][0];
                ys[r0 * NT + col + 1] = acc[i][j][1];
            }
            if (r0 + 8 < h) {
                ys[(r0 + 8) * NT + col] = acc[i][j][2];
                ys[(r0 + 8) * NT + col + 1] = acc[i][j][3];
            }
        }
    }

    spmm_tile_finish<NT>(R, c, a, slice, part_stride, ys4, rst);
}

}  // namespace
