// VBR SpMV kernels for sm_103a over item records (layout in sable_internal.h).
//
// Replaces the per-block call sequence of the generated executor
// (src/codegen.py:414-439: MKL CSR product with beta = 0, then one
// spmv_kernel call per dense block, src/codegen.py:263-291).
//
//   spmv_items_kernel  one CTA (8 warps) per item: a single TMA bulk copy
//                      (cp.async.bulk, completion counted on an mbarrier)
//                      brings the item's record into shared memory; x values
//                      are read through L1.  Split tiles are combined by a
//                      separate combine launch.  This is the plain form and
//                      the one the timed entry points use for schedules 0-1.
//   spmv_warp_items_kernel  one warp per compact item (schedule 2; described
//                      with the kernel below), the fastest on large matrices.
//   spmv_warp_kernel   persistent warp workers: every warp walks its own
//                      LPT-balanced list of parts (runs of items of one tile)
//                      through a private 2-slot TMA ring; while item k is
//                      computed, the record of item k+1 is in flight and its
//                      x values are being gathered into shared memory with
//                      cp.async.  A warp accumulates a whole part in
//                      registers (every lane owns rows) and writes its rows
//                      once; only parts of very large tiles combine across
//                      workers.  No CTA-wide barrier is ever taken.
// Dense panel: lanes own rows (rows l, l+32, ... for h > 32; for h <= 32 a
// warp step covers floor(32/h) quads), so a warp reads up to 32 consecutive
// 16-byte words per step.  CSR entries: groups of g lanes per row (g chosen
// per item from its mean row length) and one xor-shuffle reduction per row.
// All sums run in a fixed order: results are bitwise reproducible.
// Every mbarrier wait is bounded (2 s); on expiry the plan's error flag is
// set and the worker waits (bounded again) for its own copies, then returns.
#include <algorithm>
#include <cuda_runtime.h>
#include <stdint.h>
#include "sable_internal.h"
#include "spmv_item.cuh"

namespace {

template <bool TIMED>
__global__ void __launch_bounds__(SABLE_THREADS)
spmv_items_kernel(const LaunchArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    float *red = reinterpret_cast<float *>(smem);
    float *ysw = red + RED_FLOATS;
    unsigned char *stage = smem + STAGE_OFF;
    __shared__ __align__(8) unsigned long long s_bar;
    const int tid = threadIdx.x;
    long long t0 = 0;
    if (TIMED && tid == 0) t0 = clock64();
    const unsigned bar = smem_addr(&s_bar);
    const ItemRef ref = a.items[blockIdx.x];
    if (tid == CTRL) {
        mbar_init(bar);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < RED_FLOATS; i += SABLE_THREADS) ysw[i] = 0.f;
    __syncthreads();  // the barrier is initialised before anyone waits on it
    // One thread waits for the record; the CTA barrier then publishes it to
    // the others.  A record whose header disagrees with the item table is
    // never used.
    bool landed = true, bad = false;
    if (tid == CTRL) {
        tma_record(bar, stage, a.records + ref.off, (unsigned)ref.bytes);
        landed = mbar_wait(bar, 0);
        bad = !landed || reinterpret_cast<const ItemHeader *>(stage)->bytes != ref.bytes;
    }
    if (__syncthreads_or(bad)) {
        if (tid == CTRL) {
            atomicExch(a.error, 1);
            if (!landed) mbar_wait(bar, 0);
        }
        return;
    }
    const ItemHeader hd = *reinterpret_cast<const ItemHeader *>(stage);
    const MatIO &io = mat_of(a, hd.mat);
    cta_accumulate(stage, hd, io.x, nullptr, red, ysw);
    __syncthreads();
    cta_finish(hd, io, red, ysw);
    if (TIMED) {
        __syncthreads();
        if (tid == 0) a.cycles[blockIdx.x] = (int64_t)(clock64() - t0);
    }
}

// ---------------------------------------------------------------------------
// One warp per work item (schedule 2), over compact records.  The record is
// read straight from HBM with coalesced streaming loads after a bulk L2
// prefetch of its head: no shared-memory staging of the record, no TMA wait and no CTA
// barrier, so every warp of the SM is an independent stream.  The item's x
// window (panel columns, then the columns of its CSR entries) is gathered
// once into shared memory from its column runs, so neither part waits on a
// column index before its x load.  Dense panel: for h <= 32 a warp step
// covers floor(32/h) quads (lane = (row, quad offset)), eight per lane in
// flight; for 32 < h <= 64 lanes own rows lane and lane+32, two quads per
// step.  CSR entries: 256 per warp step (8 per lane: values and 16-bit
// window position / row words), the next step's loads issued before this
// step's row sums, which a segmented scan over the lanes adds into a
// per-warp row buffer in shared memory (warp-synchronous only).  The items
// of a split tile store partial row sums and the last one to arrive adds
// them, so a launch needs no combine pass.
// ---------------------------------------------------------------------------
constexpr int WI_WARPS = 4;       // warps (one item each) per CTA of the per-warp executor
constexpr int WI_XW = SABLE_CW_MAX;  // x window floats per warp
constexpr int WI_GU = 8;          // window positions per lane in flight while gathering

__device__ __forceinline__ float4 ld_stream(const float4 *p) { return __ldcs(p); }

// One bulk L2 prefetch of the first bytes of a record (16-byte aligned, a
// multiple of 16 bytes): the header, the window runs and the first panel
// steps are in L2 by the time the warp asks for them.  Only the head: with
// whole records prefetched, the first wave of warps put ~130 MB of requests
// before DRAM at once, their headers waited behind them and the SMs took
// about 5 us to reach full occupancy (1.5 us with an 8 KB head); the kernel
// was 6 % slower on the 100000^2 workload.  Prefetching the rest later (after
// the window gather, rolling ahead of the panel, or the next item's head) was
// slower or no faster: the warps' own loads stream the body.
constexpr int WI_PREFETCH_BYTES = 8192;
__device__ __forceinline__ void prefetch_record(const unsigned char *R, int bytes) {
    const unsigned n = (unsigned)min(bytes, WI_PREFETCH_BYTES);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(R), "r"(n) : "memory");
}

// The x window of a compact record into xw[0, nw).  Runs are taken 32 at a
// time, one per lane; every lane finds the run of each of its positions by a
// binary search over the lanes' run starts (shuffles only; the WI_GU searches
// of a lane are independent, so they overlap), and keeps WI_GU x loads in
// flight.  A run with column -1 reads as zeros.
__device__ __forceinline__ void gather_window(const int2 *runs, int nrun, const float *__restrict__ x, float *xw,
                                              int lane) {
    constexpr int ZERO = -(1 << 30);  // column offset of a zero run: offset + position < 0
    int wbase = 0;
    for (int r0 = 0; r0 < nrun; r0 += 32) {
        const int nr = min(32, nrun - r0);
        const int2 run = lane < nr ? runs[r0 + lane] : make_int2(0, 0);
        int incl = run.y;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const int start = wbase + incl - run.y;
        const int key = lane < nr ? start : 0x7fffffff;                     // lanes without a run never match
        const int coff = (lane < nr && run.x >= 0) ? run.x - start : ZERO;  // x column = coff + position
        const int bend = __shfl_sync(FULL, wbase + incl, 31);
        for (int p0 = wbase; p0 < bend; p0 += 32 * WI_GU) {
            float v[WI_GU];
#pragma unroll
            for (int u = 0; u < WI_GU; ++u) {
                const int p = p0 + lane + 32 * u;
                int j = 0;  // last lane whose run starts at or before p
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1)
                    if (__shfl_sync(FULL, key, j + step) <= p) j += step;
                const int col = __shfl_sync(FULL, coff, j) + p;
                v[u] = (p < bend && col >= 0) ? __ldg(x + col) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < WI_GU; ++u) {
                const int p = p0 + lane + 32 * u;
                if (p < bend) xw[p] = v[u];
            }
        }
        wbase = bend;
    }
}

// CSR entries of a compact record, 256 per warp step: lane l takes the 8
// consecutive entries 8l..8l+7 of the step (two 16-byte value loads, one
// 16-byte load of their meta words), multiplies each value by its x from
// the window and sums the products by row in registers.  Entries are sorted
// by row, so a lane's entries form a few row segments: a segment that starts
// and ends inside the lane is complete and is added to rows[] at once; the
// lanes' last segments are summed by a scan inside each group of lanes that
// end on the same row, and the group's last lane adds the total plus the
// next lane's first segment when that continues the row.
// Every row of a step is added to rows[] by exactly one lane, and all sums
// run in a fixed order.  Entries past ns take row CW_NOROW and are dropped.
constexpr int CW_NOROW = 127;

__device__ __forceinline__ void warp_csr_window(const float *val, const uint16_t *meta, int ns, int lane,
                                                const float *xw, float *rows) {
    // raw loads of a step (the record holds whole groups of 8 up to ns)
    auto fetch = [&](int c0, float4 &va, float4 &vb, uint4 &mw) {
        const int e0 = c0 + 8 * lane;
        if (e0 < ns) {
            va = *reinterpret_cast<const float4 *>(val + e0);
            vb = *reinterpret_cast<const float4 *>(val + e0 + 4);
            mw = *reinterpret_cast<const uint4 *>(meta + e0);
        } else {
            va = vb = make_float4(0.f, 0.f, 0.f, 0.f);
            mw = make_uint4(0u, 0u, 0u, 0u);
        }
    };
    float4 va, vb;
    uint4 mw;
    fetch(0, va, vb, mw);
    for (int c0 = 0; c0 < ns; c0 += 256) {
        // the next step's loads go out before this step's sums (one step ahead)
        float4 na = va, nb = vb;
        uint4 nm = mw;
        if (c0 + 256 < ns) fetch(c0 + 256, na, nb, nm);
        const int e0 = c0 + 8 * lane;
        float v[8];
        int r[8];
        {
            const unsigned m[4] = {mw.x, mw.y, mw.z, mw.w};
            const float vv[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const unsigned mk = (m[k >> 1] >> (16 * (k & 1))) & 0xffffu;
                const bool live = e0 + k < ns;
                v[k] = live ? vv[k] * xw[mk & 1023u] : 0.f;
                r[k] = live ? (int)(mk >> 10) : CW_NOROW;
            }
        }
        va = na;
        vb = nb;
        mw = nm;
        // row segments inside the lane
        int rf = r[0], rl = r[0];
        float sf = 0.f, sl = v[0];
        bool multi = false;
#pragma unroll
        for (int k = 1; k < 8; ++k) {
            if (r[k] == rl) {
                sl += v[k];
            } else {
                if (!multi) sf = sl;                    // the first segment ends
                else if (rl < CW_NOROW) rows[rl] += sl;  // a middle segment: complete, this lane's alone
                multi = true;
                rl = r[k];
                sl = v[k];
            }
        }
        if (!multi) sf = sl;
        // The lanes whose last segment is row rl form one contiguous group
        // (rows never decrease along the entries): an inclusive scan inside
        // the group leaves the group's total in its last lane.
        const unsigned grp = __match_any_sync(FULL, rl);
        const int gfirst = __ffs(grp) - 1, glast = 31 - __clz(grp);
        float acc = sl;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float t = __shfl_up_sync(FULL, acc, o);
            if (lane - o >= gfirst) acc += t;
        }
        // The first segment of a multi-segment lane: added here when it
        // starts a row, by the previous lane's group when it continues it.
        const int prev_rl = __shfl_up_sync(FULL, rl, 1);
        const bool cont = multi && lane > 0 && prev_rl == rf;
        const float to_prev = __shfl_down_sync(FULL, cont ? sf : 0.f, 1);
        if (multi && !cont && rf < CW_NOROW) rows[rf] += sf;
        if (lane == glast && rl < CW_NOROW) rows[rl] += lane < 31 ? acc + to_prev : acc;
        __syncwarp();
    }
}

// One compact work item by one warp (every lane calls it with the same
// item): the x window into shared memory, CSR entries into the tile's rows,
// the panel quads against the window, and the rows written to y or, for a
// split tile, to the item's partial rows, the last of the tile's items adding
// them into y.  rows: SABLE_CW_MAX_ROWS floats, xw: WI_XW floats of the
// warp's shared memory.  TIMED: SM cycles of the item into a.cycles[item].
template <bool TIMED, bool BATCH>
__device__ __forceinline__ void warp_item(const LaunchArgs &a, int item, int64_t off, int bytes, int lane, float *rows,
                                          float *xw, int mat) {
    long long t0 = 0;
    if (TIMED && lane == 0) t0 = clock64();
    const unsigned char *R = a.records + off;
    const CompactHeader hd = *reinterpret_cast<const CompactHeader *>(R);
    if (hd.bytes != bytes || hd.h < 1 || hd.h > SABLE_CW_MAX_ROWS || hd.nw > WI_XW) {
        if (lane == 0) atomicExch(a.error, 1);
        return;
    }
    const MatIO &io = BATCH ? a.mats[mat] : a.mat0;
    const int h = hd.h, nq = hd.nq, ns = hd.ns;
    __syncwarp();  // the previous item's reads of rows / xw are done
    for (int i = lane; i < h; i += 32) rows[i] = 0.f;
    gather_window(reinterpret_cast<const int2 *>(R + hd.runs_off), hd.nrun, io.x, xw, lane);
    __syncwarp();
    if (ns > 0)
        warp_csr_window(reinterpret_cast<const float *>(R + hd.val_off), reinterpret_cast<const uint16_t *>(R + hd.meta_off),
                        ns, lane, xw, rows);
    const float4 *P = reinterpret_cast<const float4 *>(R + hd.panel_off);
    const float4 *xw4 = reinterpret_cast<const float4 *>(xw);
    auto put = [&](int i, float v) {
        if (hd.nitem <= 1) io.y[hd.row0 + i] = v;
        else io.partial[hd.part_base + (int64_t)hd.kidx * h + i] = v;
    };
    if (h <= 32) {
        const int qpw = 32 / h, r = lane % h, sidx = lane / h;
        float a0 = 0.f, a1 = 0.f;
        if (lane < qpw * h) {
            int q = sidx;
            for (; q + 7 * qpw < nq; q += 8 * qpw) {  // 8 quads per lane in flight
                float4 p[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) p[k] = ld_stream(P + (q + k * qpw) * h + r);
#pragma unroll
                for (int k = 0; k < 8; k += 2) {
                    a0 = dot4(p[k], xw4[q + k * qpw], a0);
                    a1 = dot4(p[k + 1], xw4[q + (k + 1) * qpw], a1);
                }
            }
            for (; q + 3 * qpw < nq; q += 4 * qpw) {
                const float4 p0 = ld_stream(P + q * h + r), p1 = ld_stream(P + (q + qpw) * h + r);
                const float4 p2 = ld_stream(P + (q + 2 * qpw) * h + r), p3 = ld_stream(P + (q + 3 * qpw) * h + r);
                a0 = dot4(p0, xw4[q], a0);
                a1 = dot4(p1, xw4[q + qpw], a1);
                a0 = dot4(p2, xw4[q + 2 * qpw], a0);
                a1 = dot4(p3, xw4[q + 3 * qpw], a1);
            }
            for (; q < nq; q += qpw) a0 = dot4(ld_stream(P + q * h + r), xw4[q], a0);
        }
        const float v = a0 + a1;
        float tot = 0.f;
        for (int k = 0; k < qpw; ++k) tot += __shfl_sync(FULL, v, r + k * h);  // fixed order over the quad offsets
        __syncwarp();
        if (lane < h) put(lane, tot + rows[lane]);
    } else {  // 32 < h <= 64: lanes own rows lane and lane + 32
        const bool v1 = lane + 32 < h;
        float c0 = 0.f, c1 = 0.f;
        int q = 0;
        for (; q + 1 < nq; q += 2) {
            const float4 xa = xw4[q], xb = xw4[q + 1];
            const float4 *Pa = P + q * h + lane, *Pb = Pa + h;
            const float4 pa0 = ld_stream(Pa), pb0 = ld_stream(Pb);
            float4 pa1 = make_float4(0.f, 0.f, 0.f, 0.f), pb1 = pa1;
            if (v1) { pa1 = ld_stream(Pa + 32); pb1 = ld_stream(Pb + 32); }
            c0 = dot4(pb0, xb, dot4(pa0, xa, c0));
            c1 = dot4(pb1, xb, dot4(pa1, xa, c1));
        }
        if (q < nq) {
            const float4 xa = xw4[q];
            const float4 *Pa = P + q * h + lane;
            c0 = dot4(ld_stream(Pa), xa, c0);
            if (v1) c1 = dot4(ld_stream(Pa + 32), xa, c1);
        }
        __syncwarp();
        put(lane, c0 + rows[lane]);
        if (v1) put(lane + 32, c1 + rows[lane + 32]);
    }
    if (hd.nitem > 1) {
        // Split tile: the last of its items to arrive adds all partials in
        // item order and writes y (no combine launch).  Each lane orders its
        // own partial stores at gpu scope before the warp's arrival; the last
        // warp's lanes fence again before reading the other items' partials
        // through L2.
        __threadfence();
        __syncwarp();
        int last = 0;
        if (lane == 0) last = arrive_acq_rel(io.counters + hd.tile) == hd.nitem - 1;
        last = __shfl_sync(FULL, last, 0);
        if (last) {
            __threadfence();
            const float *Pp = io.partial + hd.part_base;
            for (int i = lane; i < h; i += 32) {
                float sum = 0.f;
                for (int k = 0; k < hd.nitem; ++k) sum += __ldcg(Pp + (int64_t)k * h + i);
                io.y[hd.row0 + i] = sum;
            }
            __syncwarp();
            if (lane == 0) io.counters[hd.tile] = 0;  // ready for the next launch
        }
    }
    if (TIMED) {
        __syncwarp();
        if (lane == 0) a.cycles[item] = (int64_t)(clock64() - t0);
    }
}

// One compact item per warp, in item-table order (largest first); BATCH:
// items of many matrices (a.item_mat, a.mats), a form of its own so that the
// one-matrix kernel keeps its registers.
template <bool TIMED, bool BATCH>
__global__ void __launch_bounds__(WI_WARPS * 32, 32 / WI_WARPS)
spmv_warp_items_kernel(const LaunchArgs a) {
    __shared__ float s_rows[WI_WARPS][SABLE_CW_MAX_ROWS];  // CSR row sums of each warp's item
    __shared__ __align__(16) float s_xw[WI_WARPS][WI_XW];    // x window of each warp's item
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * WI_WARPS + w;
    if (item >= a.n_items) return;  // the whole warp leaves; no CTA barrier follows
    const ItemRef ref = a.items[item];
    const int mat = BATCH ? a.item_mat[item] : 0;   // a batch's matrix (loaded beside the item)
    if (lane == 0) prefetch_record(a.records + ref.off, ref.bytes);
    warp_item<TIMED, BATCH>(a, item, ref.off, ref.bytes, lane, s_rows[w], s_xw[w], mat);
}

// dst[0, n) = src[0, n) (either side may be mapped host memory): 16-byte
// loads and stores when both are 16-byte aligned, grid-stride.
__global__ void __launch_bounds__(256)
copy_floats_kernel(float *__restrict__ dst, const float *__restrict__ src, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if ((((uintptr_t)dst | (uintptr_t)src) & 15) == 0) {
        const int64_t n4 = n / 4;
        for (int64_t k = i; k < n4; k += stride)
            reinterpret_cast<float4 *>(dst)[k] = reinterpret_cast<const float4 *>(src)[k];
        done = 4 * n4;
    }
    for (int64_t k = done + i; k < n; k += stride) dst[k] = src[k];
}

__global__ void __launch_bounds__(256)
spmv_combine_kernel(const SplitTile *__restrict__ tiles, int n, const MatIO *mats, const MatIO mat0) {
    const int t = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (t >= n) return;
    const SplitTile T = tiles[t];
    combine_tile(T, mats ? mats[T.mat] : mat0, threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// Persistent warp workers (one warp per CTA)
// ---------------------------------------------------------------------------
struct WarpSmem {
    unsigned char *slot[SABLE_WSTAGES];
    float *xg[SABLE_WSTAGES];
    float *rowbuf;  // [0, 128) CSR row sums, [128, 160) dense temp
};

__device__ __forceinline__ WarpSmem warp_smem(unsigned char *base, int stage_bytes, int xg_floats) {
    WarpSmem s;
    for (int k = 0; k < SABLE_WSTAGES; ++k) s.slot[k] = base + (size_t)k * stage_bytes;
    float *xg0 = reinterpret_cast<float *>(base + (size_t)SABLE_WSTAGES * stage_bytes);
    for (int k = 0; k < SABLE_WSTAGES; ++k) s.xg[k] = xg0 + (size_t)k * xg_floats;
    s.rowbuf = xg0 + (size_t)SABLE_WSTAGES * xg_floats;
    return s;
}

// Gather (cp.async) every x value of the record: xg[0, 4nq) panel columns,
// xg[4nq, 4nq + ns) CSR entries, by lanes 0-30.  Completion is counted on
// the mbarrier xbar (32 arrivals per phase): each gathering lane arrives when
// its own copies land (cp.async.mbarrier.arrive.noinc), the control lane,
// which copies nothing, arrives at once.  Lanes that wait on xbar then see
// every gathered value.
__device__ __forceinline__ void warp_gather(const unsigned char *R, const float *__restrict__ x, float *xg, int lane,
                                            unsigned xbar) {
    if (lane == WCTRL) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(xbar) : "memory");
        return;
    }
    const ItemHeader *hd = reinterpret_cast<const ItemHeader *>(R);
    const int nc = 4 * hd->nq, ns = hd->ns;
    const int *xc = reinterpret_cast<const int *>(R + hd->xcol_off);
    const uint2 *E = reinterpret_cast<const uint2 *>(R + hd->csr_off);
    for (int k = lane; k < nc; k += 31) cp_async4(xg + k, x + xc[k]);
    for (int k = lane; k < ns; k += 31) cp_async4(xg + nc + k, x + E[k].y);
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" :: "r"(xbar) : "memory");
}

__global__ void __launch_bounds__(32)
spmv_warp_kernel(const LaunchArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) unsigned long long s_bar[SABLE_WSTAGES];   // records (TMA)
    __shared__ __align__(8) unsigned long long s_xbar[SABLE_WSTAGES];  // x gathers (cp.async)
    const int lane = threadIdx.x;
    const int ib = a.cta_begin[blockIdx.x], ie = a.cta_begin[blockIdx.x + 1];
    const int n = ie - ib;
    if (n <= 0) return;
    const WarpSmem S = warp_smem(smem, a.stage_bytes, a.xg_floats);
    auto bar_of = [&](int it) { return smem_addr(&s_bar[it % SABLE_WSTAGES]); };
    auto xbar_of = [&](int it) { return smem_addr(&s_xbar[it % SABLE_WSTAGES]); };
    auto parity_of = [&](int it) { return (unsigned)(it / SABLE_WSTAGES) & 1u; };
    if (lane == WCTRL) {
        for (int k = 0; k < SABLE_WSTAGES; ++k) {
            mbar_init(smem_addr(&s_bar[k]));
            mbar_init_count(smem_addr(&s_xbar[k]), 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = lane; i < ROWBUF_FLOATS; i += 32) S.rowbuf[i] = 0.f;
    __syncwarp();
    // record requests: items 0 .. WSTAGES-1 now, item it+WSTAGES after item it
    if (lane == WCTRL)
        for (int k = 0; k < SABLE_WSTAGES && k < n; ++k) {
            const WorkRef r = a.work[ib + k];
            tma_record(bar_of(k), S.slot[k], a.records + r.off, (unsigned)r.bytes);
        }
    WorkRef ahead;  // control lane: entry of the next record to request
    if (lane == WCTRL && SABLE_WSTAGES < n) ahead = a.work[ib + SABLE_WSTAGES];
    // On a wait that runs out: flag it, wait (bounded) for the record copies
    // issued and not yet consumed (items [from, upto)) and for this lane's
    // gathers, and leave.
    auto bail = [&](int from, int upto) {
        if (lane == WCTRL) {
            atomicExch(a.error, 1);
            for (int j = from; j < n && j < upto; ++j) mbar_wait(bar_of(j), parity_of(j));
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncwarp();
    };
    // Every lane waits for the record itself (one instruction for the warp)
    // and checks its header against the worker list entry: a disagreeing
    // record is never used.
    auto arrived = [&](int it, int expect_bytes) {
        const bool good = mbar_wait(bar_of(it), parity_of(it)) &&
                          reinterpret_cast<const ItemHeader *>(S.slot[it % SABLE_WSTAGES])->bytes == expect_bytes;
        return __all_sync(FULL, good);
    };
    WorkRef cur = a.work[ib];
    if (!arrived(0, cur.bytes)) { bail(0, SABLE_WSTAGES); return; }
    warp_gather(S.slot[0], mat_of(a, reinterpret_cast<const ItemHeader *>(S.slot[0])->mat).x, S.xg[0], lane,
                xbar_of(0));
    float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
    for (int it = 0; it < n; ++it) {
        const int sl = it % SABLE_WSTAGES;
        const unsigned char *R = S.slot[sl];
        WorkRef nxt;
        if (it + 1 < n) {
            nxt = a.work[ib + it + 1];
            // requested so far: items up to it + 1 (item it + 2 follows item it)
            if (!arrived(it + 1, nxt.bytes)) { bail(it + 1, it + 2); return; }
            const unsigned char *Rn = S.slot[(it + 1) % SABLE_WSTAGES];
            warp_gather(Rn, mat_of(a, reinterpret_cast<const ItemHeader *>(Rn)->mat).x, S.xg[(it + 1) % SABLE_WSTAGES],
                        lane, xbar_of(it + 1));
        }
        // x values of item it (gathered during the previous item)
        if (!__all_sync(FULL, mbar_wait(xbar_of(it), parity_of(it)))) { bail(it + 1, it + 2); return; }
        const ItemHeader hd = *reinterpret_cast<const ItemHeader *>(R);
        const float *xg = S.xg[sl];
        const int h = hd.h, nq = hd.nq, ns = hd.ns;
        if (cur.flags & SABLE_PART_FIRST) acc0 = acc1 = acc2 = acc3 = 0.f;
        // dense panel: lanes own rows
        const float4 *P = reinterpret_cast<const float4 *>(R + hd.panel_off);
        const float4 *xg4 = reinterpret_cast<const float4 *>(xg);
        if (h <= 32) {
            const int qpw = 32 / h;
            if (lane < qpw * h) {
                const int r = lane % h;
                int q = lane / h;
                for (; q + 3 * qpw < nq; q += 4 * qpw) {
                    const float4 p0 = P[q * h + r], p1 = P[(q + qpw) * h + r];
                    const float4 p2 = P[(q + 2 * qpw) * h + r], p3 = P[(q + 3 * qpw) * h + r];
                    acc0 = dot4(p0, xg4[q], acc0);
                    acc1 = dot4(p1, xg4[q + qpw], acc1);
                    acc2 = dot4(p2, xg4[q + 2 * qpw], acc2);
                    acc3 = dot4(p3, xg4[q + 3 * qpw], acc3);
                }
                for (; q < nq; q += qpw) acc0 = dot4(P[q * h + r], xg4[q], acc0);
            }
        } else {
            const bool v1 = lane + 32 < h, v2 = lane + 64 < h, v3 = lane + 96 < h;
            for (int q = 0; q < nq; ++q) {
                const float4 xv = xg4[q];
                const float4 *Pq = P + q * h + lane;
                acc0 = dot4(Pq[0], xv, acc0);
                if (v1) acc1 = dot4(Pq[32], xv, acc1);
                if (v2) acc2 = dot4(Pq[64], xv, acc2);
                if (v3) acc3 = dot4(Pq[96], xv, acc3);
            }
        }
        // CSR entries into the row buffer
        if (ns > 0) {
            const int *rp = reinterpret_cast<const int *>(R + hd.rp_off);
            const uint2 *E = reinterpret_cast<const uint2 *>(R + hd.csr_off);
            const float *xe = xg + 4 * nq;
            csr_rows(rp, E, h, hd.g, 0, ns, lane, S.rowbuf, [&](int i, unsigned) { return xe[i]; });
        }
        __syncwarp();
        // the slot is free: request the record two items ahead
        if (lane == WCTRL && it + SABLE_WSTAGES < n) {
            tma_record(bar_of(it), S.slot[sl], a.records + ahead.off, (unsigned)ahead.bytes);
            if (it + SABLE_WSTAGES + 1 < n) ahead = a.work[ib + it + SABLE_WSTAGES + 1];
        }
        if (cur.flags & SABLE_PART_LAST) {
            const MatIO &io = mat_of(a, hd.mat);
            float *tmp = S.rowbuf + SABLE_MAX_ROW_TILE;
            float tot[4] = {0.f, 0.f, 0.f, 0.f};
            int nrow = 0;
            if (h <= 32) {
                const int qpw = 32 / h;
                tmp[lane] = lane < qpw * h ? (acc0 + acc1) + (acc2 + acc3) : 0.f;
                __syncwarp();
                if (lane < h) {
                    float sd = 0.f;
                    for (int s2 = 0; s2 < qpw; ++s2) sd += tmp[s2 * h + lane];
                    tot[0] = sd + S.rowbuf[lane];
                    nrow = 1;
                }
            } else {
                tot[0] = acc0 + S.rowbuf[lane];
                tot[1] = acc1 + S.rowbuf[lane + 32];
                tot[2] = acc2 + S.rowbuf[lane + 64];
                tot[3] = acc3 + S.rowbuf[lane + 96];
                nrow = 4;
            }
            if (cur.nparts == 1) {
                for (int k = 0; k < nrow; ++k)
                    if (lane + 32 * k < h) io.y[hd.row0 + lane + 32 * k] = tot[k];
            } else {
                float *pp = io.ppartial + cur.part_base;
                for (int k = 0; k < nrow; ++k)
                    if (lane + 32 * k < h) pp[(int64_t)cur.part * h + lane + 32 * k] = tot[k];
                // every lane makes its own partial sums visible at device scope
                // before the control lane counts the part as arrived
                __threadfence();
                __syncwarp();
                int last = 0;
                if (lane == WCTRL) last = arrive_acq_rel(io.pcounters + cur.split) == cur.nparts - 1;
                last = __shfl_sync(FULL, last, WCTRL);
                __syncwarp();
                if (last) {
                    __threadfence();
                    for (int i = lane; i < h; i += 32) {
                        float s = 0.f;
                        for (int k = 0; k < cur.nparts; ++k) s += __ldcg(pp + (int64_t)k * h + i);
                        io.y[hd.row0 + i] = s;
                    }
                    if (lane == WCTRL) io.pcounters[cur.split] = 0;  // ready for the next launch
                }
            }
            __syncwarp();
            for (int i = lane; i < ROWBUF_FLOATS; i += 32) S.rowbuf[i] = 0.f;
            __syncwarp();
        }
        cur = nxt;
    }
}

}  // namespace

namespace sable {

int spmv_items_smem(int stage_bytes, int xg_floats) {
    (void)xg_floats;
    return STAGE_OFF + stage_bytes;
}

int spmv_warp_smem(int stage_bytes, int xg_floats) {
    return SABLE_WSTAGES * stage_bytes + SABLE_WSTAGES * 4 * xg_floats + 4 * ROWBUF_FLOATS;
}

// Warp workers of the persistent SpMV per SM; 1 when the records are too
// large for its ring (the plan then runs one CTA per item).  That refusal is
// expected, so its error is taken off the runtime's last-error state, where
// the next launch check would otherwise report it.
int spmv_warp_workers_per_sm(int stage_bytes, int xg_floats) {
    const int smem = spmv_warp_smem(stage_bytes, (xg_floats + 3) & ~3);
    if (cudaFuncSetAttribute(spmv_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, spmv_warp_kernel, 32, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

int launch_spmv_items(const LaunchArgs &a, bool timed, void *stream) {
    if (a.n_items <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int smem = spmv_items_smem(a.stage_bytes, a.xg_floats);
    if (timed) {
        cudaFuncSetAttribute(spmv_items_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        spmv_items_kernel<true><<<a.n_items, SABLE_THREADS, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(spmv_items_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        spmv_items_kernel<false><<<a.n_items, SABLE_THREADS, smem, s>>>(a);
    }
    return (int)cudaGetLastError();
}

int launch_spmv_warp_items(const LaunchArgs &a, bool timed, void *stream) {
    if (a.n_items <= 0) return 0;
    const unsigned grid = (a.n_items + WI_WARPS - 1) / WI_WARPS;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (a.item_mat && a.mats) spmv_warp_items_kernel<false, true><<<grid, WI_WARPS * 32, 0, s>>>(a);
    else if (timed) spmv_warp_items_kernel<true, false><<<grid, WI_WARPS * 32, 0, s>>>(a);
    else spmv_warp_items_kernel<false, false><<<grid, WI_WARPS * 32, 0, s>>>(a);
    return (int)cudaGetLastError();
}

int launch_copy_floats(float *dst, const float *src, int64_t n, void *stream) {
    if (n <= 0) return 0;
    const int64_t blocks = std::min<int64_t>((n / 4 + 255) / 256 + 1, 1024);
    copy_floats_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(dst, src, n);
    return (int)cudaGetLastError();
}

int launch_spmv_combine(const SplitTile *tiles, int n_tiles, const MatIO *mats, const MatIO &mat0, void *stream) {
    if (n_tiles <= 0) return 0;
    spmv_combine_kernel<<<(n_tiles + 7) / 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(tiles, n_tiles, mats, mat0);
    return (int)cudaGetLastError();
}

int launch_spmv_warps(const LaunchArgs &a, int n_workers, void *stream) {
    if (a.n_items <= 0 || n_workers <= 0) return 0;
    const int smem = spmv_warp_smem(a.stage_bytes, a.xg_floats);
    cudaFuncSetAttribute(spmv_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    spmv_warp_kernel<<<n_workers, 32, smem, static_cast<cudaStream_t>(stream)>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace sable
