// VBR SpMV kernels for sm_103a over item records (layout in sable_internal.h).
//
// Replaces the per-block call sequence of the generated executor
// (src/codegen.py:414-439: MKL CSR product with beta = 0, then one
// spmv_kernel call per dense block, src/codegen.py:263-291).
//
//   spmv_items_kernel  one CTA (8 warps) per item: a single TMA bulk copy
//                      (cp.async.bulk, completion counted on an mbarrier)
//                      brings the item's record into shared memory; x values
//                      are read through L1.  Split tiles are combined by the
//                      last-arriving CTA.  This is the plain form and the one
//                      the timed entry points use.
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
#include <cuda_runtime.h>
#include <stdint.h>
#include "sable_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NWARP = SABLE_NWARP;
constexpr int RED_FLOATS = NWARP * SABLE_MAX_ROW_TILE;    // dense partials (CTA kernel)
constexpr int STAGE_OFF = 2 * RED_FLOATS * 4;             // + CSR partials, bytes
constexpr unsigned long long WAIT_NS = 2000000000ull;
constexpr int CTRL = SABLE_THREADS - 1;                    // control thread (CTA kernel)
constexpr int WCTRL = 31;                                  // control lane (warp kernel)
constexpr int ROWBUF_FLOATS = SABLE_MAX_ROW_TILE + 32;     // warp kernel: CSR row sums + dense temp

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
}

// Wait for phase `parity` of an mbarrier, giving up after WAIT_NS.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    unsigned done = 0;
    const unsigned long long t0 = global_ns();
    while (true) {
        asm volatile(
            "{\n .reg .pred p;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(bar), "r"(parity), "r"(1000000u) : "memory");
        if (done) return true;
        if (global_ns() - t0 > WAIT_NS) return false;
    }
}

// Release-acquire arrival on a split-tile counter (one thread, after the
// partial-sum stores of its CTA / warp are ordered before it).
__device__ __forceinline__ int arrive_acq_rel(int *cnt) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(cnt) : "memory");
    return old;
}

// One thread: expect `bytes` on `bar` and copy the record into `dst`.
__device__ __forceinline__ void tma_record(unsigned bar, void *dst, const unsigned char *src, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ void cp_async4(void *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory"); }

__device__ __forceinline__ float dot4(const float4 a, const float4 b, float acc) {
    acc = fmaf(a.x, b.x, acc);
    acc = fmaf(a.y, b.y, acc);
    acc = fmaf(a.z, b.z, acc);
    acc = fmaf(a.w, b.w, acc);
    return acc;
}

__device__ __forceinline__ float4 xquad(const int4 *xc, int q, const float *__restrict__ x) {
    const int4 c = xc[q];
    return make_float4(__ldg(x + c.x), __ldg(x + c.y), __ldg(x + c.z), __ldg(x + c.w));
}

__device__ __forceinline__ const MatIO &mat_of(const LaunchArgs &a, int mat) { return a.mats ? a.mats[mat] : a.mat0; }

// ---------------------------------------------------------------------------
// CSR rows of one item with groups of g lanes per row: adds each row's sum
// into rowsum[row] (one writer per row).  Rows [r_lo, h), entries clipped
// to [e_lo, e_hi).  xv(i, col) gives the x value of entry i.
// ---------------------------------------------------------------------------
template <class XV>
__device__ __forceinline__ void csr_rows(const int *rp, const uint2 *E, int h, int g, int e_lo, int e_hi, int lane,
                                         float *rowsum, XV xv) {
    if (e_lo >= e_hi) return;
    const int gpw = 32 / g, sg = lane / g, sl = lane % g;
    int lo = 0, hi = h - 1;  // first row with entries at or after e_lo
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (rp[mid + 1] > e_lo) hi = mid; else lo = mid + 1;
    }
    for (int r0 = lo; r0 < h && rp[r0] < e_hi; r0 += gpw) {
        const int r = r0 + sg;
        int b = e_hi, e = e_hi;
        if (r < h) {
            b = max(rp[r], e_lo);
            e = min(rp[r + 1], e_hi);
        }
        const int nsteps = __reduce_max_sync(FULL, e > b ? (e - b + 2 * g - 1) / (2 * g) : 0);
        float s = 0.f;
        for (int k = 0; k < nsteps; ++k) {
            const int i0 = b + 2 * k * g + sl, i1 = i0 + g;
            if (i0 < e) {
                const uint2 u = E[i0];
                s = fmaf(__uint_as_float(u.x), xv(i0, u.y), s);
            }
            if (i1 < e) {
                const uint2 u = E[i1];
                s = fmaf(__uint_as_float(u.x), xv(i1, u.y), s);
            }
        }
        for (int o = g >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (sl == 0 && r < h && e > b) rowsum[r] += s;
    }
}

// ---------------------------------------------------------------------------
// CTA-per-item kernel
// ---------------------------------------------------------------------------
// x values of an item come either from x through L1 (XG == nullptr) or from
// the item's gathered copy in shared memory: xg[0, 4nq) for the panel
// columns, xg[4nq, 4nq + ns) for the CSR entries.
__device__ __forceinline__ void cta_accumulate(const unsigned char *R, const ItemHeader &hd, const float *__restrict__ x,
                                               const float *xg, float *red, float *ysw) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int h = hd.h, nq = hd.nq, ns = hd.ns;
    const int4 *xc = reinterpret_cast<const int4 *>(R + hd.xcol_off);
    const float4 *P = reinterpret_cast<const float4 *>(R + hd.panel_off);
    const float4 *xg4 = reinterpret_cast<const float4 *>(xg);
    auto xq = [&](int q) { return xg ? xg4[q] : xquad(xc, q, x); };
    if (h <= 32) {
        const int qpw = 32 / h;
        const bool act = lane < qpw * h;
        const int r = lane % h, s = lane / h;
        float acc = 0.f, accb = 0.f;
        if (nq > 0 && act) {
            const int step = NWARP * qpw;
            int q = warp * qpw + s;
            for (; q + step < nq; q += 2 * step) {
                const float4 x0 = xq(q), x1 = xq(q + step);
                acc = dot4(P[q * h + r], x0, acc);
                accb = dot4(P[(q + step) * h + r], x1, accb);
            }
            if (q < nq) acc = dot4(P[q * h + r], xq(q), acc);
        }
        red[warp * SABLE_MAX_ROW_TILE + lane] = act ? acc + accb : 0.f;
    } else {
        float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
        const bool v1 = lane + 32 < h, v2 = lane + 64 < h, v3 = lane + 96 < h;
        for (int q = warp; q < nq; q += NWARP) {
            const float4 xa = xq(q);
            const float4 *Pa = P + q * h + lane;
            acc0 = dot4(Pa[0], xa, acc0);
            if (v1) acc1 = dot4(Pa[32], xa, acc1);
            if (v2) acc2 = dot4(Pa[64], xa, acc2);
            if (v3) acc3 = dot4(Pa[96], xa, acc3);
        }
        float *rw = red + warp * SABLE_MAX_ROW_TILE;
        rw[lane] = acc0;
        if (v1) rw[lane + 32] = acc1;
        if (v2) rw[lane + 64] = acc2;
        if (v3) rw[lane + 96] = acc3;
    }
    if (ns > 0) {
        const int *rp = reinterpret_cast<const int *>(R + hd.rp_off);
        const uint2 *E = reinterpret_cast<const uint2 *>(R + hd.csr_off);
        const int e_lo = (int)(((int64_t)ns * warp) / NWARP), e_hi = (int)(((int64_t)ns * (warp + 1)) / NWARP);
        const float *xe = xg ? xg + 4 * nq : nullptr;
        csr_rows(rp, E, h, hd.g, e_lo, e_hi, lane, ysw + warp * SABLE_MAX_ROW_TILE,
                 [&](int i, unsigned col) { return xe ? xe[i] : __ldg(x + col); });
    }
}

// Row sums in a fixed order, output, split-tile reduction; leaves ysw zero.
__device__ __forceinline__ void cta_finish(const ItemHeader &hd, const MatIO &io, float *red, float *ysw, int *s_last) {
    const int tid = threadIdx.x;
    const int h = hd.h;
    const bool split = hd.nitem > 1;
    if (tid < h) {
        const int i = tid;
        float sd = 0.f;
        if (h <= 32) {
            const int qpw = 32 / h;
#pragma unroll
            for (int w = 0; w < NWARP; ++w)
                for (int s2 = 0; s2 < qpw; ++s2) sd += red[w * SABLE_MAX_ROW_TILE + s2 * h + i];
        } else {
#pragma unroll
            for (int w = 0; w < NWARP; ++w) sd += red[w * SABLE_MAX_ROW_TILE + i];
        }
        float sp = 0.f;
#pragma unroll
        for (int w = 0; w < NWARP; ++w) {
            sp += ysw[w * SABLE_MAX_ROW_TILE + i];
            ysw[w * SABLE_MAX_ROW_TILE + i] = 0.f;
        }
        const float tot = sd + sp;
        if (!split) io.y[hd.row0 + i] = tot;
        else io.partial[hd.part_base + (int64_t)hd.kidx * h + i] = tot;
    }
    if (split) {
        if (tid < h) __threadfence();  // this CTA's partial sums, visible at device scope
        __syncthreads();
        if (tid == CTRL) *s_last = (arrive_acq_rel(io.counters + hd.tile) == hd.nitem - 1);
        __syncthreads();
        if (*s_last) {
            for (int i = tid; i < h; i += SABLE_THREADS) {
                float s = 0.f;
                for (int k = 0; k < hd.nitem; ++k) s += __ldcg(io.partial + hd.part_base + (int64_t)k * h + i);
                io.y[hd.row0 + i] = s;
            }
            if (tid == CTRL) io.counters[hd.tile] = 0;  // ready for the next launch
        }
    }
}

template <bool TIMED>
__global__ void __launch_bounds__(SABLE_THREADS)
spmv_items_kernel(const LaunchArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    float *red = reinterpret_cast<float *>(smem);
    float *ysw = red + RED_FLOATS;
    unsigned char *stage = smem + STAGE_OFF;
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ int s_last;
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
    cta_finish(hd, io, red, ysw, &s_last);
    if (TIMED) {
        __syncthreads();
        if (tid == 0) a.cycles[blockIdx.x] = (int64_t)(clock64() - t0);
    }
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

__device__ __forceinline__ void mbar_init_count(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
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

int spmv_warp_workers_per_sm(int stage_bytes, int xg_floats) {
    const int smem = spmv_warp_smem(stage_bytes, (xg_floats + 3) & ~3);
    if (cudaFuncSetAttribute(spmv_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return 1;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, spmv_warp_kernel, 32, smem) != cudaSuccess) return 1;
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

int launch_spmv_warps(const LaunchArgs &a, int n_workers, void *stream) {
    if (a.n_items <= 0 || n_workers <= 0) return 0;
    const int smem = spmv_warp_smem(a.stage_bytes, a.xg_floats);
    cudaFuncSetAttribute(spmv_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    spmv_warp_kernel<<<n_workers, 32, smem, static_cast<cudaStream_t>(stream)>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace sable
