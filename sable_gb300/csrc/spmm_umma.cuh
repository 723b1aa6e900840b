// Split-BF16 SpMM of one (item record, N-slice) unit on the tcgen05 tensor
// cores, by one CTA of UMMA_THREADS threads: SABLE_THREADS producer threads
// (warps 0-7) and one issuer warp (warp 8) whose lane 0 alone starts the bulk
// copies and issues the MMAs, so that the producers never wait on that
// serial work.  Replaces the dense-block part
// of gen_single_threaded_spmm (src/codegen.py:827-937; spmm_kernel, :851-859)
// for plans built with spmm_tc and N >= 32; the CSR entries of the item stay
// FP32 on the CUDA cores (spmm_tile_finish).
//
// The product is computed transposed, so that the SpMM width fills the
// 128-row MMA:   D[m][n] = sum_k X[col(k)][n0 + m] * A[row0 + n][col(k)]
//   m  column of Y within the N-slice (M = 128 TMEM lanes; lanes >= NT unused)
//   n  row of the item's tile (the MMA's N = h rounded up to 16, <= 128)
//   k  panel column of the item (K steps of 16; col(k) = the record's xcol)
// Both operands are split into BF16 terms by repeated round-to-nearest (see
// spmm_item.cuh), and TERMS = 3 (six products) or 2 (three products) term
// products accumulate in FP32 in TMEM.
//
// Per K step ks (16 panel columns):
//   B operand  the tile's panel terms, split once on the host when the plan
//              is built, in the UMMA K-major layout (umma.cuh): per step 3
//              blocks of hp x 32 bytes (hp = h rounded up to 16); one bulk
//              copy (cp.async.bulk, mbarrier completion) brings TERMS of them
//              into a ring of bst stages, bst - 2 steps ahead of the MMAs
//              (the launch sizes the ring for 4..12 stages of its tallest
//              tile beside three CTAs per SM; an item with shorter tiles fits
//              more of its own stages in the same bytes, up to 12).
//   A operand  the 16 X rows of the step (NT floats each, from L2), loaded
//              two steps ahead into registers with 16-byte loads (their row
//              indices four steps ahead, so no load waits on another), split
//              into TERMS BF16 terms by the producer warps and stored in the
//              MN-major layout (8-byte stores, conflict-free) into a ring of
//              UMMA_NA stages; each warp then fences its stores to the async
//              proxy and arrives on the stage's "X ready" mbarrier.
//   MMA        the issuer waits for the stage's "X ready" barrier and the
//              step's panel copy, issues the products (tcgen05.mma.cta_group::1
//              .kind::f16, M = 128, N = hp, K = 16; for split3 tiles of at
//              most 64 rows four MMAs, two of them with N = 2 hp over two
//              panel terms at once into two accumulator ranges) and commits
//              them to the stage's "done" mbarrier; the producers wait on it
//              before they reuse the X stage, the issuer two steps later
//              before it reuses the panel stage.  No CTA-wide barrier inside
//              the K loop.
// After the last step the accumulator is read with tcgen05.ld into the Y
// tile in shared memory (lane m, column n -> Y[n][m]; with two ranges, their
// sum); TMEM is freed on every
// path.  Every wait is bounded (WAIT_NS); on expiry the error flag is set, the
// CTA stops issuing work, waits (bounded) for what it issued and frees TMEM.
#pragma once
#include "spmm_item.cuh"
#include "umma.cuh"

namespace {

constexpr int UMMA_BST_MIN = 4, UMMA_BST_MAX = 12;  // panel-term stages (bulk-copy ring)
// X-term stages: the producers run up to NA - 1 steps ahead of the MMAs.
// Two: a third stage takes the shared memory of two panel stages at three
// CTAs per SM, and the shorter panel-copy lookahead lost more than the
// producers gained (50000^2, N = 128: 0.1247 ms with two, 0.1280 with three,
// 0.1471 with four).
constexpr int UMMA_NA = 2;
constexpr int UMMA_M = 128;                 // MMA rows (TMEM lanes)
constexpr int UMMA_THREADS = SABLE_THREADS + 32;   // producers + the issuer warp
// Dynamic shared memory of one CTA when three CTAs share an SM (228 KB less
// the per-CTA reserve and static shared memory).
constexpr int UMMA_SMEM_BUDGET = 75776;

// A bounded mbarrier wait that first tests the phase without blocking, so
// that a phase already complete costs no clock read.
__device__ __forceinline__ bool umma_wait(unsigned bar, unsigned parity) {
    unsigned done;
    asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    return done != 0 || mbar_wait(bar, parity);
}

// Shared memory of a CTA: UMMA_NA stages of X terms, bst stages of panel
// terms of bstage bytes, then the CSR row starts; the Y tile reuses the stage
// space.
template <int NT, int TERMS>
struct UmmaSmem {
    static constexpr int A_STAGE = TERMS * UMMA_M * 32;       // X terms of one step (MN-major, 128 rows)
    static constexpr int OFF_A = 0;                           // UMMA_NA stages
    static constexpr int OFF_B = OFF_A + UMMA_NA * A_STAGE;   // bst stages
    static constexpr int YS = SABLE_MAX_ROW_TILE * NT * 4;    // Y tile (after the K loop, over the stages)
    static constexpr int RST = (SABLE_MAX_ROW_TILE + 8) * 4;
    __host__ __device__ static constexpr int off_rst(int bst, int bstage) {
        return YS > OFF_B + bst * bstage ? YS : OFF_B + bst * bstage;
    }
    __host__ __device__ static constexpr int total(int bst, int bstage) { return off_rst(bst, bstage) + RST; }
};

// Split four FP32 values into TERMS BF16 terms; t[k] packs the four k-th
// terms (first value in the low half of t[k].x).  One packed conversion per
// pair of values (round to nearest, as the scalar conversion rounds).
template <int TERMS>
__device__ __forceinline__ void split4(const float4 v, uint2 (&t)[TERMS]) {
    float r0 = v.x, r1 = v.y, r2 = v.z, r3 = v.w;
#pragma unroll
    for (int k = 0; k < TERMS; ++k) {
        const __nv_bfloat162 p01 = __floats2bfloat162_rn(r0, r1), p23 = __floats2bfloat162_rn(r2, r3);
        t[k] = make_uint2(*reinterpret_cast<const uint32_t *>(&p01), *reinterpret_cast<const uint32_t *>(&p23));
        r0 -= __low2float(p01);
        r1 -= __high2float(p01);
        r2 -= __low2float(p23);
        r3 -= __high2float(p23);
    }
}

// Read-only global loads whose issue point the compiler keeps (asm volatile):
// the K loop loads X two steps and its row indices four steps before use,
// and a load moved down to its use would wait out the memory latency.
__device__ __forceinline__ float4 ld_pinned_f4(const float *p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ int ld_pinned_s32(const int *p) {
    int v;
    asm volatile("ld.global.nc.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// Unit u of a step's X gather (4 NT units of one float4): lane bits pick
// (k & 7) and the low bits of the M quad so that a warp's 8-byte term stores
// cover 256 contiguous bytes of the MN-major block (no bank conflicts).  The
// units of one thread (u = tid + 256 i) share k.
__device__ __forceinline__ void umma_unit(int u, int &k, int &q) {
    k = ((u >> 1) & 7) | (((u >> 5) & 1) << 3);
    q = (u & 1) | (((u >> 4) & 1) << 1) | ((u >> 6) << 2);
}

// planes: the item's panel terms (3 term blocks of hp x 32 bytes per step);
// ring_bst / ring_bstage: the launch's panel ring (stages of its tallest
// tile, bytes per stage >= TERMS hp 32).
template <int NT, int TERMS>
__device__ __forceinline__ void spmm_umma_item(const unsigned char *R, const MatIO &a, int slice, int64_t part_stride,
                                               unsigned char *smem, const unsigned char *planes, int *error,
                                               int ring_bst, int ring_bstage) {
    using L = UmmaSmem<NT, TERMS>;
    constexpr int UNITS = 4 * NT;                                    // float4 loads per step
    constexpr int UPT = (UNITS + SABLE_THREADS - 1) / SABLE_THREADS; // per thread
    constexpr int NPROD = TERMS == 3 ? 6 : 3;
    __shared__ __align__(8) uint64_t s_full[UMMA_BST_MAX];   // panel copy of a stage landed
    __shared__ __align__(8) uint64_t s_afull[UMMA_NA];   // X terms of stage ks % NA written (8 warp arrivals)
    __shared__ __align__(8) uint64_t s_done[UMMA_NA];    // products of the step of stage ks % NA completed
    __shared__ uint32_t s_taddr;
    __shared__ int s_stop;        // a bounded wait ran out: every loop stops at its next check
    __shared__ int s_committed;   // steps whose products the issuer committed

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool prod = tid < SABLE_THREADS;          // producer threads
    const bool issuer = tid == SABLE_THREADS;       // lane 0 of warp 8
    const ItemHeader c = *reinterpret_cast<const ItemHeader *>(R);
    const int h = c.h, nq = c.nq, ncol = 4 * nq;
    const int n0 = slice * NT;
    float *ys = reinterpret_cast<float *>(smem);
    float4 *ys4 = reinterpret_cast<float4 *>(smem);
    int *rst = reinterpret_cast<int *>(smem + L::off_rst(ring_bst, ring_bstage));

    if (nq > 0) {
        const int nks = (ncol + 15) >> 4;
        const int hp = (h + 15) & ~15;
        // this item's panel stages in the launch's ring bytes (at most
        // UMMA_BST_MAX): a short tile copies its panel terms further ahead
        const int bstage = TERMS * hp * 32;
        const int bst = min(UMMA_BST_MAX, (ring_bst * ring_bstage) / bstage);
        const int look = bst - 2;    // panel copies run this many steps ahead
        // split3 tiles of at most 64 rows issue their six products as four
        // MMAs: two take the first two panel terms at once (N = 2 hp: the
        // term blocks lie one after another, which is the K-major layout of
        // one operand of 2 hp rows) into two accumulator ranges that the
        // epilogue adds
        const bool stacked = TERMS == 3 && hp <= 64;
        const uint32_t ncols = umma_tmem_cols(stacked ? 2 * hp : hp);
        const uint32_t step_src = 3u * (uint32_t)hp * 32u;           // bytes of a step in `planes`
        const uint32_t copy_bytes = (uint32_t)TERMS * (uint32_t)hp * 32u;
        const uint32_t a_base = smem_addr(smem + L::OFF_A), b_base = smem_addr(smem + L::OFF_B);
        const uint32_t idesc = umma_idesc_bf16(UMMA_M, hp, true), idesc2 = umma_idesc_bf16(UMMA_M, 2 * hp, true);
        const int *colmap = reinterpret_cast<const int *>(R + c.xcol_off);
        const float *__restrict__ X = a.x;
        const int64_t ldx = a.ldx;
        // this thread's panel column within a step, and its X row at step j (-1: none)
        int k0, q0;
        umma_unit(tid, k0, q0);
        const bool has_col = prod && tid < UNITS;
        const int *colp = colmap + k0;
        auto col_row = [&](int j) -> int {
            return (has_col && 16 * j + k0 < ncol) ? ld_pinned_s32(colp + 16 * j) : -1;
        };
        // this thread's X units, fixed for the item: the N-slice column of
        // unit i (-1: past N or no unit) and the byte offset of its terms in
        // an X stage (-1: no unit)
        int ucol[UPT], uoff[UPT];
#pragma unroll
        for (int i = 0; i < UPT; ++i) {
            const int u = tid + i * SABLE_THREADS;
            int k, q;
            umma_unit(u, k, q);
            const bool has = prod && u < UNITS;
            ucol[i] = has && n0 + 4 * q < a.N ? n0 + 4 * q : -1;
            uoff[i] = has ? umma_mnmajor_off(4 * q, k) : -1;
        }
        auto load_step = [&](int row, float4 (&dst)[UPT]) {
#pragma unroll
            for (int i = 0; i < UPT; ++i) {
                dst[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (row >= 0 && ucol[i] >= 0) dst[i] = ld_pinned_f4(X + (int64_t)row * ldx + ucol[i]);
            }
        };
        // The issuer initialises the barriers and starts the first panel
        // copies, and the producers load the X rows of the first two steps,
        // before the CTA barrier that publishes the barriers and the TMEM
        // address, so that those latencies overlap the TMEM allocation.
        float4 xr0[UPT], xr1[UPT];   // X values of the next even / odd step
        int cm0 = -1, cm1 = -1;
        if (issuer) {
            for (int s = 0; s < bst; ++s) mbar_init(smem_addr(&s_full[s]));
            for (int s = 0; s < UMMA_NA; ++s) {
                mbar_init(smem_addr(&s_done[s]));
                mbar_init_count(smem_addr(&s_afull[s]), SABLE_THREADS / 32);
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            s_stop = 0;
            s_committed = 0;
            for (int j = 0; j < look && j < nks; ++j)   // panel copies of the first `look` steps
                tma_record(smem_addr(&s_full[j]), smem + L::OFF_B + j * bstage, planes + (size_t)j * step_src,
                           copy_bytes);
        } else if (prod) {
            load_step(col_row(0), xr0);
            load_step(col_row(1), xr1);
            cm0 = col_row(2);
            cm1 = col_row(3);
        }
        if (warp == 0) tmem_alloc(smem_addr(&s_taddr), ncols);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        const uint32_t taddr = s_taddr;
        // The producer warps and the issuer run decoupled and hand the stages
        // over through mbarriers: a producer warp writes its part of the X
        // terms of step ks into stage ks % NA, fences them to the async proxy
        // and arrives on s_afull[ks % NA] (the eight warps' arrivals complete
        // the phase); the issuer waits for that and for the step's panel copy,
        // issues the products and commits them to s_done[ks % NA], on which
        // the producers wait NA steps later (before they reuse the X stage)
        // and the issuer two steps later (before it reuses the panel stage;
        // step ks - 2's barrier is s_done[(ks - 2) % NA]).  Phases: step ks
        // is phase (ks / NA) & 1 of its stage's barriers.  Neither side waits for the
        // other's issue work, only for the data it needs.  A wait that runs
        // out sets s_stop, which both loops check, so an error ends the item
        // after at most one more bounded wait per thread.
        if (prod) {
            // Step ks: its X values are in `slot` (loaded two steps earlier),
            // which then receives those of step ks + 2, whose row `cm` was read
            // two steps earlier still; `cm` then receives the row of step
            // ks + 4.  false: stop (warp-uniform).
            auto pstep = [&](int ks, float4 (&slot)[UPT], int &cm) -> bool {
                if (ks >= UMMA_NA) {   // the products of step ks - NA have read this X stage
                    const bool ok = umma_wait(smem_addr(&s_done[ks % UMMA_NA]), (uint32_t)(((ks - UMMA_NA) / UMMA_NA) & 1));
                    const bool stop = *reinterpret_cast<volatile int *>(&s_stop) != 0;
                    if (__any_sync(FULL, !ok || stop)) {
                        if (!ok) s_stop = 1;
                        return false;
                    }
                }
                float4 cur[UPT];
#pragma unroll
                for (int i = 0; i < UPT; ++i) cur[i] = slot[i];
                load_step(cm, slot);
                cm = col_row(ks + 4);
                unsigned char *As = smem + L::OFF_A + (ks % UMMA_NA) * L::A_STAGE;
#pragma unroll
                for (int i = 0; i < UPT; ++i) {
                    if (uoff[i] >= 0) {
                        uint2 t[TERMS];
                        split4<TERMS>(cur[i], t);
#pragma unroll
                        for (int e = 0; e < TERMS; ++e) *reinterpret_cast<uint2 *>(As + e * (UMMA_M * 32) + uoff[i]) = t[e];
                    }
                }
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_addr(&s_afull[ks % UMMA_NA]));
                return true;
            };
            for (int ks = 0; ks < nks; ks += 2) {
                if (!pstep(ks, xr0, cm0)) break;
                if (ks + 1 < nks && !pstep(ks + 1, xr1, cm1)) break;
            }
        } else if (issuer) {
            int issued = look < nks ? look : nks, landed = 0, committed = 0;
            // ring positions as counters, so that the loop divides by no
            // runtime ring depth: panel stage s of step ks with its phase
            // parity sph, and stage sj of step ks + look, which the step's
            // copy fills from src
            int s = 0, sj = look;
            uint32_t sph = 0;
            const unsigned char *src = planes + (size_t)look * step_src;
            // descriptors of the stage bases: a stage or term offset adds its
            // count of 16-byte units to the start-address field (shared
            // addresses stay below 256 KB, so the 14-bit field never carries)
            const uint64_t ad0 = umma_sdesc(a_base, UMMA_MN_LBO, UMMA_MN_SBO);
            const uint64_t bd0 = umma_sdesc(b_base, UMMA_KM_LBO, UMMA_KM_SBO);
            const uint32_t bterm16 = (uint32_t)hp * 2u, bstage16 = (uint32_t)bstage >> 4;
            for (int ks = 0; ks < nks; ++ks) {
                if (*reinterpret_cast<volatile int *>(&s_stop)) break;
                // the products of step ks - 2 have read the panel stage that
                // step ks + look takes (waited for only where that step exists)
                if (ks >= 2 && ks + look < nks && !umma_wait(smem_addr(&s_done[(ks - 2) % UMMA_NA]), (uint32_t)(((ks - 2) / UMMA_NA) & 1))) {
                    s_stop = 1;
                    break;
                }
                if (ks + look < nks) {
                    tma_record(smem_addr(&s_full[sj]), smem + L::OFF_B + sj * bstage, src, copy_bytes);
                    issued = ks + look + 1;
                }
                src += step_src;
                sj = sj + 1 == bst ? 0 : sj + 1;
                if (!umma_wait(smem_addr(&s_afull[ks % UMMA_NA]), (uint32_t)((ks / UMMA_NA) & 1))) {
                    s_stop = 1;
                    break;
                }
                if (!umma_wait(smem_addr(&s_full[s]), sph)) {
                    s_stop = 1;
                    break;
                }
                landed = ks + 1;
                tc_fence_after();
                const uint64_t ad_st = ad0 + (uint64_t)((ks % UMMA_NA) * (L::A_STAGE >> 4));
                const uint64_t bd_st = bd0 + (uint64_t)((uint32_t)s * bstage16);
                // products (x term, panel term), smallest first
                constexpr int PA[6] = {1, 0, 2, 0, 1, 0}, PB[6] = {1, 2, 0, 1, 0, 0};
                constexpr int QA[3] = {0, 1, 0}, QB[3] = {1, 0, 0};
                if (stacked) {
                    // x1 [b0 b1] (at step 0 it initialises both ranges), x0 b2
                    // into the first range, x2 b0 into the second, x0 [b0 b1]
                    constexpr uint64_t AT = UMMA_M * 32 / 16;   // one X term block, 16-byte units
                    umma_bf16(taddr, ad_st + AT, bd_st, idesc2, ks > 0 ? 1u : 0u);
                    umma_bf16(taddr, ad_st, bd_st + (uint64_t)(2u * bterm16), idesc, 1u);
                    umma_bf16(taddr + (uint32_t)hp, ad_st + 2 * AT, bd_st, idesc, 1u);
                    umma_bf16(taddr, ad_st, bd_st, idesc2, 1u);
                } else {
#pragma unroll
                    for (int p = 0; p < NPROD; ++p) {
                        const int ta = TERMS == 3 ? PA[p] : QA[p], tb = TERMS == 3 ? PB[p] : QB[p];
                        const uint64_t ad = ad_st + (uint64_t)(ta * (UMMA_M * 32 / 16));
                        const uint64_t bd = bd_st + (uint64_t)((uint32_t)tb * bterm16);
                        umma_bf16(taddr, ad, bd, idesc, (ks > 0 || p > 0) ? 1u : 0u);
                    }
                }
                umma_commit(smem_addr(&s_done[ks % UMMA_NA]));
                committed = ks + 1;
                if (++s == bst) {
                    s = 0;
                    sph ^= 1u;
                }
            }
            // every panel copy issued has landed before the CTA exits
            for (int j = landed; j < issued; ++j)
                if (!umma_wait(smem_addr(&s_full[j % bst]), (uint32_t)((j / bst) & 1))) s_stop = 1;
            s_committed = committed;
        }
        __syncthreads();
        const int committed = s_committed;
        // Every product issued has completed before TMEM is read or freed:
        // a commit tracks the MMAs issued since the previous commit, and the
        // MMAs of one accumulator complete in issue order, so the last step's
        // commit covers them all.
        if (committed > 0) {
            const int last = committed - 1;
            if (!umma_wait(smem_addr(&s_done[last % UMMA_NA]), (uint32_t)((last / UMMA_NA) & 1))) s_stop = 1;
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (s_stop || committed < nks) {
            if (tid == 0) atomicExch(error, 1);
        } else {
            // lane m of quadrant (warp & 3) -> Y column n0 + m; the two warp
            // halves take alternate 16-column chunks of the accumulator
            const int quad = warp & 3, m = 32 * quad + lane;
            if (prod && 32 * quad < NT) {
                for (int c0 = 16 * (warp >> 2); c0 < hp; c0 += 32) {
                    uint32_t r[16];
                    tmem_ld16(taddr + ((uint32_t)(32 * quad) << 16) + (uint32_t)c0, r);
                    if (stacked) {   // plus the second accumulator range
                        uint32_t r2[16];
                        tmem_ld16(taddr + ((uint32_t)(32 * quad) << 16) + (uint32_t)(hp + c0), r2);
#pragma unroll
                        for (int jj = 0; jj < 16; ++jj) r[jj] = __float_as_uint(__uint_as_float(r[jj]) + __uint_as_float(r2[jj]));
                    }
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj)
                        if (c0 + jj < h) ys[(c0 + jj) * NT + m] = __uint_as_float(r[jj]);
                }
            }
        }
        tc_fence_before();
        __syncthreads();
        if (warp == 0) {
            tc_fence_after();
            tmem_free(taddr, ncols);
        }
    } else {
        for (int e = tid; e < h * (NT / 4); e += UMMA_THREADS) ys4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    spmm_tile_finish<NT>(R, c, a, slice, part_stride, ys4, rst);
}

}  // namespace
