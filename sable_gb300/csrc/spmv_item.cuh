// SpMV of one item record by one CTA of SABLE_THREADS threads, the body shared
// by the CTA-per-item kernel and the persistent batch kernel (layout of the
// record in sable_internal.h).
//   cta_accumulate  dense panel (lanes own rows, warps split the quads) into
//                   red[warp][row], CSR entries (g lanes per row) into
//                   ysw[warp][row]
//   cta_finish      fixed-order row sums, output or split-tile partials;
//                   leaves ysw zero
//   combine_tile    y rows of a split tile from its items' partials (run by a
//                   separate launch once all items are done).
// Shared memory: red and ysw, RED_FLOATS floats each, ysw zero on entry.
#pragma once
#include "device_common.cuh"

namespace {

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
    // An item with both parts gives warps [0, wd) to the dense panel and
    // warps [wd, NWARP) to the CSR entries, in proportion to their bytes, so
    // the two latency chains run side by side; otherwise all warps take the
    // one part there is.  The split depends only on the item: fixed sum order.
    int wd = NWARP, wc = 0;
    if (nq > 0 && ns > 0) {
        const int64_t db = 16LL * nq * h, sb = 8LL * ns;
        wd = (int)((NWARP * db + (db + sb) / 2) / (db + sb));
        wd = min(max(wd, 1), NWARP - 1);
        wc = wd;
    }
    const int dense_warps = nq > 0 ? wd : 0;
    if (h <= 32) {
        const int qpw = 32 / h;
        const bool act = lane < qpw * h;
        const int r = lane % h, s = lane / h;
        float acc = 0.f, accb = 0.f;
        if (warp < dense_warps && act) {
            const int step = dense_warps * qpw;
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
        for (int q = warp; warp < dense_warps && q < nq; q += dense_warps) {
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
    if (ns > 0 && warp >= wc) {
        const int *rp = reinterpret_cast<const int *>(R + hd.rp_off);
        const uint2 *E = reinterpret_cast<const uint2 *>(R + hd.csr_off);
        const int nwc = NWARP - wc, wi = warp - wc;
        const int e_lo = (int)(((int64_t)ns * wi) / nwc), e_hi = (int)(((int64_t)ns * (wi + 1)) / nwc);
        const float *xe = xg ? xg + 4 * nq : nullptr;
        csr_rows(rp, E, h, hd.g, e_lo, e_hi, lane, ysw + warp * SABLE_MAX_ROW_TILE,
                 [&](int i, unsigned col) { return xe ? xe[i] : __ldg(x + col); });
    }
}

// Row sums in a fixed order; a single-item tile writes y, an item of a split
// tile stores its row sums as partials (the combine launch adds them).
// Leaves ysw zero.
__device__ __forceinline__ void cta_finish(const ItemHeader &hd, const MatIO &io, const float *red, float *ysw) {
    const int tid = threadIdx.x;
    const int h = hd.h;
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
        if (hd.nitem <= 1) io.y[hd.row0 + i] = tot;
        else io.partial[hd.part_base + (int64_t)hd.kidx * h + i] = tot;
    }
}

// One warp per split tile: y rows = sum of the tile's item partials, in item
// order (the same sum order on every run).
__device__ __forceinline__ void combine_tile(const SplitTile &t, const MatIO &io, int lane) {
    const float *P = io.partial + t.part_base;
    for (int i = lane; i < t.h; i += 32) {
        float s = 0.f;
        for (int k = 0; k < t.nitem; ++k) s += P[(int64_t)k * t.h + i];
        io.y[t.row0 + i] = s;
    }
}

}  // namespace
