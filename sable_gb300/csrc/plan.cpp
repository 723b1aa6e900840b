// Host side of libsable: VBR validation, plan construction (the GPU layout
// of one matrix), upload, and the executor entry points of the C ABI.
//
// Reference counterparts:
//   sable_plan_create   vbr_spmv_codegen / gen_single_threaded_spmv
//                       (src/codegen.py:1438-1447, 293-452): the inspector
//                       that turns one .vbrc matrix into an executable.
//   sable_spmv          the timed loop of the generated program
//                       (src/codegen.py:414-439).
//   sable_spmm          gen_single_threaded_spmm (src/codegen.py:827-937).
//   sable_block_features  the per-block statistics that
//                       convert_vbr_to_compressed feeds to the block model
//                       (utils/convert_real_to_vbr.py:39-58).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace sable {

static thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(SABLE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

const char *cuda_error_string(int err) { return cudaGetErrorString((cudaError_t)err); }

int set_device(int dev) {
    if (dev < 0) return SABLE_OK;
    cudaError_t e = cudaSetDevice(dev);
    return e == cudaSuccess ? SABLE_OK : cuda_fail(e, "cudaSetDevice");
}

template <typename T>
static int upload(T **dptr, const std::vector<T> &h, const char *what) {
    *dptr = nullptr;
    size_t bytes = h.size() * sizeof(T);
    if (bytes == 0) bytes = 16;  // keep every buffer non-null and aligned
    cudaError_t e = cudaMalloc((void **)dptr, bytes);
    if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "cudaMalloc %s (%zu bytes): %s", what, bytes, cudaGetErrorString(e));
    if (!h.empty()) {
        e = cudaMemcpy(*dptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, what);
    }
    return SABLE_OK;
}

// ---------------------------------------------------------------------------
// Validation of the (compressed) VBR arrays.
// ---------------------------------------------------------------------------
int validate_vbrc(const sable_vbrc_desc *d) {
    if (!d) return fail(SABLE_ERR_ARG, "null descriptor");
    if (d->n_block_rows < 0 || d->n_block_cols < 0 || d->n_blocks < 0 || d->n_dense < 0 || d->n_ublocks < 0)
        return fail(SABLE_ERR_INVALID, "negative size in descriptor");
    if (!d->rpntr || !d->cpntr) return fail(SABLE_ERR_ARG, "rpntr/cpntr missing");
    if (d->n_block_rows > 0 && (!d->bpntrb || !d->bpntre)) return fail(SABLE_ERR_ARG, "bpntrb/bpntre missing");
    if (d->n_blocks > 0 && !d->bindx) return fail(SABLE_ERR_ARG, "bindx missing");
    if (d->n_dense > 0 && (!d->val || !d->indx)) return fail(SABLE_ERR_ARG, "val/indx missing");
    if (d->n_ublocks > 0 && !d->ublocks) return fail(SABLE_ERR_ARG, "ublocks missing");
    const int32_t nbr = d->n_block_rows, nbc = d->n_block_cols;
    if (d->rpntr[0] != 0 || d->cpntr[0] != 0) return fail(SABLE_ERR_INVALID, "rpntr[0] and cpntr[0] must be 0");
    for (int32_t a = 0; a < nbr; ++a)
        if (d->rpntr[a + 1] <= d->rpntr[a]) return fail(SABLE_ERR_INVALID, "rpntr not strictly increasing at %d", a);
    for (int32_t b = 0; b < nbc; ++b)
        if (d->cpntr[b + 1] <= d->cpntr[b]) return fail(SABLE_ERR_INVALID, "cpntr not strictly increasing at %d", b);
    if (d->rpntr[nbr] != d->n_rows) return fail(SABLE_ERR_INVALID, "rpntr[-1]=%d != n_rows=%d", d->rpntr[nbr], d->n_rows);
    if (d->cpntr[nbc] != d->n_cols) return fail(SABLE_ERR_INVALID, "cpntr[-1]=%d != n_cols=%d", d->cpntr[nbc], d->n_cols);
    // Block rows must cover bindx contiguously and in order: the generator
    // numbers blocks in (block row, ascending column) order
    // (src/codegen.py:421-435) and ublocks / indx refer to that numbering.
    int64_t next = 0;
    for (int32_t a = 0; a < nbr; ++a) {
        const int32_t b0 = d->bpntrb[a], b1 = d->bpntre[a];
        if (b0 == -1) {
            if (b1 != -1 && b1 != b0) return fail(SABLE_ERR_INVALID, "bpntrb[%d]=-1 but bpntre[%d]=%d", a, a, b1);
            continue;
        }
        if (b0 != next || b1 < b0 || b1 > d->n_blocks)
            return fail(SABLE_ERR_INVALID, "block row %d range [%d,%d) does not continue at %lld", a, b0, b1, (long long)next);
        for (int32_t k = b0; k < b1; ++k) {
            const int32_t b = d->bindx[k];
            if (b < 0 || b >= nbc) return fail(SABLE_ERR_INVALID, "bindx[%d]=%d out of range", k, b);
            if (k > b0 && b <= d->bindx[k - 1]) return fail(SABLE_ERR_INVALID, "bindx not ascending in block row %d", a);
        }
        next = b1;
    }
    if (next != d->n_blocks) return fail(SABLE_ERR_INVALID, "block rows cover %lld of %lld blocks", (long long)next, (long long)d->n_blocks);
    for (int64_t u = 0; u < d->n_ublocks; ++u) {
        if (d->ublocks[u] < 0 || d->ublocks[u] >= d->n_blocks) return fail(SABLE_ERR_INVALID, "ublocks[%lld] out of range", (long long)u);
        if (u > 0 && d->ublocks[u] <= d->ublocks[u - 1]) return fail(SABLE_ERR_INVALID, "ublocks not ascending");
    }
    if (d->n_dense + d->n_ublocks != d->n_blocks)
        return fail(SABLE_ERR_INVALID, "n_dense (%lld) + n_ublocks (%lld) != n_blocks (%lld)", (long long)d->n_dense,
                    (long long)d->n_ublocks, (long long)d->n_blocks);
    if (d->indptr) {
        if (d->indptr[0] != 0) return fail(SABLE_ERR_INVALID, "indptr[0] != 0");
        for (int32_t i = 0; i < d->n_rows; ++i)
            if (d->indptr[i + 1] < d->indptr[i]) return fail(SABLE_ERR_INVALID, "indptr decreasing at %d", i);
        const int64_t nnz = d->indptr[d->n_rows];
        if (nnz > 0 && (!d->indices || !d->csr_val)) return fail(SABLE_ERR_ARG, "indices/csr_val missing");
        for (int64_t k = 0; k < nnz; ++k)
            if (d->indices[k] < 0 || d->indices[k] >= d->n_cols) return fail(SABLE_ERR_INVALID, "indices[%lld] out of range", (long long)k);
    }
    return SABLE_OK;
}

// Dense blocks per block row, in generator order, with their value offsets.
struct DenseBlock { int32_t b; int64_t off; };

static int collect_dense(const sable_vbrc_desc *d, std::vector<std::vector<DenseBlock>> &rows) {
    rows.assign(d->n_block_rows, {});
    int64_t u = 0, dense = 0;
    for (int32_t a = 0; a < d->n_block_rows; ++a) {
        if (d->bpntrb[a] == -1) continue;
        for (int32_t k = d->bpntrb[a]; k < d->bpntre[a]; ++k) {
            if (u < d->n_ublocks && d->ublocks[u] == k) { ++u; continue; }
            const int32_t b = d->bindx[k];
            const int64_t hw = (int64_t)(d->rpntr[a + 1] - d->rpntr[a]) * (d->cpntr[b + 1] - d->cpntr[b]);
            if (d->indx[dense + 1] - d->indx[dense] != hw || d->indx[dense] < 0)
                return fail(SABLE_ERR_INVALID, "indx[%lld..] spans %lld values, block is %lld", (long long)dense,
                            (long long)(d->indx[dense + 1] - d->indx[dense]), (long long)hw);
            rows[a].push_back({b, d->indx[dense]});
            ++dense;
        }
    }
    return SABLE_OK;
}

// ---------------------------------------------------------------------------
// Plan construction: tiles -> items -> records.
// ---------------------------------------------------------------------------
static inline int64_t pad16(int64_t b) { return (b + 15) & ~(int64_t)15; }

namespace {
struct Run { int32_t col0, len; };  // window run: first x column (-1: zeros), positions

// Window runs of one compact item: the panel columns xcol[4 q0, 4 q1) (-1 for
// padding), then the sorted distinct columns of CSR entries [e0, e1) of
// `indices`, runs closer than SABLE_CW_GAP merged.  Returns the window length;
// n_dense_runs = runs of the panel part.
int64_t compact_window(const int32_t *xcol, int64_t q0, int64_t q1, const int32_t *indices, int64_t e0, int64_t e1,
                       std::vector<Run> &runs, size_t &n_dense_runs, std::vector<int32_t> &scratch) {
    runs.clear();
    for (int64_t p = 4 * q0; p < 4 * q1; ++p) {
        const int32_t c = xcol[p];
        if (!runs.empty()) {
            Run &r = runs.back();
            if ((c < 0 && r.col0 < 0) || (c >= 0 && r.col0 >= 0 && r.col0 + r.len == c)) { ++r.len; continue; }
        }
        runs.push_back({c < 0 ? -1 : c, 1});
    }
    n_dense_runs = runs.size();
    int64_t nw = 4 * (q1 - q0);
    if (e1 > e0) {
        scratch.assign(indices + e0, indices + e1);
        std::sort(scratch.begin(), scratch.end());
        scratch.erase(std::unique(scratch.begin(), scratch.end()), scratch.end());
        for (int32_t c : scratch) {
            if (runs.size() > n_dense_runs) {
                Run &r = runs.back();
                if (c - (r.col0 + r.len) < SABLE_CW_GAP) { r.len = c - r.col0 + 1; continue; }
            }
            runs.push_back({c, 1});
        }
        for (size_t k = n_dense_runs; k < runs.size(); ++k) nw += runs[k].len;
    }
    return nw;
}
}  // namespace

int build_layout(const sable_vbrc_desc *d, int row_tile, int item_bytes, int split_layout, Layout &L, bool compact) {
    std::vector<std::vector<DenseBlock>> rows;
    int rc = collect_dense(d, rows);
    if (rc) return rc;
    L = Layout();
    L.n_rows = d->n_rows;
    L.n_cols = d->n_cols;
    int64_t part_floats = 0;
    int32_t split_tiles = 0;
    int64_t tile_id = 0;
    std::vector<float4> panel;      // tile panel (host scratch)
    std::vector<int32_t> xcol;      // tile panel column -> x column
    std::vector<int64_t> tp;        // tile-relative CSR row starts

    auto emit_item = [&](int32_t row0, int32_t h, int64_t q0, int64_t q1, int64_t s0, int64_t s1, int64_t k0,
                         int32_t tile, int32_t kidx, int32_t nitem, int64_t part_base) {
        const int32_t nq = (int32_t)(q1 - q0), ns = (int32_t)(s1 - s0);
        ItemHeader hd;
        memset(&hd, 0, sizeof hd);
        hd.row0 = row0;
        hd.h = h;
        hd.nq = nq;
        hd.ns = ns;
        int64_t off = sizeof(ItemHeader);
        hd.xcol_off = (int32_t)off;
        off += 16 * (int64_t)nq;                      // 4 int32 per quad
        hd.panel_off = (int32_t)off;
        off += 16 * (int64_t)nq * h;
        hd.rp_off = (int32_t)off;
        off += ns > 0 ? pad16(4 * ((int64_t)h + 1)) : 0;
        hd.csr_off = (int32_t)off;
        off += pad16(8 * (int64_t)ns);
        hd.bytes = (int32_t)off;
        hd.tile = tile;
        hd.kidx = kidx;
        hd.nitem = nitem;
        hd.part_base = part_base;
        hd.mat = 0;
        // lanes per CSR row from the mean length of the item's non-empty rows
        int32_t nonempty = 0;
        std::vector<int32_t> rp;
        if (ns > 0) {
            rp.resize(h + 1);
            for (int32_t i = 0; i <= h; ++i) rp[i] = (int32_t)std::min<int64_t>(std::max<int64_t>(tp[i] - s0, 0), s1 - s0);
            for (int32_t i = 0; i < h; ++i) nonempty += rp[i + 1] > rp[i];
        }
        const double avg = nonempty ? (double)ns / nonempty : 0.0;
        hd.g = avg <= 12 ? 4 : avg <= 24 ? 8 : avg <= 48 ? 16 : 32;
        const int64_t base = (int64_t)L.records.size();
        L.records.resize(base + hd.bytes, 0);
        unsigned char *R = L.records.data() + base;
        memcpy(R, &hd, sizeof hd);
        memcpy(R + hd.xcol_off, xcol.data() + 4 * q0, 16 * (size_t)nq);
        memcpy(R + hd.panel_off, panel.data() + q0 * h, 16 * (size_t)nq * h);
        if (ns > 0) {
            memcpy(R + hd.rp_off, rp.data(), 4 * (size_t)(h + 1));
            uint2 *E = reinterpret_cast<uint2 *>(R + hd.csr_off);
            for (int64_t k = 0; k < ns; ++k) {
                float v = d->csr_val[k0 + s0 + k];
                memcpy(&E[k].x, &v, 4);
                E[k].y = (uint32_t)d->indices[k0 + s0 + k];
            }
        }
        ItemRef ref;
        ref.off = base;
        ref.bytes = hd.bytes;
        ref.cost = hd.bytes;
        L.items.push_back(ref);
        L.item_tile.push_back(tile_id);
        L.max_item_bytes = std::max<int>(L.max_item_bytes, hd.bytes);
        L.max_xg_floats = std::max<int>(L.max_xg_floats, 4 * nq + ns);
    };

    // Compact record of quads [q0, q1) and tile CSR entries [s0, s1) (global
    // entry k0 + s); the caller has checked that its window fits.
    std::vector<Run> runs;
    std::vector<int32_t> scratch;
    auto emit_compact = [&](int32_t row0, int32_t h, int64_t q0, int64_t q1, int64_t s0, int64_t s1, int64_t k0,
                            int32_t tile, int32_t kidx, int32_t nitem, int64_t part_base) -> int {
        size_t nd_runs = 0;
        const int64_t nw = compact_window(xcol.data(), q0, q1, d->indices, k0 + s0, k0 + s1, runs, nd_runs, scratch);
        if (nw > SABLE_CW_MAX) return fail(SABLE_ERR_INVALID, "layout: compact window %lld", (long long)nw);
        const int32_t nq = (int32_t)(q1 - q0), ns = (int32_t)(s1 - s0), nrun = (int32_t)runs.size();
        CompactHeader hd;
        memset(&hd, 0, sizeof hd);
        hd.row0 = row0;
        hd.h = h;
        hd.nq = nq;
        hd.ns = ns;
        int64_t off = sizeof(CompactHeader);
        hd.runs_off = (int32_t)off;
        off += pad16(8 * (int64_t)nrun);
        hd.panel_off = (int32_t)off;
        off += 16 * (int64_t)nq * h;
        hd.rp_off = (int32_t)off;
        hd.val_off = (int32_t)off;
        off += 32 * (((int64_t)ns + 7) / 8);  // whole groups of 8 entries
        hd.meta_off = (int32_t)off;
        off += 16 * (((int64_t)ns + 7) / 8);
        hd.bytes = (int32_t)off;
        hd.tile = tile;
        hd.kidx = kidx;
        hd.nitem = nitem;
        hd.part_base = part_base;
        hd.nrun = (int16_t)nrun;
        hd.nw = (int16_t)nw;
        const int64_t base = (int64_t)L.records.size();
        L.records.resize(base + hd.bytes, 0);
        unsigned char *R = L.records.data() + base;
        memcpy(R, &hd, sizeof hd);
        memcpy(R + hd.runs_off, runs.data(), 8 * (size_t)nrun);
        memcpy(R + hd.panel_off, panel.data() + q0 * h, 16 * (size_t)nq * h);
        if (ns > 0) {
            memcpy(R + hd.val_off, d->csr_val + k0 + s0, 4 * (size_t)ns);
            // window position of each entry's column (its run's first position
            // + offset) and the entry's tile row
            std::vector<int64_t> start(nrun + 1 - nd_runs);
            start[0] = 4 * (int64_t)nq;
            for (size_t r = nd_runs; r < runs.size(); ++r) start[r - nd_runs + 1] = start[r - nd_runs] + runs[r].len;
            uint16_t *meta = reinterpret_cast<uint16_t *>(R + hd.meta_off);
            int32_t row = 0;
            for (int64_t k = 0; k < ns; ++k) {
                while (tp[row + 1] <= s0 + k) ++row;
                const int32_t c = d->indices[k0 + s0 + k];
                // last CSR run whose first column is <= c
                size_t lo = nd_runs, hi = runs.size();
                while (hi - lo > 1) {
                    const size_t mid = (lo + hi) / 2;
                    if (runs[mid].col0 <= c) lo = mid;
                    else hi = mid;
                }
                meta[k] = (uint16_t)((start[lo - nd_runs] + (c - runs[lo].col0)) | (row << 10));
            }
        }
        ItemRef ref;
        ref.off = base;
        ref.bytes = hd.bytes;
        ref.cost = hd.bytes;
        L.items.push_back(ref);
        L.item_tile.push_back(tile_id);
        L.max_item_bytes = std::max<int>(L.max_item_bytes, hd.bytes);
        L.max_xg_floats = std::max<int>(L.max_xg_floats, (int)nw);
        return SABLE_OK;
    };
    // Window length of quads [q0, q1) and CSR entries [s0, s1) of the tile.
    auto window_of = [&](int64_t q0, int64_t q1, int64_t s0, int64_t s1, int64_t k0) {
        size_t nd_runs = 0;
        return compact_window(xcol.data(), q0, q1, d->indices, k0 + s0, k0 + s1, runs, nd_runs, scratch);
    };

    // Compact items of one tile: a single item when the tile's record fits
    // item_bytes (+25 %) and its window fits; otherwise a split tile (mixed
    // layout: equal shares of quads and entries per item; separate layout:
    // dense items, then CSR items) whose item count grows until every item's
    // window fits.
    auto cut_compact = [&](int32_t row0, int32_t h, int64_t nq, int64_t ns, int64_t k0) -> int {
        const int64_t hdr = sizeof(CompactHeader);
        {
            const int64_t nw = window_of(0, nq, 0, ns, k0);
            const int64_t bytes = hdr + pad16(8 * (int64_t)runs.size()) + 16 * nq * h + 48 * ((ns + 7) / 8);
            if (nw <= SABLE_CW_MAX && bytes <= item_bytes + item_bytes / 4)
                return emit_compact(row0, h, 0, nq, 0, ns, k0, -1, 0, 1, 0);
        }
        const int64_t avail = std::max<int64_t>(1024, item_bytes - hdr - 128);
        auto grow = [](int64_t n) { return n + std::max<int64_t>(1, n / 4); };
        int64_t nd = 0, nsp = 0, nitem;
        if (split_layout == 0) {
            nitem = std::max<int64_t>(2, (16 * nq * h + 6 * ns + avail - 1) / avail);
            for (;;) {
                bool ok = true;
                for (int64_t k = 0; k < nitem && ok; ++k)
                    ok = window_of(nq * k / nitem, nq * (k + 1) / nitem, ns * k / nitem, ns * (k + 1) / nitem, k0) <=
                         SABLE_CW_MAX;
                if (ok) break;
                nitem = grow(nitem);
            }
        } else {
            if (nq > 0) nd = std::max((16 * nq * h + avail - 1) / avail, (4 * nq + SABLE_CW_MAX - 1) / SABLE_CW_MAX);
            if (ns > 0) {
                nsp = (6 * ns + avail - 1) / avail;
                for (;;) {
                    bool ok = true;
                    for (int64_t k = 0; k < nsp && ok; ++k)
                        ok = window_of(0, 0, ns * k / nsp, ns * (k + 1) / nsp, k0) <= SABLE_CW_MAX;
                    if (ok) break;
                    nsp = grow(nsp);
                }
            }
            nitem = std::max<int64_t>(2, nd + nsp);
            if (nd + nsp < 2) nd = nitem - nsp;  // one oversized part: cut its dense quads in two
        }
        if (nitem > INT32_MAX / 2) return fail(SABLE_ERR_UNSUPPORTED, "tile at row %d needs %lld items", row0, (long long)nitem);
        const int32_t sid = split_tiles++;
        const int64_t pbase = part_floats;
        part_floats += nitem * h;
        SplitTile st;
        st.part_base = pbase;
        st.row0 = row0;
        st.h = h;
        st.nitem = (int32_t)nitem;
        st.mat = 0;
        L.splits.push_back(st);
        int rc2 = SABLE_OK;
        if (split_layout == 0) {
            for (int64_t k = 0; k < nitem && !rc2; ++k)
                rc2 = emit_compact(row0, h, nq * k / nitem, nq * (k + 1) / nitem, ns * k / nitem, ns * (k + 1) / nitem, k0,
                                   sid, (int32_t)k, (int32_t)nitem, pbase);
        } else {
            int32_t kidx = 0;
            for (int64_t k = 0; k < nd && !rc2; ++k)
                rc2 = emit_compact(row0, h, nq * k / nd, nq * (k + 1) / nd, 0, 0, k0, sid, kidx++, (int32_t)nitem, pbase);
            for (int64_t k = 0; k < nsp && !rc2; ++k)
                rc2 = emit_compact(row0, h, 0, 0, ns * k / nsp, ns * (k + 1) / nsp, k0, sid, kidx++, (int32_t)nitem, pbase);
        }
        return rc2;
    };

    if (compact) row_tile = std::min(row_tile, SABLE_CW_MAX_ROWS);
    for (int32_t a = 0; a < d->n_block_rows; ++a) {
        const int32_t r0 = d->rpntr[a], hb = d->rpntr[a + 1] - r0;
        const int32_t nt = (hb + row_tile - 1) / row_tile;
        int32_t W = 0;
        for (const DenseBlock &db : rows[a]) W += d->cpntr[db.b + 1] - d->cpntr[db.b];
        const int64_t nq = (W + 3) / 4;
        for (int32_t t = 0; t < nt; ++t, ++tile_id) {
            const int32_t lo = (int32_t)((int64_t)hb * t / nt), hi = (int32_t)((int64_t)hb * (t + 1) / nt);
            const int32_t h = hi - lo, row0 = r0 + lo;
            // tile panel and its x columns
            panel.assign((size_t)(nq * h), make_float4(0.f, 0.f, 0.f, 0.f));
            xcol.assign((size_t)(4 * nq), compact ? -1 : 0);
            float *P = reinterpret_cast<float *>(panel.data());
            int32_t pc = 0;
            for (const DenseBlock &db : rows[a]) {
                const int32_t c0 = d->cpntr[db.b], w = d->cpntr[db.b + 1] - c0;
                const float *blk = d->val + db.off;
                for (int32_t j = 0; j < w; ++j, ++pc) {
                    xcol[pc] = c0 + j;
                    const int64_t q = pc >> 2, comp = pc & 3;
                    const float *colv = blk + (int64_t)j * hb + lo;
                    float *dst = P + (q * h) * 4 + comp;
                    for (int32_t i = 0; i < h; ++i) dst[(int64_t)i * 4] = colv[i];
                }
            }
            L.dense_values += (int64_t)W * h;
            L.dense_padded += 4 * nq * h;
            // CSR rows of the tile
            int64_t k0 = 0, ns = 0;
            tp.assign((size_t)h + 1, 0);
            if (d->indptr) {
                k0 = d->indptr[row0];
                ns = d->indptr[row0 + h] - k0;
                for (int32_t i = 0; i <= h; ++i) tp[i] = d->indptr[row0 + i] - k0;
            }
            L.sparse_nnz += ns;
            if (compact) {
                rc = cut_compact(row0, h, nq, ns, k0);
                if (rc) return rc;
                continue;
            }
            // cut into items
            const int64_t hdr = sizeof(ItemHeader);
            const int64_t total = hdr + 16 * nq + 16 * nq * h + (ns ? pad16(4 * ((int64_t)h + 1)) + pad16(8 * ns) : 0);
            if (total <= item_bytes + item_bytes / 4) {
                emit_item(row0, h, 0, nq, 0, ns, k0, -1, 0, 1, 0);
                continue;
            }
            // Split tile.  Mixed layout: every item takes an equal share of the
            // tile's quads and of its CSR entries (each item then mixes both
            // parts like a tile that fits one item, and no item is CSR-only).
            // Separate layout: dense items of the quads, then CSR items; each
            // part alone exceeds an item whenever the tile is split, so
            // nd + nsp >= 2.
            const int64_t avail_d = std::max<int64_t>(1024, item_bytes - hdr);
            const int64_t avail_s = std::max<int64_t>(1024, item_bytes - hdr - pad16(4 * ((int64_t)h + 1)) - 16);
            int32_t nd = 0, nsp = 0, nitem;
            if (split_layout == 0) {
                const int64_t content = 16 * nq * ((int64_t)h + 1) + 8 * ns;
                nitem = (int32_t)std::max<int64_t>(2, (content + avail_s - 1) / avail_s);
            } else {
                nd = (int32_t)((16 * nq * ((int64_t)h + 1) + avail_d - 1) / avail_d);
                nsp = (int32_t)((8 * ns + avail_s - 1) / avail_s);
                nitem = nd + nsp;
            }
            const int32_t sid = split_tiles++;
            const int64_t pbase = part_floats;
            part_floats += (int64_t)nitem * h;
            SplitTile st;
            st.part_base = pbase;
            st.row0 = row0;
            st.h = h;
            st.nitem = nitem;
            st.mat = 0;
            L.splits.push_back(st);
            if (split_layout == 0) {
                for (int32_t k = 0; k < nitem; ++k) {
                    const int64_t q0 = nq * k / nitem, q1 = nq * (k + 1) / nitem;
                    const int64_t s0 = ns * k / nitem, s1 = ns * (k + 1) / nitem;
                    emit_item(row0, h, q0, q1, s0, s1, k0, sid, k, nitem, pbase);
                }
            } else {
                int32_t kidx = 0;
                for (int32_t k = 0; k < nd; ++k)
                    emit_item(row0, h, nq * k / nd, nq * (k + 1) / nd, 0, 0, k0, sid, kidx++, nitem, pbase);
                for (int32_t k = 0; k < nsp; ++k)
                    emit_item(row0, h, 0, 0, ns * k / nsp, ns * (k + 1) / nsp, k0, sid, kidx++, nitem, pbase);
            }
        }
    }
    L.n_tiles = tile_id;
    L.n_partial = part_floats;
    L.n_split_tiles = split_tiles;
    L.compact = compact;
    return compact ? check_compact_layout(L) : check_layout(L);
}

// Every index a kernel will follow, checked on the host before upload.
int check_layout(const Layout &L) {
    const int64_t nrec = (int64_t)L.records.size();
    for (size_t k = 0; k < L.items.size(); ++k) {
        const ItemRef &r = L.items[k];
        if (r.off < 0 || (r.off & 15) || r.bytes < (int)sizeof(ItemHeader) || (r.bytes & 15) || r.off + r.bytes > nrec ||
            r.bytes > SABLE_MAX_RECORD_BYTES)
            return fail(SABLE_ERR_INVALID, "layout: item %zu record range", k);
        ItemHeader hd;
        memcpy(&hd, L.records.data() + r.off, sizeof hd);
        if (hd.bytes != r.bytes) return fail(SABLE_ERR_INVALID, "layout: item %zu size mismatch", k);
        if (hd.h < 1 || hd.h > SABLE_MAX_ROW_TILE || hd.row0 < 0 || hd.row0 + hd.h > L.n_rows)
            return fail(SABLE_ERR_INVALID, "layout: item %zu rows out of range", k);
        if (hd.nq < 0 || hd.ns < 0 || hd.xcol_off != (int)sizeof(ItemHeader) ||
            hd.panel_off != hd.xcol_off + 16 * hd.nq || (int64_t)hd.rp_off != hd.panel_off + 16 * (int64_t)hd.nq * hd.h ||
            hd.csr_off < hd.rp_off || (int64_t)hd.csr_off + 8 * (int64_t)hd.ns > hd.bytes)
            return fail(SABLE_ERR_INVALID, "layout: item %zu part offsets", k);
        const unsigned char *R = L.records.data() + r.off;
        const int32_t *xc = reinterpret_cast<const int32_t *>(R + hd.xcol_off);
        for (int i = 0; i < 4 * hd.nq; ++i)
            if (xc[i] < 0 || xc[i] >= L.n_cols) return fail(SABLE_ERR_INVALID, "layout: item %zu x column", k);
        if (hd.ns > 0) {
            const int32_t *rp = reinterpret_cast<const int32_t *>(R + hd.rp_off);
            if (rp[0] != 0 || rp[hd.h] != hd.ns) return fail(SABLE_ERR_INVALID, "layout: item %zu row pointers", k);
            for (int i = 0; i < hd.h; ++i)
                if (rp[i + 1] < rp[i]) return fail(SABLE_ERR_INVALID, "layout: item %zu row pointers decrease", k);
            const uint2 *E = reinterpret_cast<const uint2 *>(R + hd.csr_off);
            for (int i = 0; i < hd.ns; ++i)
                if ((int64_t)E[i].y >= L.n_cols) return fail(SABLE_ERR_INVALID, "layout: item %zu CSR column", k);
        }
        if (hd.g != 4 && hd.g != 8 && hd.g != 16 && hd.g != 32) return fail(SABLE_ERR_INVALID, "layout: item %zu lane group", k);
        if (hd.nitem < 1 || hd.kidx < 0 || hd.kidx >= hd.nitem) return fail(SABLE_ERR_INVALID, "layout: item %zu numbering", k);
        if (hd.nitem > 1 && (hd.tile < 0 || hd.tile >= L.n_split_tiles || hd.part_base < 0 ||
                             hd.part_base + (int64_t)hd.nitem * hd.h > L.n_partial))
            return fail(SABLE_ERR_INVALID, "layout: item %zu split-tile scratch out of bounds", k);
    }
    return SABLE_OK;
}

// Compact records: every index the per-warp kernel follows, checked on the
// host before upload (runs, window positions, row pointers, split scratch).
int check_compact_layout(const Layout &L) {
    const int64_t nrec = (int64_t)L.records.size();
    for (size_t k = 0; k < L.items.size(); ++k) {
        const ItemRef &r = L.items[k];
        if (r.off < 0 || (r.off & 15) || r.bytes < (int)sizeof(CompactHeader) || (r.bytes & 15) ||
            r.off + r.bytes > nrec || r.bytes > SABLE_MAX_ITEM_BYTES)
            return fail(SABLE_ERR_INVALID, "layout: item %zu record range", k);
        CompactHeader hd;
        memcpy(&hd, L.records.data() + r.off, sizeof hd);
        if (hd.bytes != r.bytes) return fail(SABLE_ERR_INVALID, "layout: item %zu size mismatch", k);
        if (hd.h < 1 || hd.h > SABLE_MAX_ROW_TILE || hd.row0 < 0 || hd.row0 + hd.h > L.n_rows)
            return fail(SABLE_ERR_INVALID, "layout: item %zu rows out of range", k);
        const int64_t nq = hd.nq, ns = hd.ns, nrun = hd.nrun, nw = hd.nw;
        if (hd.h > SABLE_CW_MAX_ROWS) return fail(SABLE_ERR_INVALID, "layout: item %zu compact tile height", k);
        if (nq < 0 || ns < 0 || nrun < 0 || nw < 4 * nq || nw > SABLE_CW_MAX || hd.runs_off != (int)sizeof(CompactHeader) ||
            hd.panel_off != hd.runs_off + pad16(8 * nrun) || hd.rp_off != hd.panel_off + 16 * nq * hd.h ||
            hd.val_off != hd.rp_off || hd.meta_off != hd.val_off + 32 * ((ns + 7) / 8) ||
            hd.bytes != hd.meta_off + 16 * ((ns + 7) / 8))
            return fail(SABLE_ERR_INVALID, "layout: item %zu part offsets", k);
        const unsigned char *R = L.records.data() + r.off;
        int64_t total = 0;
        for (int64_t i = 0; i < nrun; ++i) {
            int32_t run[2];
            memcpy(run, R + hd.runs_off + 8 * i, 8);
            if (run[1] < 1 || run[0] < -1 || (run[0] >= 0 && (int64_t)run[0] + run[1] > L.n_cols))
                return fail(SABLE_ERR_INVALID, "layout: item %zu window run", k);
            total += run[1];
        }
        if (total != nw) return fail(SABLE_ERR_INVALID, "layout: item %zu window length", k);
        const uint16_t *meta = reinterpret_cast<const uint16_t *>(R + hd.meta_off);
        for (int64_t i = 0; i < ns; ++i) {
            const int pos = meta[i] & 1023, row = meta[i] >> 10;
            if (pos < 4 * nq || pos >= nw) return fail(SABLE_ERR_INVALID, "layout: item %zu window position", k);
            if (row >= hd.h || (i > 0 && row < (meta[i - 1] >> 10)))
                return fail(SABLE_ERR_INVALID, "layout: item %zu CSR rows", k);
        }
        if (hd.nitem < 1 || hd.kidx < 0 || hd.kidx >= hd.nitem) return fail(SABLE_ERR_INVALID, "layout: item %zu numbering", k);
        if (hd.nitem > 1 && (hd.tile < 0 || hd.tile >= L.n_split_tiles || hd.part_base < 0 ||
                             hd.part_base + (int64_t)hd.nitem * hd.h > L.n_partial))
            return fail(SABLE_ERR_INVALID, "layout: item %zu split-tile scratch out of bounds", k);
    }
    return SABLE_OK;
}

}  // namespace sable

using namespace sable;

extern "C" {

const char *sable_strerror(int code) {
    switch (code) {
        case SABLE_OK: return "ok";
        case SABLE_ERR_INVALID: return "invalid VBR arrays";
        case SABLE_ERR_CUDA: return "CUDA error";
        case SABLE_ERR_NOMEM: return "out of memory";
        case SABLE_ERR_UNSUPPORTED: return "unsupported input";
        case SABLE_ERR_TIMEOUT: return "device wait timed out";
        case SABLE_ERR_ARG: return "bad argument";
        default: return "unknown error";
    }
}

const char *sable_last_error(void) { return g_last_error.c_str(); }

const char *sable_version(void) { return "sable-gb300 0.1 (sm_103a)"; }

int sable_plan_create(const sable_vbrc_desc *desc, const sable_plan_opts *opts, sable_plan **out) {
    if (!out) return fail(SABLE_ERR_ARG, "null output pointer");
    *out = nullptr;
    sable_plan_opts o;
    memset(&o, 0, sizeof o);
    o.device = -1;
    if (opts) o = *opts;
    const int row_tile = o.row_tile ? o.row_tile : SABLE_MAX_ROW_TILE;
    const int chunk_bytes = o.chunk_bytes ? o.chunk_bytes
                                          : (o.schedule == SABLE_SCHEDULE_ITEMS ? SABLE_ITEMS_ITEM_BYTES
                                             : o.schedule == SABLE_SCHEDULE_WARP_ITEMS ? SABLE_WARP_ITEMS_ITEM_BYTES
                                                                                       : SABLE_WARP_ITEM_BYTES);
    if (row_tile < 1 || row_tile > SABLE_MAX_ROW_TILE) return fail(SABLE_ERR_ARG, "row_tile %d outside 1..128", row_tile);
    const int max_chunk = o.schedule == SABLE_SCHEDULE_ITEMS ? SABLE_MAX_CHUNK_BYTES : SABLE_MAX_ITEM_BYTES * 4 / 5;
    if (chunk_bytes < 4096 || chunk_bytes > max_chunk)
        return fail(SABLE_ERR_ARG, "chunk_bytes %d outside 4096..%d", chunk_bytes, max_chunk);
    int rc = validate_vbrc(desc);
    if (rc) return rc;
    rc = set_device(o.device);
    if (rc) return rc;
    sable_plan *p = new (std::nothrow) sable_plan();
    if (!p) return fail(SABLE_ERR_NOMEM, "host allocation");
    cudaGetDevice(&p->device);
    p->row_tile = row_tile;
    p->item_bytes = chunk_bytes;
    if (o.schedule != SABLE_SCHEDULE_ITEMS && o.schedule != SABLE_SCHEDULE_PERSISTENT &&
        o.schedule != SABLE_SCHEDULE_WARP_ITEMS) {
        delete p;
        return fail(SABLE_ERR_ARG, "schedule %d unknown", o.schedule);
    }
    p->schedule = o.schedule;
    if (o.spmm_tc < SABLE_TC_OFF || o.spmm_tc > SABLE_TC_SPLIT3) {
        delete p;
        return fail(SABLE_ERR_ARG, "spmm_tc %d unknown", o.spmm_tc);
    }
    p->spmm_tc = o.spmm_tc;
    if (o.tc_kernel != SABLE_TC_KERNEL_UMMA && o.tc_kernel != SABLE_TC_KERNEL_MMASYNC) {
        delete p;
        return fail(SABLE_ERR_ARG, "tc_kernel %d unknown", o.tc_kernel);
    }
    p->tc_kernel = o.tc_kernel;
    Layout L;
    if (o.split_layout != 0 && o.split_layout != 1) {
        delete p;
        return fail(SABLE_ERR_ARG, "split_layout %d unknown", o.split_layout);
    }
    rc = build_layout(desc, row_tile, chunk_bytes, o.split_layout, L, o.schedule == SABLE_SCHEDULE_WARP_ITEMS);
    if (rc) { delete p; return rc; }
    rc = plan_upload(p, L);
    if (rc) { sable_plan_destroy(p); return rc; }
    *out = p;
    return SABLE_OK;
}

// Option checks and the host layout of sable_plan_create, without CUDA.
static int host_layout(const sable_vbrc_desc *desc, const sable_plan_opts *opts, Layout &L) {
    const int row_tile = opts && opts->row_tile ? opts->row_tile : SABLE_MAX_ROW_TILE;
    const int chunk_bytes = opts && opts->chunk_bytes ? opts->chunk_bytes
                            : (!opts || opts->schedule == SABLE_SCHEDULE_ITEMS ? SABLE_ITEMS_ITEM_BYTES
                               : opts->schedule == SABLE_SCHEDULE_WARP_ITEMS ? SABLE_WARP_ITEMS_ITEM_BYTES
                                                                             : SABLE_WARP_ITEM_BYTES);
    if (row_tile < 1 || row_tile > SABLE_MAX_ROW_TILE) return fail(SABLE_ERR_ARG, "row_tile %d outside 1..128", row_tile);
    const int max_chunk = (!opts || opts->schedule == SABLE_SCHEDULE_ITEMS) ? SABLE_MAX_CHUNK_BYTES
                                                                           : SABLE_MAX_ITEM_BYTES * 4 / 5;
    if (chunk_bytes < 4096 || chunk_bytes > max_chunk) return fail(SABLE_ERR_ARG, "chunk_bytes outside range");
    int rc = validate_vbrc(desc);
    if (rc) return rc;
    const int split_layout = opts ? opts->split_layout : 0;
    if (split_layout != 0 && split_layout != 1) return fail(SABLE_ERR_ARG, "split_layout %d unknown", split_layout);
    return build_layout(desc, row_tile, chunk_bytes, split_layout, L,
                        opts && opts->schedule == SABLE_SCHEDULE_WARP_ITEMS);
}

int sable_plan_dry_run(const sable_vbrc_desc *desc, const sable_plan_opts *opts, sable_plan_stats *out) {
    if (!out) return fail(SABLE_ERR_ARG, "null output pointer");
    Layout L;
    const int rc = host_layout(desc, opts, L);
    if (rc) return rc;
    memset(out, 0, sizeof *out);
    out->n_tiles = L.n_tiles;
    out->n_chunks = (int64_t)L.items.size();
    out->dense_values = L.dense_values;
    out->dense_padded = L.dense_padded;
    out->sparse_nnz = L.sparse_nnz;
    out->device_bytes = (int64_t)L.records.size() + (int64_t)L.items.size() * (int64_t)sizeof(ItemRef) +
                        (L.n_partial + L.n_split_tiles) * 4;
    out->scratch_floats = L.n_partial;
    return SABLE_OK;
}

int sable_plan_layout_host(const sable_vbrc_desc *desc, const sable_plan_opts *opts, unsigned char *records,
                           int64_t records_cap, int64_t *records_bytes, int64_t *item_off, int32_t *item_bytes,
                           int64_t items_cap, int64_t *n_items) {
    if (!records_bytes || !n_items) return fail(SABLE_ERR_ARG, "null output pointer");
    Layout L;
    const int rc = host_layout(desc, opts, L);
    if (rc) return rc;
    *records_bytes = (int64_t)L.records.size();
    *n_items = (int64_t)L.items.size();
    if (!records) return SABLE_OK;
    if (records_cap < *records_bytes || items_cap < *n_items || !item_off || !item_bytes)
        return fail(SABLE_ERR_ARG, "output buffers smaller than the layout (%lld bytes, %lld items)",
                    (long long)*records_bytes, (long long)*n_items);
    memcpy(records, L.records.data(), L.records.size());
    for (size_t k = 0; k < L.items.size(); ++k) {
        item_off[k] = L.items[k].off;
        item_bytes[k] = L.items[k].bytes;
    }
    return SABLE_OK;
}

int sable_plan_get_stats(const sable_plan *plan, sable_plan_stats *out) {
    if (!plan || !out) return fail(SABLE_ERR_ARG, "null argument");
    *out = plan->stats;
    return SABLE_OK;
}

int sable_plan_chunk_tiles(const sable_plan *plan, int64_t *tile_of_chunk) {
    if (!plan || !tile_of_chunk) return fail(SABLE_ERR_ARG, "null argument");
    memcpy(tile_of_chunk, plan->item_tile.data(), plan->item_tile.size() * sizeof(int64_t));
    return SABLE_OK;
}

int sable_block_features(const sable_vbrc_desc *d, int32_t N, float *feat) {
    if (!d || !feat) return fail(SABLE_ERR_ARG, "null argument");
    if (d->n_ublocks != 0 || d->n_dense != d->n_blocks)
        return fail(SABLE_ERR_ARG, "block features need the uncompressed form (all blocks in val)");
    int rc = validate_vbrc(d);
    if (rc) return rc;
    std::vector<int32_t> rownnz;
    for (int32_t a = 0; a < d->n_block_rows; ++a) {
        if (d->bpntrb[a] == -1) continue;
        const int32_t h = d->rpntr[a + 1] - d->rpntr[a];
        for (int32_t k = d->bpntrb[a]; k < d->bpntre[a]; ++k) {
            const int32_t b = d->bindx[k], w = d->cpntr[b + 1] - d->cpntr[b];
            if (d->indx[k + 1] - d->indx[k] != (int64_t)h * w) return fail(SABLE_ERR_INVALID, "indx[%d] size mismatch", k);
            const float *blk = d->val + d->indx[k];
            rownnz.assign(h, 0);
            int64_t nnz = 0;
            for (int32_t j = 0; j < w; ++j)
                for (int32_t i = 0; i < h; ++i)
                    if (blk[(int64_t)j * h + i] != 0.0f) { ++rownnz[i]; ++nnz; }
            double mean = (double)nnz / h, var = 0.0;
            for (int32_t i = 0; i < h; ++i) var += (rownnz[i] - mean) * (rownnz[i] - mean);
            var /= h;
            float *f = feat + (int64_t)k * 6;
            f[0] = (float)h;
            f[1] = (float)w;
            f[2] = (float)nnz;
            f[3] = (float)((double)nnz / ((double)h * w));
            f[4] = (float)var;
            f[5] = (float)N;
        }
    }
    return SABLE_OK;
}

}  // extern "C"
