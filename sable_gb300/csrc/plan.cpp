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

int build_layout(const sable_vbrc_desc *d, int row_tile, int item_bytes, int split_layout, Layout &L) {
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
            xcol.assign((size_t)(4 * nq), 0);
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
    return check_layout(L);
}

// Every index a kernel will follow, checked on the host before upload.
int check_layout(const Layout &L) {
    const int64_t nrec = (int64_t)L.records.size();
    for (size_t k = 0; k < L.items.size(); ++k) {
        const ItemRef &r = L.items[k];
        if (r.off < 0 || (r.off & 15) || r.bytes < (int)sizeof(ItemHeader) || (r.bytes & 15) || r.off + r.bytes > nrec ||
            r.bytes > SABLE_MAX_ITEM_BYTES)
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
    if (chunk_bytes < 4096 || chunk_bytes > SABLE_MAX_ITEM_BYTES * 4 / 5)
        return fail(SABLE_ERR_ARG, "chunk_bytes %d outside 4096..%d", chunk_bytes, SABLE_MAX_ITEM_BYTES * 4 / 5);
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
    Layout L;
    if (o.split_layout != 0 && o.split_layout != 1) {
        delete p;
        return fail(SABLE_ERR_ARG, "split_layout %d unknown", o.split_layout);
    }
    rc = build_layout(desc, row_tile, chunk_bytes, o.split_layout, L);
    if (rc) { delete p; return rc; }
    rc = plan_upload(p, L);
    if (rc) { sable_plan_destroy(p); return rc; }
    *out = p;
    return SABLE_OK;
}

int sable_plan_dry_run(const sable_vbrc_desc *desc, const sable_plan_opts *opts, sable_plan_stats *out) {
    if (!out) return fail(SABLE_ERR_ARG, "null output pointer");
    const int row_tile = opts && opts->row_tile ? opts->row_tile : SABLE_MAX_ROW_TILE;
    const int chunk_bytes = opts && opts->chunk_bytes ? opts->chunk_bytes
                            : (!opts || opts->schedule == SABLE_SCHEDULE_ITEMS ? SABLE_ITEMS_ITEM_BYTES
                               : opts->schedule == SABLE_SCHEDULE_WARP_ITEMS ? SABLE_WARP_ITEMS_ITEM_BYTES
                                                                             : SABLE_WARP_ITEM_BYTES);
    if (row_tile < 1 || row_tile > SABLE_MAX_ROW_TILE) return fail(SABLE_ERR_ARG, "row_tile %d outside 1..128", row_tile);
    if (chunk_bytes < 4096 || chunk_bytes > SABLE_MAX_ITEM_BYTES * 4 / 5) return fail(SABLE_ERR_ARG, "chunk_bytes outside range");
    int rc = validate_vbrc(desc);
    if (rc) return rc;
    const int split_layout = opts ? opts->split_layout : 0;
    if (split_layout != 0 && split_layout != 1) return fail(SABLE_ERR_ARG, "split_layout %d unknown", split_layout);
    Layout L;
    rc = build_layout(desc, row_tile, chunk_bytes, split_layout, L);
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
