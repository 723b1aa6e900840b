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
    if (d->n_cols > SABLE_MAX_COLS) return fail(SABLE_ERR_UNSUPPORTED, "n_cols=%d above %d", d->n_cols, SABLE_MAX_COLS);
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
// Plan construction.
// ---------------------------------------------------------------------------
int build_layout(const sable_vbrc_desc *d, int row_tile, int chunk_bytes, Layout &L) {
    std::vector<std::vector<DenseBlock>> rows;
    int rc = collect_dense(d, rows);
    if (rc) return rc;
    L = Layout();
    L.n_rows = d->n_rows;
    L.n_cols = d->n_cols;
    const int64_t sp_chunk = std::max<int64_t>(32, chunk_bytes / 8);
    struct TileWork { int32_t row0, h; int64_t panel_f4, nq, sp0, ns; int32_t run_first; };
    std::vector<TileWork> tiles;
    // Tile-local column runs (one per dense block): panel column start, x column, width.
    struct ColRun { int32_t pc, col, w; };
    std::vector<ColRun> colruns;
    std::vector<int32_t> tile_colrun_begin;

    for (int32_t a = 0; a < d->n_block_rows; ++a) {
        const int32_t r0 = d->rpntr[a], hb = d->rpntr[a + 1] - r0;
        const int32_t nt = (hb + row_tile - 1) / row_tile;
        for (int32_t t = 0; t < nt; ++t) {
            const int32_t lo = (int32_t)((int64_t)hb * t / nt), hi = (int32_t)((int64_t)hb * (t + 1) / nt);
            TileWork tw;
            tw.row0 = r0 + lo;
            tw.h = hi - lo;
            tw.panel_f4 = (int64_t)L.panel.size();
            tw.run_first = (int32_t)colruns.size();
            int32_t W = 0;
            for (const DenseBlock &db : rows[a]) {
                const int32_t w = d->cpntr[db.b + 1] - d->cpntr[db.b];
                colruns.push_back({W, d->cpntr[db.b], w});
                W += w;
            }
            const int64_t nq = (W + 3) / 4;
            tw.nq = nq;
            L.panel.resize(L.panel.size() + (size_t)(nq * tw.h), make_float4(0.f, 0.f, 0.f, 0.f));
            float *P = reinterpret_cast<float *>(L.panel.data() + tw.panel_f4);
            int32_t pc = 0;
            for (const DenseBlock &db : rows[a]) {
                const int32_t w = d->cpntr[db.b + 1] - d->cpntr[db.b];
                const float *blk = d->val + db.off;
                for (int32_t j = 0; j < w; ++j, ++pc) {
                    const int64_t q = pc >> 2, comp = pc & 3;
                    const float *colv = blk + (int64_t)j * hb + lo;
                    float *dst = P + (q * tw.h) * 4 + comp;
                    for (int32_t i = 0; i < tw.h; ++i) dst[(int64_t)i * 4] = colv[i];
                }
                L.dense_values += (int64_t)w * tw.h;
            }
            // CSR entries of the tile's rows
            tw.sp0 = (int64_t)L.sparse.size();
            tw.ns = 0;
            if (d->indptr) {
                for (int32_t i = 0; i < tw.h; ++i) {
                    const int32_t r = tw.row0 + i;
                    for (int64_t k = d->indptr[r]; k < d->indptr[r + 1]; ++k) {
                        uint2 e;
                        float v = d->csr_val[k];
                        memcpy(&e.x, &v, 4);
                        e.y = (uint32_t)d->indices[k] | ((uint32_t)i << SABLE_COL_BITS);
                        L.sparse.push_back(e);
                    }
                }
                tw.ns = (int64_t)L.sparse.size() - tw.sp0;
            }
            tiles.push_back(tw);
            tile_colrun_begin.push_back(tw.run_first);
        }
    }
    tile_colrun_begin.push_back((int32_t)colruns.size());
    L.n_tiles = (int64_t)tiles.size();

    // Work items.
    int64_t part_floats = 0;
    int32_t split_tiles = 0;
    std::vector<std::pair<int64_t, Chunk>> work;  // (bytes, chunk)
    for (size_t ti = 0; ti < tiles.size(); ++ti) {
        const TileWork &tw = tiles[ti];
        const int32_t cr0 = tile_colrun_begin[ti], cr1 = tile_colrun_begin[ti + 1];
        const int64_t dense_bytes = 16 * tw.nq * tw.h, sp_bytes = 8 * tw.ns;
        // dense pieces: [q0, q1) quads
        std::vector<std::pair<int64_t, int64_t>> dpieces;
        const int64_t qcap = std::max<int64_t>(1, std::min<int64_t>(SABLE_MAX_CHUNK_QUADS, chunk_bytes / (16 * tw.h)));
        bool single = (dense_bytes + sp_bytes) <= (chunk_bytes + chunk_bytes / 4) && tw.nq <= SABLE_MAX_CHUNK_QUADS &&
                      tw.ns <= INT32_MAX && (cr1 - cr0) <= SABLE_MAX_CHUNK_RUNS;
        if (single) {
            dpieces.push_back({0, tw.nq});
        } else {
            int64_t q0 = 0;
            int32_t r = cr0;
            while (q0 < tw.nq) {
                int64_t q1 = std::min(tw.nq, q0 + qcap);
                // keep the number of column runs of the piece within the table size
                while (r < cr1 && colruns[r].pc + colruns[r].w <= 4 * q0) ++r;
                int32_t rr = r, nrun = 0;
                while (rr < cr1 && colruns[rr].pc < 4 * q1) {
                    if (++nrun > SABLE_MAX_CHUNK_RUNS) { q1 = std::max<int64_t>(q0 + 1, colruns[rr].pc / 4); break; }
                    ++rr;
                }
                dpieces.push_back({q0, q1});
                q0 = q1;
            }
        }
        std::vector<std::pair<int64_t, int64_t>> spieces;
        if (single) {
            if (tw.ns > 0) spieces.push_back({0, tw.ns});
        } else {
            for (int64_t s0 = 0; s0 < tw.ns; s0 += sp_chunk) spieces.push_back({s0, std::min(tw.ns, s0 + sp_chunk)});
        }
        int32_t nchunk = single ? 1 : (int32_t)(dpieces.size() + spieces.size());
        if (nchunk == 0) nchunk = 1;  // zero tile (no stored blocks): writes zeros
        if (single && dpieces.empty()) dpieces.push_back({0, 0});
        const int32_t split_id = nchunk > 1 ? split_tiles++ : -1;
        const int64_t pbase = nchunk > 1 ? part_floats : 0;
        if (nchunk > 1) part_floats += (int64_t)nchunk * tw.h;
        int32_t kidx = 0;
        auto emit = [&](int64_t q0, int64_t q1, int64_t s0, int64_t s1) {
            Chunk c;
            memset(&c, 0, sizeof c);
            c.panel_f4 = tw.panel_f4 + q0 * tw.h;
            c.sp0 = tw.sp0 + s0;
            c.part_base = pbase;
            c.row0 = tw.row0;
            c.h = tw.h;
            c.nq = (int32_t)(q1 - q0);
            c.ns = (int32_t)(s1 - s0);
            c.run0 = (int32_t)L.runs.size();
            for (int32_t r = cr0; r < cr1 && c.nq > 0; ++r) {
                const int64_t a0 = std::max<int64_t>(colruns[r].pc, 4 * q0);
                const int64_t a1 = std::min<int64_t>(colruns[r].pc + colruns[r].w, 4 * q1);
                if (a0 >= a1) continue;
                L.runs.push_back(make_int4((int)(a0 - 4 * q0), (int)(colruns[r].col + (a0 - colruns[r].pc)), (int)(a1 - a0), 0));
            }
            c.nrun = (int32_t)L.runs.size() - c.run0;
            c.tile = split_id;
            c.kidx = kidx++;
            c.nchunk = nchunk;
            L.max_quads = std::max<int>(L.max_quads, c.nq);
            L.max_runs = std::max<int>(L.max_runs, c.nrun);
            const int64_t bytes = 16 * (int64_t)c.nq * c.h + 8 * (int64_t)c.ns;
            work.push_back({bytes, c});
            L.chunk_tile.push_back((int64_t)ti);
        };
        if (single) {
            emit(dpieces[0].first, dpieces[0].second, spieces.empty() ? 0 : spieces[0].first,
                 spieces.empty() ? 0 : spieces[0].second);
        } else {
            for (auto &p : dpieces) emit(p.first, p.second, 0, 0);
            for (auto &p : spieces) emit(0, 0, p.first, p.second);
        }
    }
    // Largest work first (the hardware scheduler then behaves like greedy LPT).
    std::vector<size_t> order(work.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return work[x].first > work[y].first; });
    L.chunks.resize(work.size());
    std::vector<int64_t> ct(work.size());
    for (size_t i = 0; i < order.size(); ++i) {
        L.chunks[i] = work[order[i]].second;
        ct[i] = L.chunk_tile[order[i]];
    }
    L.chunk_tile.swap(ct);
    L.n_partial = part_floats;
    L.n_split_tiles = split_tiles;
    L.sparse_nnz = (int64_t)L.sparse.size();
    return check_layout(L);
}

// Every index a kernel will follow, checked on the host before upload.
int check_layout(const Layout &L) {
    const int64_t npanel = (int64_t)L.panel.size(), nsp = (int64_t)L.sparse.size(), nruns = (int64_t)L.runs.size();
    for (size_t k = 0; k < L.chunks.size(); ++k) {
        const Chunk &c = L.chunks[k];
        if (c.h < 1 || c.h > SABLE_MAX_ROW_TILE || c.row0 < 0 || c.row0 + c.h > L.n_rows)
            return fail(SABLE_ERR_INVALID, "layout: chunk %zu rows out of range", k);
        if (c.nq < 0 || c.nq > SABLE_MAX_CHUNK_QUADS || c.panel_f4 < 0 || c.panel_f4 + (int64_t)c.nq * c.h > npanel)
            return fail(SABLE_ERR_INVALID, "layout: chunk %zu panel range out of bounds", k);
        if (c.ns < 0 || c.sp0 < 0 || c.sp0 + c.ns > nsp) return fail(SABLE_ERR_INVALID, "layout: chunk %zu sparse range", k);
        if (c.nrun < 0 || c.nrun > SABLE_MAX_CHUNK_RUNS || c.run0 < 0 || c.run0 + c.nrun > nruns)
            return fail(SABLE_ERR_INVALID, "layout: chunk %zu run range", k);
        if (c.nq > 0 && c.nrun == 0) return fail(SABLE_ERR_INVALID, "layout: chunk %zu has quads but no runs", k);
        for (int r = 0; r < c.nrun; ++r) {
            const int4 run = L.runs[c.run0 + r];
            if (run.x < 0 || run.z < 1 || run.x + run.z > 4 * c.nq || run.y < 0 || run.y + run.z > L.n_cols ||
                (r > 0 && run.x < L.runs[c.run0 + r - 1].x + L.runs[c.run0 + r - 1].z))
                return fail(SABLE_ERR_INVALID, "layout: chunk %zu run %d out of bounds", k, r);
        }
        for (int64_t e = c.sp0; e < c.sp0 + c.ns; ++e) {
            const uint32_t col = L.sparse[e].y & SABLE_COL_MASK, lrow = L.sparse[e].y >> SABLE_COL_BITS;
            if ((int64_t)col >= L.n_cols || (int)lrow >= c.h) return fail(SABLE_ERR_INVALID, "layout: sparse entry %lld", (long long)e);
        }
        if (c.nchunk < 1 || c.kidx < 0 || c.kidx >= c.nchunk) return fail(SABLE_ERR_INVALID, "layout: chunk %zu numbering", k);
        if (c.nchunk > 1 && (c.tile < 0 || c.tile >= L.n_split_tiles || c.part_base < 0 ||
                             c.part_base + (int64_t)c.nchunk * c.h > L.n_partial))
            return fail(SABLE_ERR_INVALID, "layout: chunk %zu split-tile scratch out of bounds", k);
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
    const int chunk_bytes = o.chunk_bytes ? o.chunk_bytes : 32768;
    if (row_tile < 1 || row_tile > SABLE_MAX_ROW_TILE) return fail(SABLE_ERR_ARG, "row_tile %d outside 1..128", row_tile);
    if (chunk_bytes < 256 || chunk_bytes > (64 << 20)) return fail(SABLE_ERR_ARG, "chunk_bytes %d outside 256..64M", chunk_bytes);
    int rc = validate_vbrc(desc);
    if (rc) return rc;
    rc = set_device(o.device);
    if (rc) return rc;
    sable_plan *p = new (std::nothrow) sable_plan();
    if (!p) return fail(SABLE_ERR_NOMEM, "host allocation");
    cudaGetDevice(&p->device);
    p->row_tile = row_tile;
    p->chunk_bytes = chunk_bytes;
    p->spmm_tc = o.spmm_tc;
    Layout L;
    rc = build_layout(desc, row_tile, chunk_bytes, L);
    if (rc) { delete p; return rc; }
    rc = plan_upload(p, L);
    if (rc) { sable_plan_destroy(p); return rc; }
    *out = p;
    return SABLE_OK;
}

int sable_plan_dry_run(const sable_vbrc_desc *desc, const sable_plan_opts *opts, sable_plan_stats *out) {
    if (!out) return fail(SABLE_ERR_ARG, "null output pointer");
    const int row_tile = opts && opts->row_tile ? opts->row_tile : SABLE_MAX_ROW_TILE;
    const int chunk_bytes = opts && opts->chunk_bytes ? opts->chunk_bytes : 32768;
    if (row_tile < 1 || row_tile > SABLE_MAX_ROW_TILE) return fail(SABLE_ERR_ARG, "row_tile %d outside 1..128", row_tile);
    if (chunk_bytes < 256 || chunk_bytes > (64 << 20)) return fail(SABLE_ERR_ARG, "chunk_bytes outside 256..64M");
    int rc = validate_vbrc(desc);
    if (rc) return rc;
    Layout L;
    rc = build_layout(desc, row_tile, chunk_bytes, L);
    if (rc) return rc;
    memset(out, 0, sizeof *out);
    out->n_tiles = L.n_tiles;
    out->n_chunks = (int64_t)L.chunks.size();
    out->dense_values = L.dense_values;
    out->dense_padded = (int64_t)L.panel.size() * 4;
    out->sparse_nnz = L.sparse_nnz;
    out->device_bytes = (int64_t)(L.panel.size() * 16 + L.sparse.size() * 8 + L.runs.size() * 16 +
                                  L.chunks.size() * sizeof(Chunk) + (L.n_partial + L.n_split_tiles) * 4);
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
    memcpy(tile_of_chunk, plan->chunk_tile.data(), plan->chunk_tile.size() * sizeof(int64_t));
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
