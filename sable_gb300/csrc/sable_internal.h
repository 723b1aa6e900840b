// Internal layout shared by the host plan builder and the device kernels.
//
// Device layout of one plan (HBM, built once by sable_plan_create):
//
//   tiles     A block row of height <= row_tile is one tile; a taller block
//             row is cut into near-equal tiles.  Empty block rows become
//             zero tiles so that every output row is written by exactly one
//             tile (no memset of y is ever needed).
//   items     A tile's work is cut into items of at most ~item_bytes.  Each
//             item is one contiguous, 16-byte aligned record:
//
//               ItemHeader                       64 bytes
//               xcol   int32[4*nq]               x column of each panel column
//               panel  float4[nq*h]              quad panel: (q, i) = A[i, 4q..4q+3]
//               rowptr int32[h+1] (16 B padded)  CSR row starts, item-relative
//               csr    uint2[ns]  (16 B padded)  (value bits, column)
//
//             The dense blocks of a tile are concatenated column by column
//             (bindx order) and padded to a multiple of 4 columns; a panel
//             quad holds 4 columns of one row, so consecutive threads read
//             consecutive 16-byte words while every thread keeps its row.
//             One TMA bulk copy brings a whole item into shared memory.
//             Plans of the per-warp SpMV executor (schedule 2) hold compact
//             records instead (CompactHeader below), on tiles of at most
//             SABLE_CW_MAX_ROWS rows: x is addressed through a per-item
//             window of at most SABLE_CW_MAX positions given as column runs,
//             and every CSR entry stores its window position and its row:
//
//               CompactHeader                    64 bytes
//               runs   int2[nrun]  (16 B padded) (first x column, length); column -1: zeros
//               panel  float4[nq*h]              as above; window positions [0, 4nq)
//               val    float[ns]  (8-entry padded)  CSR values, row-major
//               meta   uint16[ns] (8-entry padded)  window position | tile row << 10
//
//             Window positions [0, 4nq) are the panel columns, [4nq, nw) the
//             columns of the item's CSR entries (sorted, runs closer than
//             SABLE_CW_GAP columns merged).  A warp gathers the window into
//             shared memory once per item with coalesced loads.
//   table     int64 offset / bytes of each item, and per persistent CTA the
//             [begin, end) range of its items (greedy LPT over item bytes).
//   Split tiles publish per-item partial row sums; the last-arriving CTA
//   adds them in item order (deterministic, no atomics on y).
#pragma once
#include <stddef.h>
#include <stdint.h>

#define SABLE_MAX_ROW_TILE 128
#define SABLE_THREADS 256
#define SABLE_NWARP (SABLE_THREADS / 32)
#define SABLE_MAX_ITEM_BYTES 98304   // record bytes the SpMV / batch executors stage in shared memory
#define SABLE_MAX_RECORD_BYTES (1 << 22)  // any record (SpMM streams records in K steps)
#define SABLE_MAX_CHUNK_BYTES (1 << 20)   // chunk_bytes of one-CTA-per-item plans (larger items: SpMM only)
#define SABLE_WSTAGES 2              // TMA ring depth of a persistent warp worker
#define SABLE_ITEMS_ITEM_BYTES 32768 // default item size, one CTA per item
#define SABLE_WARP_ITEM_BYTES 8192   // default item size, warp workers
#define SABLE_SCHEDULE_ITEMS 0
#define SABLE_SCHEDULE_PERSISTENT 1
#define SABLE_SCHEDULE_WARP_ITEMS 2
#define SABLE_WARP_ITEMS_ITEM_BYTES 32768  // default item size, one warp per compact item

struct __align__(16) ItemHeader {
    int32_t row0;       // first output row of the tile
    int32_t h;          // rows of the tile
    int32_t nq;         // panel quads in this item
    int32_t ns;         // CSR entries in this item
    int32_t xcol_off;   // byte offsets of the record's parts
    int32_t panel_off;
    int32_t rp_off;
    int32_t csr_off;
    int32_t tile;       // split-tile counter index, -1 for a single-item tile
    int32_t kidx;       // position of the item within its tile
    int32_t nitem;      // items of the tile
    int32_t g;          // lanes per CSR row (4, 8, 16 or 32)
    int64_t part_base;  // float offset of the tile's partial slots (split tiles)
    int32_t bytes;      // record bytes (multiple of 16)
    int32_t mat;        // matrix index inside a batch (0 for a single plan)
};
static_assert(sizeof(ItemHeader) == 64, "ItemHeader must stay 64 bytes");

#define SABLE_CW_MAX 1024     // window positions of a compact record (x floats a warp stages; 10 bits)
#define SABLE_CW_MAX_ROWS 64  // rows of a compact tile (6 bits of a CSR entry's meta word)
#define SABLE_CW_GAP 8        // CSR column runs closer than this share one window run

// Header of a compact record.  Every field an ItemHeader also has sits at the
// same offset, so the host code that reads tile / split fields reads both.
struct __align__(16) CompactHeader {
    int32_t row0, h, nq, ns;
    int32_t runs_off;   // byte offsets of the record's parts
    int32_t panel_off;
    int32_t rp_off;     // = val_off (no row pointers: each entry carries its row)
    int32_t val_off;
    int32_t tile, kidx, nitem;
    int32_t meta_off;
    int64_t part_base;
    int32_t bytes;
    int16_t nrun;       // window runs
    int16_t nw;         // window positions (<= SABLE_CW_MAX)
};
static_assert(sizeof(CompactHeader) == 64, "CompactHeader must stay 64 bytes");
static_assert(offsetof(CompactHeader, h) == offsetof(ItemHeader, h) &&
                  offsetof(CompactHeader, panel_off) == offsetof(ItemHeader, panel_off) &&
                  offsetof(CompactHeader, rp_off) == offsetof(ItemHeader, rp_off) &&
                  offsetof(CompactHeader, tile) == offsetof(ItemHeader, tile) &&
                  offsetof(CompactHeader, nitem) == offsetof(ItemHeader, nitem) &&
                  offsetof(CompactHeader, part_base) == offsetof(ItemHeader, part_base) &&
                  offsetof(CompactHeader, bytes) == offsetof(ItemHeader, bytes),
              "CompactHeader shares ItemHeader's field offsets");

struct ItemRef {        // item table entry
    int64_t off;        // byte offset of the record
    int32_t bytes;      // record bytes
    int32_t cost;       // scheduling weight (bytes or SpMM work)
};

// Entry of a warp worker's list (persistent schedule).  Consecutive items of
// one tile form a part; a warp accumulates over the items of a part in
// registers and writes the rows once, at the part's last item.
#define SABLE_PART_FIRST 1
#define SABLE_PART_LAST 2
struct WorkRef {
    int64_t off;        // byte offset of the record
    int64_t part_base;  // float offset of the tile's part partials (multi-part tiles)
    int32_t bytes;      // record bytes
    int32_t flags;      // SABLE_PART_FIRST / SABLE_PART_LAST
    int32_t part;       // index of the part within its tile
    int32_t nparts;     // parts of the tile
    int32_t split;      // counter index of a multi-part tile, -1 otherwise
    int32_t pad[3];
};
static_assert(sizeof(WorkRef) == 48, "WorkRef must stay 48 bytes");

// A tile cut into several SpMV items.  Its items store per-item row sums in
// the matrix's partial buffer ([part_base + k h, +h) for item k); a separate
// combine launch adds them in item order and writes y.
struct SplitTile {
    int64_t part_base;
    int32_t row0, h, nitem, mat;
};
static_assert(sizeof(SplitTile) == 24, "SplitTile must stay 24 bytes");

// One matrix of a launch: its operand / result and (SpMM) width.
struct MatIO {
    const float *x;
    float *y;
    float *partial;     // split-tile partial sums of this matrix (per item)
    int *counters;      // split-tile arrival counters (self-resetting)
    float *ppartial;    // multi-part tile partial sums (persistent schedule)
    int *pcounters;     // multi-part tile arrival counters (self-resetting)
    int64_t ldx, ldy;
    int32_t N;          // 1 for SpMV
    int32_t pad;        // SpMM: split-tile counters per N-slice
    int64_t part_stride;  // SpMM: partial floats per N-slice (batch kernel)
};

struct LaunchArgs {
    const unsigned char *records;
    const ItemRef *items;
    const WorkRef *work;    // persistent: worker lists, concatenated
    const int *cta_begin;   // persistent: worker w's entries are [cta_begin[w], cta_begin[w+1])
    const MatIO *mats;      // per matrix (batch); nullptr: every item uses mat0
    const int32_t *item_mat;  // per-warp SpMV of a batch: matrix of each item (compact headers carry none)
    MatIO mat0;
    int64_t *cycles;        // per-item SM cycles (timed variant) or nullptr
    const void *tcplanes;   // SpMM split-BF16: pre-split A fragments (uint4 words) or nullptr
    const int64_t *tcoff;   // word offset of each item's fragments in tcplanes (item-table order)
    const unsigned char *umma;    // SpMM split-BF16 on tcgen05: panel terms in the UMMA K-major layout
    const int64_t *umma_off;      // byte offset of each item's terms in umma (item-table order), -1: none
    int umma_hp;                  // tallest tile with a panel, rounded up to 16 (sizes the panel ring)
    int *error;             // set to 1 when a bounded device wait runs out
    int n_items;
    int stage_bytes;        // TMA staging bytes per stage (>= largest record)
    int xg_floats;          // x-gather buffer floats (>= 4 nq + ns of any item)
};

namespace sable {
// Width of one SpMM N-slice (one CTA per item and slice): the smallest power
// of two from 4 to 128 that covers N.  The split-tile scratch of an SpMM call
// holds n_partial * nt floats per slice, so every entry point that sizes that
// scratch uses this one function.
inline int spmm_slice_width(int N) {
    int nt = 4;
    while (nt < N && nt < 128) nt <<= 1;
    return nt;
}
int launch_spmv_items(const LaunchArgs &a, bool timed, void *stream);
int launch_spmv_warp_items(const LaunchArgs &a, bool timed, void *stream);
// y rows of split tiles from their items' partial sums (after the items ran).
int launch_spmv_combine(const SplitTile *tiles, int n_tiles, const MatIO *mats, const MatIO &mat0, void *stream);
// dst[0, n) = src[0, n) by a kernel (either side may be mapped host memory).
int launch_copy_floats(float *dst, const float *src, int64_t n, void *stream);
int launch_spmv_warps(const LaunchArgs &a, int n_workers, void *stream);
int spmv_items_smem(int stage_bytes, int xg_floats);
int spmv_warp_smem(int stage_bytes, int xg_floats);
int spmv_warp_workers_per_sm(int stage_bytes, int xg_floats);
int launch_spmm_fp32(const LaunchArgs &a, int N, int nt, int64_t part_stride, bool timed, void *stream);
// terms = 2: three BF16 products (hi+lo split); 3: six products (hi+mid+lo).
int launch_spmm_tc(const LaunchArgs &a, int N, int nt, int terms, int64_t part_stride, bool timed, void *stream);
// The same product on the tcgen05 tensor cores (TMEM accumulators); nt 32..128.
int launch_spmm_umma(const LaunchArgs &a, int N, int nt, int terms, int64_t part_stride, bool timed, void *stream);
const char *cuda_error_string(int err);
}  // namespace sable
