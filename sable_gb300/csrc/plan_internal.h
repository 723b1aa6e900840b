// Host-side plan object shared by the C++ translation units of libsable.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>

#include "sable.h"
#include "sable_internal.h"

namespace sable {

// Host image of a plan's device layout (see sable_internal.h).
struct Layout {
    int32_t n_rows = 0, n_cols = 0;
    std::vector<unsigned char> records;   // item records, 16-byte aligned
    std::vector<ItemRef> items;           // in record order
    std::vector<int64_t> item_tile;       // tile of each item
    int64_t n_tiles = 0, n_partial = 0, dense_values = 0, dense_padded = 0, sparse_nnz = 0;
    int32_t n_split_tiles = 0;
    std::vector<SplitTile> splits;        // split tiles (counter index order)
    int max_item_bytes = 0;
    int max_xg_floats = 0;      // largest 4 nq + ns over items (compact records: largest window)
    bool compact = false;       // records are CompactHeader records (per-warp SpMV executor)
};

int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
int set_device(int dev);
int validate_vbrc(const sable_vbrc_desc *d);
// compact: CompactHeader records for the per-warp SpMV executor (schedule 2).
int build_layout(const sable_vbrc_desc *d, int row_tile, int item_bytes, int split_layout, Layout &L,
                 bool compact = false);
int check_layout(const Layout &L);
int check_compact_layout(const Layout &L);
// Persistent schedule: tiles' items grouped into parts of <= part_bytes,
// parts assigned to n_workers warp workers by greedy LPT (schedule.cpp).
int build_warp_schedule(const Layout &L, int n_workers, int64_t part_bytes, std::vector<WorkRef> &work,
                        std::vector<int> &begin, int64_t &ppartial_floats, int64_t &n_multi, int64_t &n_parts);

}  // namespace sable

struct sable_plan {
    int device = 0;
    int32_t n_rows = 0, n_cols = 0;
    int row_tile = 0, item_bytes = 0, spmm_tc = 0, schedule = 0;
    unsigned char *d_records = nullptr;
    int64_t records_bytes = 0;
    ItemRef *d_items = nullptr;          // item table, largest first
    WorkRef *d_work = nullptr;           // warp-worker lists (persistent schedule)
    int *d_cta_begin = nullptr;          // worker ranges into d_work
    int n_ctas = 0;                      // warp workers of the persistent schedule
    bool compact = false;                // compact records: SpMV through the per-warp executor only
    bool staged_ok = true;               // records fit the shared-memory staging of SpMV and batches
    void *d_tcplanes = nullptr;          // split-BF16 SpMM: pre-split A fragments (16-byte words)
    int64_t *d_tcoff = nullptr;          // word offset of each item's fragments (item-table order)
    std::vector<int64_t> tcoff_host;     // the same on the host (empty: no fragments)
    int64_t tc_words = 0;                // 16-byte words in d_tcplanes
    int tc_kernel = 0;                   // SABLE_TC_KERNEL_UMMA or SABLE_TC_KERNEL_MMASYNC
    unsigned char *d_umma = nullptr;     // split-BF16 SpMM on tcgen05: panel terms, UMMA K-major layout
    int64_t *d_umma_off = nullptr;       // byte offset of each item's terms (item-table order), -1: none
    std::vector<int64_t> umma_off_host;  // the same on the host
    int64_t umma_bytes = 0;
    int umma_hp = 16;                    // tallest tile with a panel, rounded up to 16
    // sable_spmv_host on pinned buffers: the copy of x into the device
    // staging and the SpMV, captured once as a graph for the last (x, y) pair
    cudaGraphExec_t host_exec = nullptr;
    const float *host_x = nullptr;       // mapped x the graph reads
    float *host_y = nullptr;             // mapped y the graph writes
    const float *host_dx = nullptr;      // device staging of x the graph copies into
    float *d_ppartial = nullptr;         // multi-part tile partials
    int *d_pcounters = nullptr;          // multi-part tile counters
    int64_t n_parts = 0, n_multi = 0;
    float *d_partial = nullptr;
    int *d_counters = nullptr;
    SplitTile *d_splits = nullptr;       // SpMV combine table
    std::vector<SplitTile> splits_host;
    int *d_error = nullptr;
    int64_t n_items = 0, n_partial = 0;
    int32_t n_split_tiles = 0;
    int max_item_bytes = 0;
    int max_xg_floats = 0;
    sable_plan_stats stats{};
    std::vector<int64_t> item_tile;      // tile of each item (item table order)
    std::vector<ItemRef> items_host;     // item table (item table order)
    // Split-BF16 tensor-core panels of the dense part (SpMM, built lazily).
    void *tc = nullptr;
    // SpMM scratch, grown on demand by the first call that needs more.
    float *d_spmm_partial = nullptr;
    int64_t spmm_partial_cap = 0;
    int *d_spmm_counters = nullptr;
    int64_t spmm_counters_cap = 0;
    // Device staging of the *_host entry points.
    float *d_x = nullptr, *d_y = nullptr;
    int64_t dx_cap = 0, dy_cap = 0;
};

namespace sable {
int plan_upload(sable_plan *p, const Layout &L);
LaunchArgs spmv_args(const sable_plan *p, const float *x, float *y, int64_t *cycles);
// SpMM launch of a plan at width N (slice width nt); sets the plan's
// tensor-core operands in `a` and picks the kernel as sable_spmm does.
int launch_spmm_plan(const sable_plan *p, LaunchArgs &a, int N, int nt, bool timed, void *stream);
}  // namespace sable
