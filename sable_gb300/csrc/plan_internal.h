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
    std::vector<float4> panel;
    std::vector<uint2> sparse;
    std::vector<int4> runs;
    std::vector<Chunk> chunks;
    std::vector<int64_t> chunk_tile;
    int64_t n_tiles = 0, n_partial = 0, dense_values = 0, sparse_nnz = 0;
    int32_t n_split_tiles = 0;
    int max_quads = 0, max_runs = 0;
};

int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
int set_device(int dev);
int validate_vbrc(const sable_vbrc_desc *d);
int build_layout(const sable_vbrc_desc *d, int row_tile, int chunk_bytes, Layout &L);
int check_layout(const Layout &L);

}  // namespace sable

struct sable_plan {
    int device = 0;
    int32_t n_rows = 0, n_cols = 0;
    int row_tile = 0, chunk_bytes = 0, spmm_tc = 0;
    float4 *d_panel = nullptr;
    uint2 *d_sparse = nullptr;
    int4 *d_runs = nullptr;
    Chunk *d_chunks = nullptr;
    float *d_partial = nullptr;
    int *d_counters = nullptr;
    int64_t n_chunks = 0, n_partial = 0;
    int32_t n_split_tiles = 0;
    int max_quads = 0, max_runs = 0;
    sable_plan_stats stats{};
    std::vector<int64_t> chunk_tile;
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
SpmvArgs spmv_args(const sable_plan *p, const float *x, float *y, int64_t *cycles);
}  // namespace sable
