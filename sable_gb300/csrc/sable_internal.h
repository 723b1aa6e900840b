// Internal layout shared by the host plan builder and the device kernels.
//
// Device layout of one plan (all in HBM, built once by sable_plan_create):
//
//   tiles     A block row of height <= row_tile is one tile; a taller block
//             row is cut into near-equal tiles.  Empty block rows become
//             zero tiles so that every output row is written by exactly one
//             tile (no memset of y is ever needed).
//   panel     float4[]  For each tile, the columns of its dense blocks (bindx
//             order) are concatenated and padded to a multiple of 4; element
//             (q, i) = A[i, 4q .. 4q+3] of quad q, row i, stored at q*h + i.
//             A tile's panel is therefore one contiguous float4 stream in
//             which consecutive threads read consecutive 16-byte words while
//             every thread keeps a fixed row.
//   sparse    uint2[]   The CSR entries of the tile's rows, in CSR order:
//             .x = value bits, .y = column | local_row << 25.  8 bytes per
//             nonzero, no row pointer array.
//   runs      int4[]    x gather runs of a work item: (dst, col0, len, 0):
//             xs[dst + k] = x[col0 + k] for k < len.
//   chunks    Chunk[]   Work items of at most ~chunk_bytes of matrix data;
//             a tile split over several chunks reduces its partial sums in a
//             fixed order in the last-arriving CTA (deterministic).
#pragma once
#include <stdint.h>

#define SABLE_MAX_ROW_TILE 128
#define SABLE_COL_BITS 25
#define SABLE_COL_MASK ((1u << SABLE_COL_BITS) - 1u)
#define SABLE_MAX_COLS (1 << SABLE_COL_BITS)
#define SABLE_MAX_CHUNK_QUADS 1024   // xs staging: 16 KB of shared memory
#define SABLE_MAX_CHUNK_RUNS 256     // run table: 4 KB of shared memory
#define SABLE_THREADS 256
#define SABLE_VT 4                   // virtual row-threads per thread (dense SpMV)

struct __align__(16) Chunk {
    int64_t panel_f4;   // float4 index of the chunk's first panel word
    int64_t sp0;        // first sparse entry
    int64_t part_base;  // float offset of the tile's partial slots (split tiles)
    int32_t row0;       // first output row of the tile
    int32_t h;          // rows of the tile
    int32_t nq;         // dense quads in this chunk
    int32_t ns;         // sparse entries in this chunk
    int32_t run0;       // first x run
    int32_t nrun;       // x runs
    int32_t tile;       // split-tile counter index, -1 for a single-chunk tile
    int32_t kidx;       // position of the chunk within its tile
    int32_t nchunk;     // chunks of the tile
    int32_t pad;
};
static_assert(sizeof(Chunk) == 64, "Chunk must stay 64 bytes");

struct SpmvArgs {
    const Chunk *chunks;
    const float4 *panel;
    const uint2 *sparse;
    const int4 *runs;
    const float *x;
    float *y;
    float *partial;     // split-tile partial sums
    int *counters;      // split-tile arrival counters (self-resetting)
    int64_t *ns_out;    // per-chunk durations (timed variant) or nullptr
    int n_chunks;
    int *work_counter;  // persistent variant: next chunk to take (self-resetting)
    int *done_counter;  // persistent variant: CTAs finished (self-resetting)
};

struct SpmmArgs {
    const Chunk *chunks;
    const float4 *panel;
    const uint2 *sparse;
    const int4 *runs;
    const float *X;
    float *Y;
    float *partial;
    int *counters;
    int64_t *ns_out;
    int64_t ldx, ldy;
    int N;              // total width
    int nt;             // width handled by one work item (power of two, <= 128)
    int n_slices;       // ceil(N / nt)
    int n_chunks;
    int64_t part_stride; // floats of partial scratch per N-slice
};

// Host-side launchers implemented in the .cu files.
namespace sable {
int launch_spmv(const SpmvArgs &a, int smem_bytes, bool timed, void *stream);
int launch_spmm_fp32(const SpmmArgs &a, int smem_bytes, bool timed, void *stream);
int spmv_smem_bytes(int max_quads, int max_runs);
int spmm_smem_bytes(int nt, int max_quads, int max_runs, int row_tile);
const char *cuda_error_string(int err);
}  // namespace sable
