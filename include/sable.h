/*
 * sable.h — C ABI of the GB300 VBR SpMV/SpMM library (libsable.so).
 *
 * The reference (reikdas/SABLE) has no library boundary: its Python code
 * generator writes one C program per matrix, which reads the matrix and the
 * dense operand from text files and prints y (src/codegen.py:293-452 SpMV,
 * :827-937 SpMM).  The entry points below replace that generated executable.
 * A plan is the GPU counterpart of one generated program: it is built once
 * from the VBR arrays (the inspector step) and then executed many times.
 *
 * Conventions
 *   - Every function returns SABLE_OK (0) or a negative SABLE_ERR_* code;
 *     sable_strerror() gives its text, sable_last_error() the detail of the
 *     most recent failure on the calling thread.
 *   - Device pointers (`*_dev`) are CUDA global-memory pointers owned by the
 *     caller.  The plan owns its own device copy of the matrix.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     All device work is stream-ordered; nothing synchronises the device
 *     except the *_host entry points, which synchronise `stream`.
 *   - A plan may be used from one host thread at a time.
 *   - Values are FP32 on the device.  Index arrays are int32 except block
 *     value offsets (indx) and CSR row pointers (indptr), which are int64.
 */
#ifndef SABLE_H
#define SABLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SABLE_OK               0
#define SABLE_ERR_INVALID     -1  /* inconsistent VBR / CSR arrays            */
#define SABLE_ERR_CUDA        -2  /* a CUDA runtime call failed               */
#define SABLE_ERR_NOMEM       -3  /* host or device allocation failed         */
#define SABLE_ERR_UNSUPPORTED -4  /* valid input outside the supported range  */
#define SABLE_ERR_TIMEOUT     -5  /* a bounded device-side wait ran out       */
#define SABLE_ERR_ARG         -6  /* null pointer, bad size or bad option     */

typedef struct sable_plan  sable_plan;
typedef struct sable_batch sable_batch;
typedef struct sable_mlp   sable_mlp;

/*
 * A VBR matrix in the reference's compressed (.vbrc) form
 * (utils/convert_real_to_vbr.py:18-96, read back by utils/fileio.py:66-93):
 *   rpntr[n_block_rows+1], cpntr[n_block_cols+1]  partition bounds
 *   bpntrb/bpntre[n_block_rows]   [begin,end) into bindx, -1 = empty row
 *   bindx[n_blocks]               block column of every stored block,
 *                                 block-row-major, ascending within a row
 *   val, indx[n_dense+1]          values of the blocks kept dense, each
 *                                 column-major h x w, in bindx order
 *   ublocks[n_ublocks]            ascending ordinals (over bindx) of the
 *                                 blocks moved to the CSR part
 *   indptr[n_rows+1], indices, csr_val   global CSR of those blocks
 * An uncompressed .vbr matrix is the case n_ublocks = 0, n_dense = n_blocks,
 * indptr = NULL.
 */
typedef struct sable_vbrc_desc {
    int32_t n_rows, n_cols, n_block_rows, n_block_cols;
    const int32_t *rpntr, *cpntr, *bpntrb, *bpntre, *bindx;
    int64_t n_blocks;
    const float   *val;
    const int64_t *indx;
    int64_t n_dense;
    const int32_t *ublocks;
    int64_t n_ublocks;
    const int64_t *indptr;
    const int32_t *indices;
    const float   *csr_val;
} sable_vbrc_desc;

/* Plan layout options; zero-initialise for defaults. */
typedef struct sable_plan_opts {
    int32_t row_tile;     /* rows per tile, 1..128 (0: 128; schedule 2 caps
                             tiles at 64 rows)                                 */
    int32_t chunk_bytes;  /* target matrix bytes per work item, 4096..78643
                             (0: 32768; 8192 for schedule 1);
                             schedule 0 takes up to 1048576: a plan whose
                             items exceed 98304 bytes is an SpMM-only plan
                             (long K loops, no split tiles): SpMV and batches
                             return SABLE_ERR_UNSUPPORTED for it               */
    int32_t spmm_tc;      /* dense blocks of SpMM with N >= 32 on the tensor
                             cores as split BF16 with FP32 accumulation:
                             SABLE_TC_SPLIT2 (1): hi+lo, three products,
                               per-product error <= 3*2^-16 |a||b|;
                             SABLE_TC_SPLIT3 (2): hi+mid+lo, six products,
                               FP32-level error.  0: FP32 CUDA cores.          */
    int32_t device;       /* CUDA device ordinal (-1: current)                 */
    int32_t schedule;     /* 0: one CTA per work item (TMA-staged record);
                             1: persistent warp workers over an LPT schedule
                             of tile parts, each with a private TMA ring;
                             2: one warp per work item over compact records
                             (x columns as runs, CSR entries of 6 bytes),
                             read with coalesced loads, no CTA barrier; an
                             SpMV-only plan: SpMM, the no-allocation SpMM and
                             batches return SABLE_ERR_UNSUPPORTED for it    */
    int32_t split_layout; /* a row tile larger than one work item is cut into
                             0: items that each take a share of the tile's
                                dense quads and of its CSR entries (SpMV runs
                                both parts on separate warps side by side);
                             1: dense items, then CSR items (better for SpMM,
                                whose CTAs run the two parts one after the
                                other)                                         */
    int32_t tc_kernel;    /* split-BF16 SpMM kernel (plans with spmm_tc):
                             0: tcgen05 MMAs with TMEM accumulators (default);
                             1: mma.sync (the warp-level tensor-core path)     */
} sable_plan_opts;

#define SABLE_TC_KERNEL_UMMA    0
#define SABLE_TC_KERNEL_MMASYNC 1

#define SABLE_TC_OFF    0
#define SABLE_TC_SPLIT2 1
#define SABLE_TC_SPLIT3 2

/* Sizes of a built plan (for byte accounting and tests). */
typedef struct sable_plan_stats {
    int64_t n_tiles, n_chunks;
    int64_t dense_values;     /* stored dense values (padding excluded)       */
    int64_t dense_padded;     /* float slots in the dense panels              */
    int64_t sparse_nnz;       /* entries in the CSR segments                  */
    int64_t device_bytes;     /* device memory held by the plan               */
    int64_t scratch_floats;   /* partial-sum scratch used by split tiles      */
} sable_plan_stats;

/* Inspector: replaces vbr_spmv_codegen / gen_single_threaded_spmv
 * (src/codegen.py:1438-1447, 293-452) — validates the arrays, lays the
 * matrix out for the GPU and uploads it. */
int sable_plan_create(const sable_vbrc_desc *desc, const sable_plan_opts *opts, sable_plan **out);
int sable_plan_destroy(sable_plan *plan);
int sable_plan_get_stats(const sable_plan *plan, sable_plan_stats *out);
/* Host-only inspector run: validates the arrays, builds and bounds-checks
 * the device layout, and reports its sizes without touching the GPU. */
int sable_plan_dry_run(const sable_vbrc_desc *desc, const sable_plan_opts *opts, sable_plan_stats *out);

/* Host-only layout build (no CUDA; no counterpart in the reference, whose
 * inspector emits C instead): the work-item records exactly as a plan of
 * these options uploads them, and each item's record offset and bytes in
 * record order.  With records == NULL only *records_bytes and *n_items are
 * set; SABLE_ERR_ARG when the buffers are smaller than the layout.  Lets
 * host code check a layout (the record formats are in sable_internal.h). */
int sable_plan_layout_host(const sable_vbrc_desc *desc, const sable_plan_opts *opts, unsigned char *records,
                           int64_t records_cap, int64_t *records_bytes, int64_t *item_off, int32_t *item_bytes,
                           int64_t items_cap, int64_t *n_items);

/* Executor, SpMV: y = A x (replaces the timed loop of the generated program,
 * src/codegen.py:414-439).  x has n_cols floats, y n_rows floats. */
int sable_spmv(sable_plan *plan, const float *x_dev, float *y_dev, void *stream);

/* Synchronises `stream` and reports SABLE_ERR_TIMEOUT (then clears the flag)
 * if a bounded device-side wait of an earlier launch of this plan ran out. */
int sable_plan_check(sable_plan *plan, void *stream);

/* Same, from host buffers: copies x in, runs, copies y out, synchronises.
 * Pinned (page-locked) buffers are read and written by the kernels
 * themselves; pageable ones are copied with cudaMemcpyAsync through the
 * plan's device staging buffers. */
int sable_spmv_host(sable_plan *plan, const float *x_host, float *y_host, void *stream);

/* Executor, SpMM: Y = A X with X row-major n_cols x N (leading dimension
 * ldx), Y row-major n_rows x N (ldy).  Replaces gen_single_threaded_spmm
 * (src/codegen.py:827-937), whose width is the literal 512.
 * Requires N % 4 == 0, ldx % 4 == 0, ldy % 4 == 0, 16-byte aligned X and Y. */
int sable_spmm(sable_plan *plan, const float *X_dev, int64_t ldx, float *Y_dev, int64_t ldy,
               int32_t N, void *stream);
int sable_spmm_host(sable_plan *plan, const float *X_host, float *Y_host, int32_t N, void *stream);

/* SpMM that allocates no memory (no counterpart in the reference).
 * Same arguments, kernels and result as sable_spmm (split BF16 on the tensor
 * cores for plans built with spmm_tc at N >= 32, FP32 otherwise), for callers
 * that cannot let a library allocate device memory during a call: runtimes
 * whose pool allocator owns all device memory and forbids later cudaMalloc,
 * and real-time loops that must not block on the driver's allocator.
 * sable_spmm allocates split-tile scratch on its first call at a given width;
 * this entry point uses a fixed scratch array compiled into the library
 * instead (8 MiB of partial sums + 256 KiB of counters, held by every device
 * that loads the library until the process exits) and returns
 * SABLE_ERR_UNSUPPORTED when a plan at width N needs more than that.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), which also loads the library's device code on that
 * device if it is not loaded yet and so reserves the array: make that first
 * call before any stream capture, and before a pool allocator takes the
 * whole device.  All calls share the one array and each call clears its
 * counters first: calls that may overlap on the GPU (other streams, other
 * host threads) race and must be serialised by the caller. */
int sable_spmm_noalloc(sable_plan *plan, const float *X_dev, int64_t ldx, float *Y_dev, int64_t ldy,
                       int32_t N, void *stream);

/* Per-work-item device time (SM clock cycles) of one SpMV / SpMM launch
 * (SpMV: one CTA per item, or one warp per item for plans of schedule 2),
 * written to cycles_dev[n_chunks] (SpMM: [n_slices][n_chunks]); used to
 * time blocks for the learned block model (the GPU counterpart of
 * studies/threshold.py:32-86). */
int sable_spmv_timed(sable_plan *plan, const float *x_dev, float *y_dev, int64_t *cycles_dev, void *stream);
int sable_spmm_timed(sable_plan *plan, const float *X_dev, float *Y_dev, int32_t N,
                     int64_t *cycles_dev, void *stream);
/* Tile index of every work item (host array of n_chunks int64). */
int sable_plan_chunk_tiles(const sable_plan *plan, int64_t *tile_of_chunk);

/*
 * Batch: many plans (matrices) run together, one graph launch per run.  No
 * reference counterpart (the reference times one matrix per process).
 * widths[i] = 1 runs SpMV on plan i; widths[i] = N > 1 (N % 4 == 0) runs SpMM
 * of width N, on the tensor cores when plan i was created with spmm_tc and
 * N >= 32.  Each matrix goes to the fastest executor its plan allows:
 * split-BF16 SpMM of plans with tcgen05 panel terms to the tcgen05 kernel
 * (one launch per N-slice width over the items of all of them, largest
 * first), SpMV of per-warp plans (schedule 2) to the per-warp kernel (one
 * launch over all their items), the rest to a persistent kernel whose CTAs
 * take (item, N-slice) units from an atomic queue sorted by class (split-BF16
 * SpMM, FP32 SpMM, SpMV) and size, keeping several SpMV records in flight
 * (TMA ring of `stages` records per CTA).  The batch copies the plans'
 * records; the plans may be destroyed after sable_batch_create.
 */
typedef struct sable_batch_opts {
    int32_t ctas_per_sm;  /* persistent CTAs per SM (0: as many as fit)       */
    int32_t use_graph;    /* 1: sable_batch_run replays a CUDA graph of the
                             queue reset and the kernel launch                 */
    int32_t stages;       /* SpMV records in flight per CTA: 2, 3, 4, 6 or 8
                             (SpMV-only batches), 2 or 4 with SpMM (0: auto)   */
} sable_batch_opts;

typedef struct sable_batch_info {
    int32_t n_mats;
    int32_t n_ctas;           /* persistent CTAs of the launch               */
    int64_t n_units;          /* work units: tcgen05 (item, slice) pairs,
                                 per-warp items and the queue's units        */
    int64_t device_bytes;     /* records, tables and scratch of the batch    */
    int32_t smem_bytes;       /* dynamic shared memory per CTA               */
    int32_t stage_bytes;      /* TMA staging bytes per SpMV stage            */
    int32_t stages;           /* SpMV ring depth                              */
} sable_batch_info;

int sable_batch_create(sable_plan *const *plans, int32_t n_plans, const int32_t *widths,
                       const sable_batch_opts *opts, sable_batch **out);
/* x_devs[i] / y_devs[i]: operand and result of matrix i, row-major with
 * leading dimension N (SpMM: 16-byte aligned).  One graph launch for the
 * whole batch (without use_graph, its launches in a row), stream-ordered on
 * `stream`. */
int sable_batch_run(sable_batch *batch, const float *const *x_devs, float *const *y_devs, void *stream);
/* Synchronises `stream`; SABLE_ERR_TIMEOUT if a bounded wait ran out. */
int sable_batch_check(sable_batch *batch, void *stream);
int sable_batch_get_info(const sable_batch *batch, sable_batch_info *out);
int sable_batch_destroy(sable_batch *batch);

/*
 * GPU inspector steps upstream of the plan (no plan needed).  Inputs are host
 * arrays; the functions upload them, run on the device (current device when
 * `device` < 0) and synchronise.
 */
typedef struct sable_csr_desc {
    int32_t n_rows, n_cols;
    const int64_t *indptr;   /* n_rows + 1 entries, from 0 to nnz, non-decreasing */
    const int32_t *indices;  /* column of every entry, 0 <= c < n_cols          */
    const void *data;        /* value of every entry: FP32 or FP64               */
    int32_t value_bytes;     /* 4 or 8                                           */
    int64_t nnz;
} sable_csr_desc;

/* VBR construction from a CSR matrix and its partition: replaces
 * convert_sparse_to_vbr (utils/convert_real_to_vbr.py:98-199).  Every
 * (rpntr x cpntr) block holding at least one stored entry (explicit zeros
 * count) becomes a stored block, dense and column-major, in block-row order,
 * ascending block column; duplicate entries are summed in CSR order.  Values
 * keep the CSR's type.  A block row without a stored entry gets
 * bpntrb = bpntre = -1 (the reference asserts that none exists).
 * SABLE_ERR_UNSUPPORTED when a block row's bitmap of n_block_cols bits does
 * not fit in shared memory (about 1.5 million block columns). */
typedef struct sable_vbr_build sable_vbr_build;
int sable_vbr_from_csr(const sable_csr_desc *csr, int32_t n_block_rows, const int32_t *rpntr, int32_t n_block_cols,
                       const int32_t *cpntr, int32_t device, sable_vbr_build **out);
/* Number of stored blocks and of values (val holds n_val entries of the
 * CSR's value type; indx n_blocks + 1; bpntrb / bpntre n_block_rows). */
int sable_vbr_build_sizes(const sable_vbr_build *build, int64_t *n_blocks, int64_t *n_val);
int sable_vbr_build_copy(const sable_vbr_build *build, void *val, int64_t *indx, int32_t *bindx, int32_t *bpntrb,
                         int32_t *bpntre);
int sable_vbr_build_destroy(sable_vbr_build *build);

/* Row and column partition by adjacent-line similarity: replaces cut_indices2
 * (src/autopartition.py:34-68) with similarity2 (:87-89, mode 0) or its numba
 * variant similarity2_numba (:91-107, mode 1, which scores a pair with an
 * all-zero line 0 instead of NaN).  `csr` is the matrix, `csc` its transpose
 * in CSR form (the matrix's CSC); indices must increase strictly within each
 * line.  Writes the row cuts (rpntr, at most n_rows + 1 entries) and the
 * column cuts (cpntr, at most n_cols + 1), each starting at 0 and ending at
 * the dimension, and their counts.  Similarities are computed in FP64. */
int sable_similarity_cuts(const sable_csr_desc *csr, const sable_csr_desc *csc, double threshold, int32_t mode,
                          int32_t device, int32_t *rpntr_out, int32_t *n_rpntr, int32_t *cpntr_out,
                          int32_t *n_cpntr);

/* Block features for the block model, one row of 6 floats per stored block
 * (bindx order): rows, cols, nnz, density, variance of nnz per row, N.
 * Host-side; `desc` must be uncompressed (all blocks in val). */
int sable_block_features(const sable_vbrc_desc *desc, int32_t N, float *feat_out);

/*
 * Block cost model: MLP 6 -> 64 -> 64 -> 2 (ReLU), FP32, predicting log2 of
 * the device time (SM cycles) of the dense and of the sparse form of a block;
 * a block is stored dense iff its first output is the smaller.  It replaces
 * the pickled RandomForest threshold (models/density_threshold_spmv.pkl,
 * loaded at utils/convert_real_to_vbr.py:20 and queried per block at :58).
 * Training and inference run on the device in this library's own kernels.
 * Features are the rows of sable_block_features; the kernels transform them
 * to log2(1 + f) (all but density) and then to (g - mean) / std.
 * Parameter order in flat buffers (row-major, out x in):
 *   W1[64x6], b1[64], W2[64x64], b2[64], W3[2x64], b3[2] = 4738 floats.
 */
#define SABLE_MLP_NPARAMS 4738
int sable_mlp_create(sable_mlp **out);            /* on the current device, params 0 */
int sable_mlp_destroy(sable_mlp *m);
/* Loads parameters and resets the optimiser state (Adam moments, step). */
int sable_mlp_set_params(sable_mlp *m, const float *params_host);
int sable_mlp_get_params(const sable_mlp *m, float *params_host);
/* Feature normalisation of the transformed features; std6[i] > 0. */
int sable_mlp_set_norm(sable_mlp *m, const float *mean6, const float *std6);
/* out_dev[n x 2] = MLP(feat_dev[n x 6]); n = 0 is a no-op. */
int sable_mlp_infer(sable_mlp *m, const float *feat_dev, int32_t n, float *out_dev, void *stream);
/* Loss L = 1/(2n) sum (out - target)^2 over the n x 2 outputs and its
 * gradient with respect to every parameter (grad_dev[SABLE_MLP_NPARAMS],
 * loss_dev[1] or NULL); no parameter update.  Deterministic: the same inputs
 * give bit-identical results. */
int sable_mlp_loss_grad(sable_mlp *m, const float *feat_dev, const float *target_dev, int32_t n,
                        float *grad_dev, float *loss_dev, void *stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on a batch of n samples:
 * sample s is row idx_dev[s] of feat_dev / target_dev (idx_dev NULL: row s).
 * loss_dev (may be NULL) receives the batch loss before the step. */
int sable_mlp_train_step(sable_mlp *m, const float *feat_dev, const float *target_dev, const int32_t *idx_dev,
                         int32_t n, float lr, float *loss_dev, void *stream);

/* Self-test of the bounded device waits (no counterpart in the reference):
 * a one-thread kernel waits up to limit_us (1..2e6) microseconds for an
 * mbarrier phase; with arrive == 0 nothing completes it, the wait runs out
 * and the call returns SABLE_ERR_TIMEOUT, as the kernels report a wait that
 * ran out (the context stays usable); with arrive != 0 the thread arrives
 * first and the call returns SABLE_OK.  *elapsed_ns (if not NULL): the
 * time the wait took on the device.  Synchronises `stream`. */
int sable_selftest_wait(int64_t limit_us, int32_t arrive, int64_t *elapsed_ns, void *stream);

const char *sable_strerror(int code);
const char *sable_last_error(void);
/* Library version string. */
const char *sable_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SABLE_H */
