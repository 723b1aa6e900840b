// Batched VBR SpMV / SpMM: many matrices, one graph launch per run.
//
// The reference runs one generated program per matrix; serving many small
// and mid-size matrices that way leaves the GPU idle between launches and
// gives every launch its own tail.  A batch merges the item records of all
// its plans into one device buffer (a standard record's header carries its
// matrix index; compact records get theirs from a per-item table) and builds
// one work queue of units for the persistent kernel:
//   SpMV unit   one item record of a width-1 matrix
//   SpMM unit   one (item record, N-slice) pair, FP32 or split-BF16
// sorted by class (split-BF16 SpMM, FP32 SpMM, SpMV) and within a class by
// size, largest first.  A grid of SMs x k persistent CTAs takes units in
// queue order from an atomic head, so the largest units start first and the
// small ones fill the tail (greedy list scheduling).
//
// Split-BF16 SpMM items of plans that hold tcgen05 panel terms (the default
// for plans built with spmm_tc) do not enter the queue: they run on the
// tcgen05 kernel (spmm_umma.cu), one launch per N-slice width over the items
// of all such matrices (largest first, each CTA reading its matrix from the
// batch's matrix table), before the persistent kernel, in the same graph.
// Likewise the SpMV matrices of plans of the per-warp executor (compact
// records) run on the per-warp kernel (spmv.cu), one launch over all their
// items, largest first, with a per-item matrix table; those records combine
// their split tiles themselves.
// The other SpMM units run the bodies of spmm_item.cuh from global memory.  SpMV units
// run the CTA-per-item body (spmv_item.cuh) from an S-stage TMA ring that
// keeps S claimed records in flight per CTA (S = 2..8; by default the
// deepest ring that still allows the most CTAs per SM).  A CTA's shared memory is used by one
// phase at a time (the queue order makes the phases disjoint, see the
// kernel).  Every mbarrier wait is bounded; on expiry the
// batch's error flag is set and the CTA waits (bounded) for its own copies
// and leaves.  The split tiles of the queue's SpMV matrices are combined by
// one launch after the kernel.  A run launches only what has work: the
// tcgen05 launches, the per-warp launch, the persistent kernel, the combine.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "sable.h"
#include "plan_internal.h"
#include "spmv_item.cuh"
#include "spmm_item.cuh"

namespace {

enum UnitKind : int16_t {
    U_SPMV = 0,
    U_F32_16, U_F32_32, U_F32_64,
    U_TC2_32, U_TC2_64,
    U_TC3_32, U_TC3_64,
};

struct BatchUnit {
    int32_t item;    // index into the merged item table
    int16_t slice;   // N-slice (SpMM)
    int16_t kind;
};
static_assert(sizeof(BatchUnit) == 8, "BatchUnit must stay 8 bytes");

struct BatchArgs {
    const unsigned char *records;
    const ItemRef *items;
    const uint4 *tcplanes;  // pre-split A fragments of the plans that have them, merged
    const int64_t *tcoff;   // per merged item: word offset in tcplanes, -1: split per K step
    const BatchUnit *units;
    const MatIO *mats;
    int *head;           // queue head, zero before each launch
    int *error;
    int n_units;
    int stage_bytes;     // bytes of one SpMV stage (>= largest SpMV record)
};

__device__ __forceinline__ void run_spmm_unit(const BatchArgs &b, const BatchUnit U, const unsigned char *R,
                                              const MatIO &io, unsigned char *smem) {
    const int64_t po = (U.kind >= U_TC2_32 && b.tcoff) ? b.tcoff[U.item] : -1;
    const uint4 *pl = po >= 0 ? b.tcplanes + po : nullptr;
    switch (U.kind) {
        case U_F32_16: spmm_fp32_item<16>(R, io, U.slice, io.part_stride, smem); break;
        case U_F32_32: spmm_fp32_item<32>(R, io, U.slice, io.part_stride, smem); break;
        case U_F32_64: spmm_fp32_item<64>(R, io, U.slice, io.part_stride, smem); break;
        case U_TC2_32:
            if (pl) spmm_tc_item<32, 2, true>(R, io, U.slice, io.part_stride, smem, pl);
            else spmm_tc_item<32, 2>(R, io, U.slice, io.part_stride, smem);
            break;
        case U_TC2_64:
            if (pl) spmm_tc_item<64, 2, true>(R, io, U.slice, io.part_stride, smem, pl);
            else spmm_tc_item<64, 2>(R, io, U.slice, io.part_stride, smem);
            break;
        case U_TC3_32:
            if (pl) spmm_tc_item<32, 3, true>(R, io, U.slice, io.part_stride, smem, pl);
            else spmm_tc_item<32, 3>(R, io, U.slice, io.part_stride, smem);
            break;
        case U_TC3_64:
            if (pl) spmm_tc_item<64, 3, true>(R, io, U.slice, io.part_stride, smem, pl);
            else spmm_tc_item<64, 3>(R, io, U.slice, io.part_stride, smem);
            break;
        default: break;
    }
}

// Queue order puts every SpMM unit before every SpMV unit, and a CTA's claims
// (atomicAdd on the head) only grow, so a CTA runs SpMM units until its first
// SpMV claim and SpMV units from then on:
//   phase 1  SpMM units straight from global memory, no copy in flight;
//   phase 2  SpMV units through an S-stage ring: the CTA keeps S claimed units'
//            records in flight (TMA bulk copies, one mbarrier per stage), waits
//            for the oldest, computes it, and refills its stage with a new claim.
// SPMM = false compiles the SpMV-only form (fewer registers, more CTAs per SM).
template <int S, bool SPMM>
__global__ void __launch_bounds__(SABLE_THREADS, SPMM ? 2 : 3)
batch_kernel(const BatchArgs b) {
    extern __shared__ __align__(128) unsigned char smem[];
    float *red = reinterpret_cast<float *>(smem);
    float *ysw = red + RED_FLOATS;
    unsigned char *const stage0 = smem + STAGE_OFF;
    __shared__ __align__(8) unsigned long long s_bar[S];
    __shared__ int s_unit[S];   // unit claimed into each stage (>= n_units: none)
    __shared__ int s_claim;
    __shared__ int s_bad;
    const int tid = threadIdx.x;
    const int n = b.n_units;
    unsigned phase_bits = 0;    // control thread: parity of each stage's next wait
    auto bar = [&](int k) { return smem_addr(&s_bar[k]); };
    auto stage = [&](int k) { return stage0 + (size_t)k * b.stage_bytes; };
    // control thread: claim a unit for stage k and start its record copy
    auto refill = [&](int k) {
        const int u = atomicAdd(b.head, 1);
        s_unit[k] = u;
        if (u < n) {
            const ItemRef r = b.items[b.units[u].item];
            tma_record(bar(k), stage(k), b.records + r.off, (unsigned)r.bytes);
        }
    };
    if (tid == CTRL) {
        for (int k = 0; k < S; ++k) mbar_init(bar(k));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_claim = atomicAdd(b.head, 1);
        s_bad = 0;
    }
    for (int i = tid; i < RED_FLOATS; i += SABLE_THREADS) ysw[i] = 0.f;
    __syncthreads();

    // ---- phase 1: SpMM units -------------------------------------------------
    if (SPMM) {
        while (true) {
            const int u = s_claim;
            if (u >= n || b.units[u].kind == U_SPMV) break;
            const BatchUnit U = b.units[u];
            const ItemRef ref = b.items[U.item];
            const unsigned char *R = b.records + ref.off;
            if (reinterpret_cast<const ItemHeader *>(R)->bytes == ref.bytes) {
                run_spmm_unit(b, U, R, b.mats[reinterpret_cast<const ItemHeader *>(R)->mat], smem);
            } else if (tid == CTRL) {
                atomicExch(b.error, 1);
            }
            __syncthreads();
            if (tid == CTRL) s_claim = atomicAdd(b.head, 1);
            __syncthreads();
        }
        // the SpMM bodies used the whole shared memory: restore the zero CSR rows
        for (int i = tid; i < RED_FLOATS; i += SABLE_THREADS) ysw[i] = 0.f;
        __syncthreads();
    }

    // ---- phase 2: SpMV ring --------------------------------------------------
    if (s_claim >= n) return;
    if (tid == CTRL) {
        const int u0 = s_claim;
        s_unit[0] = u0;
        const ItemRef r = b.items[b.units[u0].item];
        tma_record(bar(0), stage(0), b.records + r.off, (unsigned)r.bytes);
        for (int k = 1; k < S; ++k) refill(k);
    }
    __syncthreads();
    for (int it = 0;; ++it) {
        const int k = it % S;
        const int u = s_unit[k];
        if (u >= n) break;
        if (tid == CTRL) {
            const bool landed = mbar_wait(bar(k), (phase_bits >> k) & 1u);
            if (landed) phase_bits ^= 1u << k;
            const ItemRef ref = b.items[b.units[u].item];
            if (!landed || reinterpret_cast<const ItemHeader *>(stage(k))->bytes != ref.bytes) {
                // flag, then wait (bounded) for every copy this CTA has in flight
                atomicExch(b.error, 1);
                for (int j = 0; j < S; ++j) {
                    const int kk = (k + j) % S;
                    if (s_unit[kk] < n && (kk != k || !landed)) mbar_wait(bar(kk), (phase_bits >> kk) & 1u);
                }
                s_bad = 1;
            }
        }
        __syncthreads();
        if (s_bad) return;
        const unsigned char *R = stage(k);
        const ItemHeader hd = *reinterpret_cast<const ItemHeader *>(R);
        const MatIO &io = b.mats[hd.mat];
        cta_accumulate(R, hd, io.x, nullptr, red, ysw);
        __syncthreads();
        cta_finish(hd, io, red, ysw);
        __syncthreads();   // stage k is free
        if (tid == CTRL) refill(k);
        __syncthreads();
    }
}

// Writes each merged record's matrix index into its header.
__global__ void patch_mat_kernel(unsigned char *records, const ItemRef *items, const int32_t *mat, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) reinterpret_cast<ItemHeader *>(records + items[k].off)->mat = mat[k];
}

int spmm_nt(int N) { return N <= 16 ? 16 : N <= 32 ? 32 : 64; }

// A split-BF16 SpMM matrix whose plan holds tcgen05 panel terms runs on the
// tcgen05 kernel, outside the persistent kernel's queue.
bool runs_umma(const sable_plan *p, int W) {
    return W >= 32 && p->spmm_tc && p->tc_kernel == SABLE_TC_KERNEL_UMMA && p->d_umma &&
           p->umma_off_host.size() == (size_t)p->n_items;
}

int16_t spmm_kind(int nt, int tc_terms) {
    if (tc_terms == 0) return nt == 16 ? U_F32_16 : nt == 32 ? U_F32_32 : U_F32_64;
    if (tc_terms == 2) return nt == 32 ? U_TC2_32 : U_TC2_64;
    return nt == 32 ? U_TC3_32 : U_TC3_64;
}

// pre: the unit's A fragments come pre-split (a larger A stage)
int spmm_unit_smem(int16_t kind, bool pre) {
    switch (kind) {
        case U_F32_16: return SpmmSmem<16>::TOTAL;
        case U_F32_32: return SpmmSmem<32>::TOTAL;
        case U_F32_64: return SpmmSmem<64>::TOTAL;
        case U_TC2_32: case U_TC3_32: return pre ? TcSmem<32, true>::TOTAL : TcSmem<32>::TOTAL;
        case U_TC2_64: case U_TC3_64: return pre ? TcSmem<64, true>::TOTAL : TcSmem<64>::TOTAL;
        default: return 0;
    }
}

using BatchKernel = void (*)(BatchArgs);

// Instantiated ring depths: 2/4 with SpMM bodies, 2/3/4/6/8 SpMV-only.
BatchKernel batch_kernel_for(int S, bool spmm) {
    if (spmm) return S >= 4 ? batch_kernel<4, true> : batch_kernel<2, true>;
    switch (S) {
        case 2: return batch_kernel<2, false>;
        case 3: return batch_kernel<3, false>;
        case 4: return batch_kernel<4, false>;
        case 6: return batch_kernel<6, false>;
        default: return batch_kernel<8, false>;
    }
}

}  // namespace

// Split-BF16 SpMM items run by the tcgen05 kernel, per N-slice width and
// number of terms.
struct UmmaGroup {
    int nt = 0, terms = 0, N = 0, hp = 16;
    int n_items = 0;
    ItemRef *d_items = nullptr;     // merged records, largest first
    int64_t *d_off = nullptr;       // byte offset of each item's panel terms in d_umma, -1: none
};

struct sable_batch {
    int device = 0;
    std::vector<UmmaGroup> umma;
    int n_warp_items = 0;                // per-warp SpMV items (compact records)
    ItemRef *d_warp_items = nullptr;     // their merged records, largest first
    int32_t *d_warp_mat = nullptr;       // and their matrices
    unsigned char *d_umma = nullptr;     // merged tcgen05 panel terms
    int n_mats = 0;
    std::vector<int32_t> width;
    std::vector<int64_t> n_rows, n_cols;
    unsigned char *d_records = nullptr;
    ItemRef *d_items = nullptr;
    uint4 *d_tcplanes = nullptr;         // merged pre-split A fragments (or nullptr)
    int64_t *d_tcoff = nullptr;          // per merged item, -1: none
    BatchUnit *d_units = nullptr;
    MatIO *d_mats = nullptr;
    MatIO *h_mats = nullptr;          // pinned staging of the matrix table
    float *d_partial = nullptr;
    int *d_counters = nullptr;
    int *d_head = nullptr;
    int *d_error = nullptr;
    SplitTile *d_splits = nullptr;       // SpMV split tiles of every matrix (combine launch)
    int n_splits = 0;
    int64_t n_units = 0, device_bytes = 0;
    int64_t n_queue = 0;                 // units of the persistent kernel's queue (n_units adds the tcgen05 ones)
    int stage_bytes = 0, smem = 0, n_ctas = 0, stages = 0;
    BatchKernel kernel = nullptr;
    bool mats_valid = false;
    bool use_graph = false;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;
};

using namespace sable;

namespace {

int batch_launch(sable_batch *bt, cudaStream_t s) {
    BatchArgs a;
    a.records = bt->d_records;
    a.items = bt->d_items;
    a.tcplanes = bt->d_tcplanes;
    a.tcoff = bt->d_tcplanes ? bt->d_tcoff : nullptr;
    a.units = bt->d_units;
    a.mats = bt->d_mats;
    a.head = bt->d_head;
    a.error = bt->d_error;
    a.n_units = (int)bt->n_queue;
    a.stage_bytes = bt->stage_bytes;
    for (const UmmaGroup &g : bt->umma) {
        LaunchArgs la;
        memset(&la, 0, sizeof la);
        la.records = bt->d_records;
        la.items = g.d_items;
        la.mats = bt->d_mats;
        la.umma = bt->d_umma;
        la.umma_off = g.d_off;
        la.umma_hp = g.hp;
        la.error = bt->d_error;
        la.n_items = g.n_items;
        const int ec = launch_spmm_umma(la, g.N, g.nt, g.terms, 0, false, s);
        if (ec) return cuda_fail((cudaError_t)ec, "batch tcgen05 SpMM launch");
    }
    if (bt->n_warp_items > 0) {
        LaunchArgs la;
        memset(&la, 0, sizeof la);
        la.records = bt->d_records;
        la.items = bt->d_warp_items;
        la.item_mat = bt->d_warp_mat;
        la.mats = bt->d_mats;
        la.error = bt->d_error;
        la.n_items = bt->n_warp_items;
        const int ec = launch_spmv_warp_items(la, false, s);
        if (ec) return cuda_fail((cudaError_t)ec, "batch per-warp SpMV launch");
    }
    cudaError_t e = cudaSuccess;
    if (bt->n_queue > 0) {
        e = cudaMemsetAsync(bt->d_head, 0, sizeof(int), s);
        if (e != cudaSuccess) return cuda_fail(e, "batch queue reset");
        bt->kernel<<<bt->n_ctas, SABLE_THREADS, bt->smem, s>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "batch kernel launch");
    }
    if (bt->n_splits > 0) {
        MatIO none;
        memset(&none, 0, sizeof none);
        const int ec = launch_spmv_combine(bt->d_splits, bt->n_splits, bt->d_mats, none, s);
        if (ec) return cuda_fail((cudaError_t)ec, "batch combine launch");
    }
    return SABLE_OK;
}

template <class T>
int dev_alloc(T **p, size_t n, int64_t *bytes, const char *what) {
    cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "batch %s: %s", what, cudaGetErrorString(e));
    *bytes += (int64_t)(std::max<size_t>(n, 1) * sizeof(T));
    return SABLE_OK;
}

}  // namespace

extern "C" {

int sable_batch_destroy(sable_batch *bt) {
    if (!bt) return SABLE_OK;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(bt->device);
    if (bt->done) cudaEventSynchronize(bt->done);
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    if (bt->cap_stream) cudaStreamDestroy(bt->cap_stream);
    if (bt->done) cudaEventDestroy(bt->done);
    cudaFree(bt->d_records);
    cudaFree(bt->d_tcplanes);
    cudaFree(bt->d_tcoff);
    cudaFree(bt->d_items);
    cudaFree(bt->d_units);
    cudaFree(bt->d_mats);
    cudaFree(bt->d_partial);
    cudaFree(bt->d_counters);
    cudaFree(bt->d_head);
    cudaFree(bt->d_error);
    cudaFree(bt->d_splits);
    for (UmmaGroup &g : bt->umma) {
        cudaFree(g.d_items);
        cudaFree(g.d_off);
    }
    cudaFree(bt->d_umma);
    cudaFree(bt->d_warp_items);
    cudaFree(bt->d_warp_mat);
    if (bt->h_mats) cudaFreeHost(bt->h_mats);
    if (prev >= 0) cudaSetDevice(prev);
    delete bt;
    return SABLE_OK;
}

int sable_batch_create(sable_plan *const *plans, int32_t n_plans, const int32_t *widths,
                       const sable_batch_opts *opts, sable_batch **out) {
    if (!plans || !widths || !out || n_plans <= 0) return fail(SABLE_ERR_ARG, "bad argument");
    *out = nullptr;
    sable_batch_opts o{};
    if (opts) o = *opts;
    if (o.ctas_per_sm < 0) return fail(SABLE_ERR_ARG, "ctas_per_sm must be >= 0");
    for (int i = 0; i < n_plans; ++i) {
        if (!plans[i]) return fail(SABLE_ERR_ARG, "plan %d is null", i);
        if (plans[i]->device != plans[0]->device) return fail(SABLE_ERR_ARG, "plans on different devices");
        if (plans[i]->compact && widths[i] != 1)
            return fail(SABLE_ERR_UNSUPPORTED, "plan %d: a plan of the per-warp SpMV executor (schedule 2) runs SpMV only", i);
        // the tcgen05 and per-warp kernels stream their records; everything
        // else in a batch stages whole records in shared memory
        if (!plans[i]->staged_ok && !runs_umma(plans[i], widths[i]) && !plans[i]->compact)
            return fail(SABLE_ERR_UNSUPPORTED, "plan %d: work items larger than the batch's staging (%d bytes)", i,
                        SABLE_MAX_ITEM_BYTES);
        if (widths[i] < 1 || (widths[i] > 1 && (widths[i] & 3)))
            return fail(SABLE_ERR_UNSUPPORTED, "width %d of matrix %d: 1, or a multiple of 4", widths[i], i);
    }
    int rc = set_device(plans[0]->device);
    if (rc) return rc;
    sable_batch *bt = new (std::nothrow) sable_batch();
    if (!bt) return fail(SABLE_ERR_NOMEM, "host allocation");
    bt->device = plans[0]->device;
    bt->n_mats = n_plans;
    bt->use_graph = o.use_graph != 0;
    auto bail = [&](int code) {
        sable_batch_destroy(bt);
        return code;
    };

    // merged records and item table; per-matrix scratch and the unit queue
    int64_t rec_total = 0, n_items = 0;
    for (int i = 0; i < n_plans; ++i) {
        rec_total += plans[i]->records_bytes;
        n_items += plans[i]->n_items;
    }
    if (n_items >= INT32_MAX) return bail(fail(SABLE_ERR_UNSUPPORTED, "batch of %lld items", (long long)n_items));
    std::vector<ItemRef> items;
    std::vector<int64_t> item_tcoff;  // merged pre-split fragment offsets, -1: none
    int64_t tc_base = 0;
    std::vector<int32_t> item_mat;
    items.reserve(n_items);
    item_mat.reserve(n_items);
    std::vector<MatIO> mats(n_plans);
    std::vector<SplitTile> splits;
    struct Sortable {
        int32_t cls;
        int64_t cost;
        BatchUnit u;
    };
    std::vector<Sortable> q;
    int64_t partial_total = 0, counter_total = 0, rec_base = 0;
    std::vector<int64_t> part_off(n_plans), cnt_off(n_plans);
    // tcgen05 items per (slice width, terms): merged item, panel-term offset, cost
    struct UmmaItem {
        ItemRef r;
        int64_t off;
    };
    std::vector<UmmaGroup> groups;
    std::vector<std::vector<UmmaItem>> group_items;
    struct WarpItem {
        ItemRef r;
        int32_t mat;
    };
    std::vector<WarpItem> warp_items;
    int64_t umma_base = 0;
    for (int i = 0; i < n_plans; ++i) {
        const sable_plan *p = plans[i];
        const int W = widths[i];
        bt->width.push_back(W);
        bt->n_rows.push_back(p->n_rows);
        bt->n_cols.push_back(p->n_cols);
        const int terms = (W >= 32 && p->spmm_tc) ? (p->spmm_tc == SABLE_TC_SPLIT3 ? 3 : 2) : 0;
        // split-BF16 SpMM of a plan with tcgen05 panel terms: the tcgen05
        // kernel, with the slice width of sable_spmm
        const bool umma = terms && runs_umma(p, W);
        const int nt = W == 1 ? 1 : umma ? spmm_slice_width(W) : spmm_nt(W);
        const int slices = W == 1 ? 1 : (W + nt - 1) / nt;
        int gidx = -1;
        if (umma) {
            for (size_t g = 0; g < groups.size(); ++g)
                if (groups[g].nt == nt && groups[g].terms == terms) gidx = (int)g;
            if (gidx < 0) {
                UmmaGroup g;
                g.nt = nt;
                g.terms = terms;
                groups.push_back(g);
                group_items.emplace_back();
                gidx = (int)groups.size() - 1;
            }
            groups[gidx].N = std::max(groups[gidx].N, W);
            groups[gidx].hp = std::max(groups[gidx].hp, p->umma_hp);
        }
        const int16_t kind = W == 1 ? (int16_t)U_SPMV : spmm_kind(nt, terms);
        const int32_t cls = W == 1 ? 2 : (terms ? 0 : 1);
        const int64_t nsplit = std::max<int32_t>(p->n_split_tiles, 1);
        MatIO &m = mats[i];
        memset(&m, 0, sizeof m);
        m.ldx = m.ldy = W;
        m.N = W;
        m.pad = (int32_t)nsplit;
        m.part_stride = p->n_partial * nt;
        // regions start on 256-byte boundaries: the SpMM bodies move float4s
        part_off[i] = partial_total;
        cnt_off[i] = counter_total;
        partial_total += (std::max<int64_t>(p->n_partial * nt * slices, 1) + 63) & ~(int64_t)63;
        counter_total += nsplit * slices;
        for (int64_t k = 0; k < p->n_items; ++k) {
            ItemRef r = p->items_host[k];
            r.off += rec_base;
            if (p->compact) {   // the per-warp kernel; its header layout has no matrix field
                warp_items.push_back({r, i});
                bt->n_units += 1;
                continue;
            }
            const int32_t idx = (int32_t)items.size();
            items.push_back(r);
            item_tcoff.push_back(terms && !umma && !p->tcoff_host.empty() ? tc_base + p->tcoff_host[k] : -1);
            item_mat.push_back(i);
            if (kind == U_SPMV) bt->stage_bytes = std::max(bt->stage_bytes, r.bytes);
            if (umma) {
                const int64_t po = p->umma_off_host[k];
                group_items[gidx].push_back({r, po >= 0 ? umma_base + po : -1});
                bt->n_units += slices;
                continue;
            }
            for (int sl = 0; sl < slices; ++sl) {
                Sortable s;
                s.cls = cls;
                s.cost = (int64_t)r.bytes * (W == 1 ? 1 : nt);
                s.u.item = idx;
                s.u.slice = (int16_t)sl;
                s.u.kind = kind;
                q.push_back(s);
            }
        }
        if (W == 1 && !p->compact)   // compact records combine their split tiles themselves
            for (SplitTile t : p->splits_host) {
                t.mat = i;
                splits.push_back(t);
            }
        rec_base += p->records_bytes;
        if (terms && !umma && !p->tcoff_host.empty()) tc_base += p->tc_words;
        if (umma) umma_base += p->umma_bytes;
    }
    std::stable_sort(warp_items.begin(), warp_items.end(),
                     [](const WarpItem &a, const WarpItem &b) { return a.r.cost > b.r.cost; });
    for (auto &gi : group_items)   // largest first
        std::stable_sort(gi.begin(), gi.end(), [](const UmmaItem &a, const UmmaItem &b) { return a.r.bytes > b.r.bytes; });
    std::stable_sort(q.begin(), q.end(), [](const Sortable &a, const Sortable &b) {
        return a.cls != b.cls ? a.cls < b.cls : a.cost > b.cost;
    });
    std::vector<BatchUnit> units(q.size());
    int spmm_smem = 0;
    for (size_t k = 0; k < q.size(); ++k) {
        units[k] = q[k].u;
        spmm_smem = std::max(spmm_smem, spmm_unit_smem(q[k].u.kind, item_tcoff[q[k].u.item] >= 0));
    }
    bt->n_queue = (int64_t)units.size();
    bt->n_units += bt->n_queue;
    if (bt->n_queue >= INT32_MAX) return bail(fail(SABLE_ERR_UNSUPPORTED, "batch of %lld units", (long long)bt->n_queue));
    bt->stage_bytes = (bt->stage_bytes + 127) & ~127;
    bool has_spmm = false;
    for (const BatchUnit &u : units) has_spmm |= u.kind != U_SPMV;
    int dev_max = 0, sms = 0;
    cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, bt->device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, bt->device);
    // ring depth: as asked, else the most CTAs per SM first (each CTA's compute
    // is latency-bound, so concurrent CTAs matter more than depth), then the
    // deepest ring at that CTA count
    {
        const int cand_spmm[] = {2, 4}, cand_spmv[] = {2, 3, 4, 6, 8};
        const int *cand = has_spmm ? cand_spmm : cand_spmv;
        const int ncand = has_spmm ? 2 : 5;
        const int sm_budget = 227 * 1024;
        int best_s = 2;
        int64_t best_score = -1;
        for (int c = 0; c < ncand; ++c) {
            const int S = cand[c];
            if (o.stages && S != o.stages) continue;
            const int need = std::max(STAGE_OFF + S * bt->stage_bytes, spmm_smem);
            if (need > dev_max) continue;
            int per_sm = std::min(sm_budget / (need + 1024), has_spmm ? 2 : 3);
            if (o.ctas_per_sm) per_sm = std::min(per_sm, o.ctas_per_sm);
            if (per_sm < 1) continue;
            const int64_t score = (int64_t)per_sm * 16 + S;
            if (score > best_score) {
                best_score = score;
                best_s = S;
            }
        }
        if (o.stages && best_score < 0)
            return bail(fail(SABLE_ERR_UNSUPPORTED, "stages=%d does not fit shared memory", o.stages));
        bt->stages = best_s;
    }
    bt->kernel = batch_kernel_for(bt->stages, has_spmm);
    bt->smem = std::max(bt->stage_bytes ? STAGE_OFF + bt->stages * bt->stage_bytes : 0, spmm_smem);
    bt->smem = std::max(bt->smem, STAGE_OFF);

    int64_t &bytes = bt->device_bytes;
    if ((rc = dev_alloc(&bt->d_records, (size_t)rec_total, &bytes, "records"))) return bail(rc);
    if (tc_base > 0) {
        if ((rc = dev_alloc(&bt->d_tcplanes, (size_t)tc_base, &bytes, "split-BF16 panels"))) return bail(rc);
        if ((rc = dev_alloc(&bt->d_tcoff, item_tcoff.size(), &bytes, "split-BF16 offsets"))) return bail(rc);
    }
    if ((rc = dev_alloc(&bt->d_items, items.size(), &bytes, "items"))) return bail(rc);
    if (umma_base > 0 && (rc = dev_alloc(&bt->d_umma, (size_t)umma_base, &bytes, "tcgen05 panel terms"))) return bail(rc);
    bt->n_warp_items = (int)warp_items.size();
    if (!warp_items.empty()) {
        if ((rc = dev_alloc(&bt->d_warp_items, warp_items.size(), &bytes, "per-warp items"))) return bail(rc);
        if ((rc = dev_alloc(&bt->d_warp_mat, warp_items.size(), &bytes, "per-warp item matrices"))) return bail(rc);
    }
    for (size_t g = 0; g < groups.size(); ++g) {
        UmmaGroup &G = groups[g];
        G.n_items = (int)group_items[g].size();
        if ((rc = dev_alloc(&G.d_items, group_items[g].size(), &bytes, "tcgen05 items"))) return bail(rc);
        if ((rc = dev_alloc(&G.d_off, group_items[g].size(), &bytes, "tcgen05 term offsets"))) {
            bt->umma.push_back(G);
            return bail(rc);
        }
        bt->umma.push_back(G);
    }
    if ((rc = dev_alloc(&bt->d_units, units.size(), &bytes, "units"))) return bail(rc);
    if ((rc = dev_alloc(&bt->d_mats, mats.size(), &bytes, "matrix table"))) return bail(rc);
    if ((rc = dev_alloc(&bt->d_partial, (size_t)partial_total, &bytes, "partials"))) return bail(rc);
    if ((rc = dev_alloc(&bt->d_counters, (size_t)counter_total, &bytes, "counters"))) return bail(rc);
    if ((rc = dev_alloc(&bt->d_head, 1, &bytes, "queue head"))) return bail(rc);
    if ((rc = dev_alloc(&bt->d_error, 1, &bytes, "error flag"))) return bail(rc);
    bt->n_splits = (int)splits.size();
    if ((rc = dev_alloc(&bt->d_splits, splits.size(), &bytes, "split tiles"))) return bail(rc);
    int32_t *d_item_mat = nullptr;
    int64_t scratch_bytes = 0;
    if ((rc = dev_alloc(&d_item_mat, item_mat.size(), &scratch_bytes, "item matrices"))) return bail(rc);
    cudaError_t e = cudaSuccess;
    rec_base = 0;
    for (int i = 0; i < n_plans && e == cudaSuccess; ++i) {
        if (plans[i]->records_bytes)
            e = cudaMemcpy(bt->d_records + rec_base, plans[i]->d_records, (size_t)plans[i]->records_bytes,
                           cudaMemcpyDeviceToDevice);
        rec_base += plans[i]->records_bytes;
    }
    if (tc_base > 0) {
        int64_t wb = 0;
        for (int i = 0; i < n_plans && e == cudaSuccess; ++i) {
            const sable_plan *p = plans[i];
            const bool tc = widths[i] >= 32 && p->spmm_tc && !p->tcoff_host.empty() && !runs_umma(p, widths[i]);
            if (!tc) continue;
            e = cudaMemcpy(bt->d_tcplanes + wb, p->d_tcplanes, (size_t)p->tc_words * sizeof(uint4), cudaMemcpyDeviceToDevice);
            wb += p->tc_words;
        }
        if (e == cudaSuccess)
            e = cudaMemcpy(bt->d_tcoff, item_tcoff.data(), item_tcoff.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    }
    if (umma_base > 0) {
        int64_t ub = 0;
        for (int i = 0; i < n_plans && e == cudaSuccess; ++i) {
            const sable_plan *p = plans[i];
            if (!runs_umma(p, widths[i])) continue;
            e = cudaMemcpy(bt->d_umma + ub, p->d_umma, (size_t)p->umma_bytes, cudaMemcpyDeviceToDevice);
            ub += p->umma_bytes;
        }
    }
    for (size_t g = 0; g < bt->umma.size() && e == cudaSuccess; ++g) {
        std::vector<ItemRef> gr;
        std::vector<int64_t> go;
        for (const UmmaItem &it : group_items[g]) {
            gr.push_back(it.r);
            go.push_back(it.off);
        }
        e = cudaMemcpy(bt->umma[g].d_items, gr.data(), gr.size() * sizeof(ItemRef), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(bt->umma[g].d_off, go.data(), go.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && !warp_items.empty()) {
        std::vector<ItemRef> wr;
        std::vector<int32_t> wm;
        for (const WarpItem &w : warp_items) {
            wr.push_back(w.r);
            wm.push_back(w.mat);
        }
        e = cudaMemcpy(bt->d_warp_items, wr.data(), wr.size() * sizeof(ItemRef), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(bt->d_warp_mat, wm.data(), wm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_items, items.data(), items.size() * sizeof(ItemRef), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(bt->d_units, units.data(), units.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_item_mat, item_mat.data(), item_mat.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !splits.empty())
        e = cudaMemcpy(bt->d_splits, splits.data(), splits.size() * sizeof(SplitTile), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items.empty()) {
        patch_mat_kernel<<<(unsigned)((items.size() + 255) / 256), 256>>>(bt->d_records, bt->d_items, d_item_mat,
                                                                          (int)items.size());
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d_item_mat);
    if (e == cudaSuccess) e = cudaMemset(bt->d_counters, 0, (size_t)std::max<int64_t>(counter_total, 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(bt->d_error, 0, sizeof(int));
    if (e != cudaSuccess) return bail(cuda_fail(e, "batch upload"));
    for (int i = 0; i < n_plans; ++i) {
        mats[i].partial = bt->d_partial + part_off[i];
        mats[i].counters = bt->d_counters + cnt_off[i];
    }
    e = cudaMallocHost((void **)&bt->h_mats, mats.size() * sizeof(MatIO));
    if (e != cudaSuccess) return bail(cuda_fail(e, "batch pinned table"));
    memcpy(bt->h_mats, mats.data(), mats.size() * sizeof(MatIO));

    // launch shape
    int occ = 0;
    if (bt->smem > dev_max)
        return bail(fail(SABLE_ERR_UNSUPPORTED, "batch needs %d bytes of shared memory per CTA (device: %d)", bt->smem,
                         dev_max));
    e = cudaFuncSetAttribute(bt->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bt->smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bt->kernel, SABLE_THREADS, bt->smem);
    if (e != cudaSuccess) return bail(cuda_fail(e, "batch kernel occupancy"));
    occ = std::max(occ, 1);
    const int per_sm = o.ctas_per_sm ? std::min(o.ctas_per_sm, occ) : occ;
    bt->n_ctas = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * per_sm, std::max<int64_t>(bt->n_queue, 1)));
    e = cudaEventCreateWithFlags(&bt->done, cudaEventDisableTiming);
    if (e != cudaSuccess) return bail(cuda_fail(e, "batch event"));
    if (bt->use_graph) {
        e = cudaStreamCreateWithFlags(&bt->cap_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return bail(cuda_fail(e, "batch capture stream"));
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(bt->cap_stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return bail(cuda_fail(e, "batch graph capture"));
        rc = batch_launch(bt, bt->cap_stream);
        e = cudaStreamEndCapture(bt->cap_stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return bail(rc);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&bt->exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return bail(cuda_fail(e, "batch graph instantiate"));
    }
    *out = bt;
    return SABLE_OK;
}

int sable_batch_run(sable_batch *bt, const float *const *x_devs, float *const *y_devs, void *stream) {
    if (!bt || !x_devs || !y_devs) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(bt->device);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bool changed = !bt->mats_valid;
    for (int i = 0; i < bt->n_mats; ++i) {
        if (!x_devs[i] || !y_devs[i]) return fail(SABLE_ERR_ARG, "null operand of matrix %d", i);
        if (bt->width[i] > 1 && (((uintptr_t)x_devs[i] & 15) || ((uintptr_t)y_devs[i] & 15)))
            return fail(SABLE_ERR_UNSUPPORTED, "SpMM operands of matrix %d must be 16-byte aligned", i);
        changed |= bt->h_mats[i].x != x_devs[i] || bt->h_mats[i].y != y_devs[i];
    }
    cudaError_t e;
    if (changed) {
        // the previous run's copy of the pinned table must have completed
        e = cudaEventSynchronize(bt->done);
        if (e != cudaSuccess) return cuda_fail(e, "batch table wait");
        for (int i = 0; i < bt->n_mats; ++i) {
            bt->h_mats[i].x = x_devs[i];
            bt->h_mats[i].y = y_devs[i];
        }
        e = cudaMemcpyAsync(bt->d_mats, bt->h_mats, (size_t)bt->n_mats * sizeof(MatIO), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "batch table upload");
        bt->mats_valid = true;
    }
    if (bt->exec) {
        e = cudaGraphLaunch(bt->exec, s);
        if (e != cudaSuccess) return cuda_fail(e, "batch graph launch");
    } else if ((rc = batch_launch(bt, s))) {
        return rc;
    }
    e = cudaEventRecord(bt->done, s);
    if (e != cudaSuccess) return cuda_fail(e, "batch event record");
    return SABLE_OK;
}

int sable_batch_check(sable_batch *bt, void *stream) {
    if (!bt) return fail(SABLE_ERR_ARG, "null batch");
    int rc = set_device(bt->device);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, bt->d_error, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "batch check");
    if (flag) {
        cudaMemsetAsync(bt->d_error, 0, sizeof(int), s);
        cudaStreamSynchronize(s);
        return fail(SABLE_ERR_TIMEOUT, "a bounded device wait ran out (or a record failed its check) in the batch");
    }
    return SABLE_OK;
}

int sable_batch_get_info(const sable_batch *bt, sable_batch_info *out) {
    if (!bt || !out) return fail(SABLE_ERR_ARG, "null argument");
    out->n_mats = bt->n_mats;
    out->n_ctas = bt->n_ctas;
    out->n_units = bt->n_units;
    out->device_bytes = bt->device_bytes;
    out->smem_bytes = bt->smem;
    out->stage_bytes = bt->stage_bytes;
    out->stages = bt->stages;
    return SABLE_OK;
}

}  // extern "C"
