// Executor entry points of the C ABI: plan upload / destroy, SpMV and SpMM
// launches (device and host-buffer forms), timed variants, error check.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace sable {

template <typename T>
static int upload_vec(T **dptr, const T *h, size_t n, const char *what, int64_t *bytes_acc) {
    *dptr = nullptr;
    size_t bytes = n * sizeof(T);
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc((void **)dptr, bytes);
    if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "cudaMalloc %s (%zu bytes): %s", what, bytes, cudaGetErrorString(e));
    *bytes_acc += (int64_t)bytes;
    if (n) {
        e = cudaMemcpy(*dptr, h, n * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, what);
    } else {
        e = cudaMemset(*dptr, 0, bytes);
        if (e != cudaSuccess) return cuda_fail(e, what);
    }
    return SABLE_OK;
}

static int build_tc_planes(sable_plan *p, const Layout &L, int64_t *bytes);
static int build_umma_planes(sable_plan *p, const Layout &L, int64_t *bytes);


int plan_upload(sable_plan *p, const Layout &L) {
    p->n_rows = L.n_rows;
    p->n_cols = L.n_cols;
    p->n_items = (int64_t)L.items.size();
    p->n_partial = L.n_partial;
    p->n_split_tiles = L.n_split_tiles;
    p->max_item_bytes = std::max(L.max_item_bytes, 64);
    p->max_xg_floats = std::max(L.max_xg_floats, 4);
    p->records_bytes = (int64_t)L.records.size();
    p->compact = L.compact;
    int64_t bytes = 0;
    int rc;
    // item table, largest first (one CTA per item launches and the timed form)
    std::vector<int> desc_order(L.items.size());
    for (size_t i = 0; i < desc_order.size(); ++i) desc_order[i] = (int)i;
    std::stable_sort(desc_order.begin(), desc_order.end(),
                     [&](int a, int b) { return L.items[a].cost > L.items[b].cost; });
    std::vector<ItemRef> table;
    p->item_tile.clear();
    for (int i : desc_order) {
        table.push_back(L.items[i]);
        p->item_tile.push_back(L.item_tile[i]);
    }
    p->items_host = table;
    // persistent schedule: parts of tiles, greedy LPT over SMs x resident warp workers
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, p->device);
    const int per_sm = std::max(1, spmv_warp_workers_per_sm(p->max_item_bytes, p->max_xg_floats));
    int64_t total_bytes = 0;
    for (const ItemRef &r : L.items) total_bytes += r.bytes;
    const int64_t workers = (int64_t)dev_sms * per_sm;
    // parts of about a quarter of a worker's mean load keep LPT balanced
    const int64_t part_bytes = std::max<int64_t>(p->item_bytes, total_bytes / std::max<int64_t>(1, 4 * workers));
    std::vector<WorkRef> work;
    std::vector<int> wbegin;
    int64_t pp_floats = 0;
    build_warp_schedule(L, (int)workers, part_bytes, work, wbegin, pp_floats, p->n_multi, p->n_parts);
    p->n_ctas = (int)workers;
    if ((rc = upload_vec(&p->d_records, L.records.data(), L.records.size(), "records", &bytes))) return rc;
    if ((rc = upload_vec(&p->d_items, table.data(), table.size(), "item table", &bytes))) return rc;
    if ((rc = upload_vec(&p->d_work, work.data(), work.size(), "worker lists", &bytes))) return rc;
    if ((rc = upload_vec(&p->d_cta_begin, wbegin.data(), wbegin.size(), "schedule", &bytes))) return rc;
    std::vector<float> pp((size_t)std::max<int64_t>(pp_floats, 1), 0.f);
    if ((rc = upload_vec(&p->d_ppartial, pp.data(), pp.size(), "part partials", &bytes))) return rc;
    std::vector<int> pc((size_t)std::max<int64_t>(p->n_multi, 1), 0);
    if ((rc = upload_vec(&p->d_pcounters, pc.data(), pc.size(), "part counters", &bytes))) return rc;
    std::vector<float> part((size_t)std::max<int64_t>(L.n_partial, 1), 0.f);
    if ((rc = upload_vec(&p->d_partial, part.data(), part.size(), "partial", &bytes))) return rc;
    std::vector<int> cnt((size_t)std::max<int32_t>(L.n_split_tiles, 1), 0);
    if ((rc = upload_vec(&p->d_counters, cnt.data(), cnt.size(), "counters", &bytes))) return rc;
    p->splits_host = L.splits;
    if (!L.splits.empty() && (rc = upload_vec(&p->d_splits, L.splits.data(), L.splits.size(), "split tiles", &bytes)))
        return rc;
    std::vector<int> err(4, 0);
    if ((rc = upload_vec(&p->d_error, err.data(), err.size(), "error flag", &bytes))) return rc;
    int dev_max = 0;
    cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
    // Plans whose items are too large for a warp worker's ring run one CTA per item.
    if (p->schedule == SABLE_SCHEDULE_PERSISTENT && spmv_warp_smem(p->max_item_bytes, p->max_xg_floats) > dev_max)
        p->schedule = SABLE_SCHEDULE_ITEMS;
    // Records too large to stage in shared memory (items above ~96 KB, for
    // SpMM's long K loops) leave an SpMM-only plan: the SpMM kernels stream
    // records in K steps, the SpMV and batch executors stage whole records.
    p->staged_ok = p->compact || (p->max_item_bytes <= SABLE_MAX_ITEM_BYTES &&
                                  spmv_items_smem(p->max_item_bytes, p->max_xg_floats + 4) <= dev_max);
    p->stats.n_tiles = L.n_tiles;
    p->stats.n_chunks = p->n_items;
    p->stats.dense_values = L.dense_values;
    p->stats.dense_padded = L.dense_padded;
    p->stats.sparse_nnz = L.sparse_nnz;
    // split-BF16 SpMM: the panel terms of the tcgen05 kernel, and the
    // m16n8k16 fragments of the mma.sync kernel (also what batches read)
    if (p->spmm_tc != SABLE_TC_OFF && !L.compact) {
        if (p->tc_kernel == SABLE_TC_KERNEL_UMMA && (rc = build_umma_planes(p, L, &bytes))) return rc;
        if ((rc = build_tc_planes(p, L, &bytes))) return rc;
    }
    p->stats.device_bytes = bytes;
    p->stats.scratch_floats = L.n_partial;
    return SABLE_OK;
}

// Round to nearest even FP32 -> BF16 (bit pattern); NaN stays a quiet NaN.
static uint16_t bf16_rn(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

static float bf16_value(uint16_t b) {
    const uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Split-BF16 SpMM: every item's dense panel split once into BF16 terms
// (t_k = bf16(v - t_0 - ... - t_{k-1}), round to nearest even, the same split
// the tensor-core kernel otherwise does per K step) and laid out as the
// m16n8k16 A fragments of each lane: for K step ks (16 panel columns) and M
// tile mt (16 rows), TC_TERMS x 32 words of 16 bytes, word (ks, mt, term,
// lane) = the four BF16 pairs (rows 16mt + g and + 8, columns 16ks + 2t,
// + 1 and + 8, + 9; g = lane / 4, t = lane % 4; zero outside the panel).
static int build_tc_planes(sable_plan *p, const Layout &L, int64_t *bytes) {
    constexpr int TERMS = 3;
    const std::vector<ItemRef> &table = p->items_host;
    std::vector<int64_t> off(table.size(), 0);
    std::vector<uint32_t> words;  // 4 per 16-byte word
    for (size_t idx = 0; idx < table.size(); ++idx) {
        const unsigned char *R = L.records.data() + table[idx].off;
        ItemHeader hd;
        memcpy(&hd, R, sizeof hd);
        off[idx] = (int64_t)(words.size() / 4);
        if (hd.nq <= 0) continue;
        const float *P = reinterpret_cast<const float *>(R + hd.panel_off);
        const int h = hd.h, ncol = 4 * hd.nq, nks = (ncol + 15) / 16, mtiles = (h + 15) / 16;
        auto A = [&](int i, int c) -> float {
            return (i < h && c < ncol) ? P[((int64_t)(c >> 2) * h + i) * 4 + (c & 3)] : 0.f;
        };
        const size_t base = words.size();
        words.resize(base + (size_t)nks * mtiles * TERMS * 32 * 4, 0u);
        for (int ks = 0; ks < nks; ++ks)
            for (int mt = 0; mt < mtiles; ++mt)
                for (int lane = 0; lane < 32; ++lane) {
                    const int g = lane >> 2, t = lane & 3, r0 = 16 * mt + g, c0 = 16 * ks + 2 * t;
                    const float v[4][2] = {{A(r0, c0), A(r0, c0 + 1)}, {A(r0 + 8, c0), A(r0 + 8, c0 + 1)},
                                           {A(r0, c0 + 8), A(r0, c0 + 9)}, {A(r0 + 8, c0 + 8), A(r0 + 8, c0 + 9)}};
                    for (int reg = 0; reg < 4; ++reg) {
                        float a0 = v[reg][0], a1 = v[reg][1];
                        for (int k = 0; k < TERMS; ++k) {
                            const uint16_t b0 = bf16_rn(a0), b1 = bf16_rn(a1);
                            a0 -= bf16_value(b0);
                            a1 -= bf16_value(b1);
                            const size_t w = base + ((((size_t)ks * mtiles + mt) * TERMS + k) * 32 + lane) * 4 + reg;
                            words[w] = (uint32_t)b0 | ((uint32_t)b1 << 16);
                        }
                    }
                }
    }
    if (words.empty()) return SABLE_OK;
    int rc = upload_vec(reinterpret_cast<uint32_t **>(&p->d_tcplanes), words.data(), words.size(), "split-BF16 panels",
                        bytes);
    if (rc) return rc;
    p->tcoff_host = off;
    p->tc_words = (int64_t)(words.size() / 4);
    return upload_vec(&p->d_tcoff, off.data(), off.size(), "split-BF16 offsets", bytes);
}

// Split-BF16 SpMM on tcgen05: every item's dense panel split once into three
// BF16 terms (t_k = bf16(v - t_0 - ... - t_{k-1}), round to nearest even) and
// laid out as the B operand of the transposed product (umma.cuh, K-major, no
// swizzle): per K step ks (16 panel columns) and term t, one block of hp x 32
// bytes (hp = tile rows rounded up to 16) in which element (row n, column k)
// sits at byte (n & 7) * 16 + (n >> 3) * 256 + (k & 7) * 2 + (k >> 3) * 128;
// zeros outside the panel.  An item's blocks are contiguous, [ks][t].
static int build_umma_planes(sable_plan *p, const Layout &L, int64_t *bytes) {
    constexpr int TERMS = 3;
    const std::vector<ItemRef> &table = p->items_host;
    std::vector<int64_t> off(table.size(), -1);
    int64_t total = 0;
    for (size_t idx = 0; idx < table.size(); ++idx) {
        ItemHeader hd;
        memcpy(&hd, L.records.data() + table[idx].off, sizeof hd);
        if (hd.nq <= 0) continue;
        const int64_t hp = (hd.h + 15) & ~15, nks = (4 * (int64_t)hd.nq + 15) / 16;
        p->umma_hp = std::max<int>(p->umma_hp, (int)hp);
        off[idx] = total;
        total += nks * TERMS * hp * 32;
    }
    if (total == 0) return SABLE_OK;
    std::vector<unsigned char> buf((size_t)total, 0);
    for (size_t idx = 0; idx < table.size(); ++idx) {
        if (off[idx] < 0) continue;
        const unsigned char *R = L.records.data() + table[idx].off;
        ItemHeader hd;
        memcpy(&hd, R, sizeof hd);
        const float *P = reinterpret_cast<const float *>(R + hd.panel_off);
        const int h = hd.h, ncol = 4 * hd.nq, hp = (h + 15) & ~15;
        unsigned char *dst = buf.data() + off[idx];
        for (int c = 0; c < ncol; ++c) {
            const int ks = c >> 4, k = c & 15;
            for (int n = 0; n < h; ++n) {
                float v = P[((int64_t)(c >> 2) * h + n) * 4 + (c & 3)];
                const int e = (n & 7) * 16 + (n >> 3) * 256 + (k & 7) * 2 + (k >> 3) * 128;
                for (int t = 0; t < TERMS; ++t) {
                    const uint16_t b = bf16_rn(v);
                    v -= bf16_value(b);
                    memcpy(dst + ((int64_t)ks * TERMS + t) * hp * 32 + e, &b, 2);
                }
            }
        }
    }
    int rc = upload_vec(&p->d_umma, buf.data(), buf.size(), "split-BF16 panel terms", bytes);
    if (rc) return rc;
    p->umma_off_host = off;
    p->umma_bytes = total;
    return upload_vec(&p->d_umma_off, off.data(), off.size(), "split-BF16 term offsets", bytes);
}

LaunchArgs spmv_args(const sable_plan *p, const float *x, float *y, int64_t *cycles) {
    LaunchArgs a;
    memset(&a, 0, sizeof a);
    a.records = p->d_records;
    a.items = p->d_items;
    a.work = p->d_work;
    a.cta_begin = p->d_cta_begin;
    a.mats = nullptr;
    a.mat0.x = x;
    a.mat0.y = y;
    a.mat0.partial = p->d_partial;
    a.mat0.counters = p->d_counters;
    a.mat0.ppartial = p->d_ppartial;
    a.mat0.pcounters = p->d_pcounters;
    a.mat0.ldx = 1;
    a.mat0.ldy = 1;
    a.mat0.N = 1;
    a.cycles = cycles;
    a.error = p->d_error;
    a.n_items = (int)p->n_items;
    a.stage_bytes = p->max_item_bytes;
    a.xg_floats = (p->max_xg_floats + 3) & ~3;
    return a;
}

static int run_spmv(sable_plan *p, const float *x, float *y, int64_t *cycles, void *stream) {
    if (!p || !x || !y) return fail(SABLE_ERR_ARG, "null argument");
    if (!p->staged_ok)
        return fail(SABLE_ERR_UNSUPPORTED, "work items of %d bytes: an SpMM-only plan (SpMV stages items of at most %d bytes)",
                    p->max_item_bytes, SABLE_MAX_ITEM_BYTES);
    int rc = set_device(p->device);
    if (rc) return rc;
    LaunchArgs a = spmv_args(p, x, y, cycles);
    int e;
    if (p->schedule == SABLE_SCHEDULE_WARP_ITEMS) {
        e = launch_spmv_warp_items(a, cycles != nullptr, stream);  // combines split tiles itself
    } else if (cycles || p->schedule == SABLE_SCHEDULE_ITEMS) {
        e = launch_spmv_items(a, cycles != nullptr, stream);
        if (!e && p->n_split_tiles > 0) e = launch_spmv_combine(p->d_splits, p->n_split_tiles, nullptr, a.mat0, stream);
    } else {
        e = launch_spmv_warps(a, p->n_ctas, stream);
    }
    if (e) return cuda_fail((cudaError_t)e, "spmv launch");
    return SABLE_OK;
}

static int ensure_spmm_scratch(sable_plan *p, int nt, int n_slices) {
    const int64_t need = std::max<int64_t>(1, p->n_partial * nt * n_slices);
    if (need > p->spmm_partial_cap) {
        if (p->d_spmm_partial) cudaFree(p->d_spmm_partial);
        p->d_spmm_partial = nullptr;
        p->spmm_partial_cap = 0;
        cudaError_t e = cudaMalloc((void **)&p->d_spmm_partial, need * sizeof(float));
        if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "SpMM scratch: %s", cudaGetErrorString(e));
        p->spmm_partial_cap = need;
    }
    const int64_t needc = std::max<int64_t>(1, (int64_t)std::max<int32_t>(p->n_split_tiles, 1) * n_slices);
    if (needc > p->spmm_counters_cap) {
        if (p->d_spmm_counters) cudaFree(p->d_spmm_counters);
        p->d_spmm_counters = nullptr;
        p->spmm_counters_cap = 0;
        cudaError_t e = cudaMalloc((void **)&p->d_spmm_counters, needc * sizeof(int));
        if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "SpMM counters: %s", cudaGetErrorString(e));
        e = cudaMemset(p->d_spmm_counters, 0, needc * sizeof(int));
        if (e != cudaSuccess) return cuda_fail(e, "SpMM counters memset");
        p->spmm_counters_cap = needc;
    }
    return SABLE_OK;
}

void spmm_tc_free(sable_plan *p);

static int run_spmm(sable_plan *p, const float *X, int64_t ldx, float *Y, int64_t ldy, int N, int64_t *cycles,
                    void *stream) {
    if (!p || !X || !Y) return fail(SABLE_ERR_ARG, "null argument");
    if (N <= 0 || (N & 3) || (ldx & 3) || (ldy & 3) || ldx < N || ldy < N)
        return fail(SABLE_ERR_UNSUPPORTED, "SpMM needs N %% 4 == 0 and ld >= N, ld %% 4 == 0 (N=%d ldx=%lld ldy=%lld)", N,
                    (long long)ldx, (long long)ldy);
    if (((uintptr_t)X & 15) || ((uintptr_t)Y & 15)) return fail(SABLE_ERR_UNSUPPORTED, "SpMM operands must be 16-byte aligned");
    if (p->compact) return fail(SABLE_ERR_UNSUPPORTED, "a plan of the per-warp SpMV executor (schedule 2) runs SpMV only");
    int rc = set_device(p->device);
    if (rc) return rc;
    const int nt = spmm_slice_width(N);
    const int n_slices = (N + nt - 1) / nt;
    rc = ensure_spmm_scratch(p, nt, n_slices);
    if (rc) return rc;
    LaunchArgs a;
    memset(&a, 0, sizeof a);
    a.records = p->d_records;
    a.items = p->d_items;
    a.mat0.x = X;
    a.mat0.y = Y;
    a.mat0.partial = p->d_spmm_partial;
    a.mat0.counters = p->d_spmm_counters;
    a.mat0.ldx = ldx;
    a.mat0.ldy = ldy;
    a.mat0.N = N;
    a.mat0.pad = std::max<int32_t>(p->n_split_tiles, 1);  // counters per N-slice
    a.cycles = cycles;
    a.error = p->d_error;
    a.n_items = (int)p->n_items;
    a.stage_bytes = p->max_item_bytes;
    (void)n_slices;
    const int e = launch_spmm_plan(p, a, N, nt, cycles != nullptr, stream);
    if (e) return cuda_fail((cudaError_t)e, "spmm launch");
    return SABLE_OK;
}

// The SpMM kernel of a plan at width N: dense blocks on the tensor cores
// (split BF16) when the plan was built with them and N >= 32, else on the
// FP32 CUDA cores.  `a` carries the operands and the scratch.
int launch_spmm_plan(const sable_plan *p, LaunchArgs &a, int N, int nt, bool timed, void *stream) {
    a.tcplanes = p->d_tcplanes;
    a.tcoff = p->d_tcoff;
    a.umma = p->d_umma;
    a.umma_off = p->d_umma_off;
    a.umma_hp = p->umma_hp;
    const int64_t part_stride = p->n_partial * nt;
    if (p->spmm_tc && N >= 32) {
        const int terms = p->spmm_tc == SABLE_TC_SPLIT3 ? 3 : 2;
        if (p->tc_kernel == SABLE_TC_KERNEL_UMMA && p->d_umma)
            return launch_spmm_umma(a, N, nt, terms, part_stride, timed, stream);
        return launch_spmm_tc(a, N, nt, terms, part_stride, timed, stream);
    }
    return launch_spmm_fp32(a, N, nt, part_stride, timed, stream);
}

static int ensure_host_staging(sable_plan *p, int64_t nx, int64_t ny) {
    if (nx > p->dx_cap) {
        if (p->d_x) cudaFree(p->d_x);
        p->d_x = nullptr;
        p->dx_cap = 0;
        cudaError_t e = cudaMalloc((void **)&p->d_x, nx * sizeof(float));
        if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "staging x: %s", cudaGetErrorString(e));
        p->dx_cap = nx;
    }
    if (ny > p->dy_cap) {
        if (p->d_y) cudaFree(p->d_y);
        p->d_y = nullptr;
        p->dy_cap = 0;
        cudaError_t e = cudaMalloc((void **)&p->d_y, ny * sizeof(float));
        if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "staging y: %s", cudaGetErrorString(e));
        p->dy_cap = ny;
    }
    return SABLE_OK;
}

}  // namespace sable

using namespace sable;

extern "C" {

int sable_plan_destroy(sable_plan *p) {
    if (!p) return SABLE_OK;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(p->device);
    if (p->host_exec) cudaGraphExecDestroy(p->host_exec);
    cudaFree(p->d_records);
    cudaFree(p->d_items);
    cudaFree(p->d_work);
    cudaFree(p->d_cta_begin);
    cudaFree(p->d_ppartial);
    cudaFree(p->d_pcounters);
    cudaFree(p->d_partial);
    cudaFree(p->d_counters);
    cudaFree(p->d_splits);
    cudaFree(p->d_error);
    cudaFree(p->d_spmm_partial);
    cudaFree(p->d_spmm_counters);
    cudaFree(p->d_x);
    cudaFree(p->d_y);
    spmm_tc_free(p);
    cudaFree(p->d_umma);
    cudaFree(p->d_umma_off);
    if (prev >= 0) cudaSetDevice(prev);
    delete p;
    return SABLE_OK;
}

int sable_plan_check(sable_plan *p, void *stream) {
    if (!p) return fail(SABLE_ERR_ARG, "null plan");
    int rc = set_device(p->device);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, p->d_error, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "plan check");
    if (flag) {
        cudaMemsetAsync(p->d_error, 0, sizeof(int), s);
        cudaStreamSynchronize(s);
        return fail(SABLE_ERR_TIMEOUT, "a bounded device wait ran out in an earlier launch of this plan");
    }
    return SABLE_OK;
}

int sable_spmv(sable_plan *plan, const float *x_dev, float *y_dev, void *stream) {
    return run_spmv(plan, x_dev, y_dev, nullptr, stream);
}

int sable_spmv_timed(sable_plan *plan, const float *x_dev, float *y_dev, int64_t *cycles_dev, void *stream) {
    if (!cycles_dev) return fail(SABLE_ERR_ARG, "null cycles buffer");
    return run_spmv(plan, x_dev, y_dev, cycles_dev, stream);
}

// Device address of pinned (page-locked, mapped) host memory, or nullptr for
// any other pointer (pageable memory, device memory).
static void *mapped_host(const void *ptr) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// The graph of sable_spmv_host for pinned x / y (device addresses xm / ym):
// kept while the pair and the plan's x staging stay the same, captured on a
// private stream otherwise (the caller's stream is never put in capture).
static int host_graph(sable_plan *p, const float *xm, float *ym) {
    if (p->host_exec && p->host_x == xm && p->host_y == ym && p->host_dx == p->d_x) return SABLE_OK;
    if (p->host_exec) cudaGraphExecDestroy(p->host_exec);
    p->host_exec = nullptr;
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "host graph stream");
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SABLE_OK;
    if (e == cudaSuccess) {
        const int ec = launch_copy_floats(p->d_x, xm, p->n_cols, cs);
        rc = ec ? cuda_fail((cudaError_t)ec, "copy x to device (capture)") : run_spmv(p, p->d_x, ym, nullptr, cs);
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e2 != cudaSuccess && !rc) rc = cuda_fail(e2, "host graph capture");
    } else {
        rc = cuda_fail(e, "host graph capture");
    }
    if (!rc) {
        e = cudaGraphInstantiate(&p->host_exec, g, 0);
        if (e != cudaSuccess) {
            p->host_exec = nullptr;
            rc = cuda_fail(e, "host graph instantiate");
        }
    }
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    p->host_x = xm;
    p->host_y = ym;
    p->host_dx = p->d_x;
    return SABLE_OK;
}

int sable_spmv_host(sable_plan *p, const float *x_host, float *y_host, void *stream) {
    if (!p || !x_host || !y_host) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(p->device);
    if (rc) return rc;
    if ((rc = ensure_host_staging(p, p->n_cols, p->n_rows))) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Pinned host buffers are read and written by the kernels themselves
    // (one copy kernel for x, the SpMV's own stores for y): no copy-engine
    // transfer and its setup on either side.  Other buffers go through
    // cudaMemcpyAsync and the plan's device staging.
    const float *xm = static_cast<const float *>(mapped_host(x_host));
    float *ym = static_cast<float *>(mapped_host(y_host));
    cudaError_t e = cudaSuccess;
    if (xm && ym) {
        // both buffers pinned: one graph launch for the copy of x and the
        // SpMV (7-8 % less time per call than launching them one by one)
        if ((rc = host_graph(p, xm, ym))) return rc;
        e = cudaGraphLaunch(p->host_exec, s);
        if (e != cudaSuccess) return cuda_fail(e, "host graph launch");
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
        return SABLE_OK;
    }
    if (xm) {
        if ((rc = launch_copy_floats(p->d_x, xm, p->n_cols, stream))) return cuda_fail((cudaError_t)rc, "copy x to device");
    } else {
        e = cudaMemcpyAsync(p->d_x, x_host, (size_t)p->n_cols * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "copy x to device");
    }
    if ((rc = run_spmv(p, p->d_x, ym ? ym : p->d_y, nullptr, stream))) return rc;
    if (!ym) {
        e = cudaMemcpyAsync(y_host, p->d_y, (size_t)p->n_rows * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_fail(e, "copy y to host");
    }
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
    return SABLE_OK;
}

int sable_spmm(sable_plan *plan, const float *X_dev, int64_t ldx, float *Y_dev, int64_t ldy, int32_t N, void *stream) {
    return run_spmm(plan, X_dev, ldx, Y_dev, ldy, N, nullptr, stream);
}

int sable_spmm_timed(sable_plan *plan, const float *X_dev, float *Y_dev, int32_t N, int64_t *cycles_dev, void *stream) {
    if (!cycles_dev) return fail(SABLE_ERR_ARG, "null cycles buffer");
    return run_spmm(plan, X_dev, N, Y_dev, N, N, cycles_dev, stream);
}

int sable_spmm_host(sable_plan *p, const float *X_host, float *Y_host, int32_t N, void *stream) {
    if (!p || !X_host || !Y_host) return fail(SABLE_ERR_ARG, "null argument");
    if (N <= 0) return fail(SABLE_ERR_ARG, "N must be positive");
    int rc = set_device(p->device);
    if (rc) return rc;
    if ((rc = ensure_host_staging(p, (int64_t)p->n_cols * N, (int64_t)p->n_rows * N))) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(p->d_x, X_host, (size_t)p->n_cols * N * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "copy X to device");
    if ((rc = run_spmm(p, p->d_x, N, p->d_y, N, N, nullptr, stream))) return rc;
    e = cudaMemcpyAsync(Y_host, p->d_y, (size_t)p->n_rows * N * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "copy Y to host");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
    return SABLE_OK;
}

}  // extern "C"
