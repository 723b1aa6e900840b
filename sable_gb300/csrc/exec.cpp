// Executor entry points of the C ABI: plan upload / destroy, SpMV and SpMM
// launches (device and host-buffer forms), timed variants.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace sable {

template <typename T>
static int upload_vec(T **dptr, const std::vector<T> &h, const char *what, int64_t *bytes_acc) {
    *dptr = nullptr;
    size_t bytes = h.size() * sizeof(T);
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc((void **)dptr, bytes);
    if (e != cudaSuccess) return fail(SABLE_ERR_NOMEM, "cudaMalloc %s (%zu bytes): %s", what, bytes, cudaGetErrorString(e));
    *bytes_acc += (int64_t)bytes;
    if (!h.empty()) {
        e = cudaMemcpy(*dptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, what);
    }
    return SABLE_OK;
}

int plan_upload(sable_plan *p, const Layout &L) {
    p->n_rows = L.n_rows;
    p->n_cols = L.n_cols;
    p->n_chunks = (int64_t)L.chunks.size();
    p->n_partial = L.n_partial;
    p->n_split_tiles = L.n_split_tiles;
    p->max_quads = L.max_quads;
    p->max_runs = L.max_runs;
    p->chunk_tile = L.chunk_tile;
    int64_t bytes = 0;
    int rc;
    if ((rc = upload_vec(&p->d_panel, L.panel, "panel", &bytes))) return rc;
    if ((rc = upload_vec(&p->d_sparse, L.sparse, "sparse", &bytes))) return rc;
    if ((rc = upload_vec(&p->d_runs, L.runs, "runs", &bytes))) return rc;
    if ((rc = upload_vec(&p->d_chunks, L.chunks, "chunks", &bytes))) return rc;
    std::vector<float> part((size_t)std::max<int64_t>(L.n_partial, 1), 0.f);
    if ((rc = upload_vec(&p->d_partial, part, "partial", &bytes))) return rc;
    std::vector<int> cnt((size_t)std::max<int32_t>(L.n_split_tiles, 1), 0);
    if ((rc = upload_vec(&p->d_counters, cnt, "counters", &bytes))) return rc;
    p->stats.n_tiles = L.n_tiles;
    p->stats.n_chunks = p->n_chunks;
    p->stats.dense_values = L.dense_values;
    p->stats.dense_padded = (int64_t)L.panel.size() * 4;
    p->stats.sparse_nnz = L.sparse_nnz;
    p->stats.device_bytes = bytes;
    p->stats.scratch_floats = L.n_partial;
    return SABLE_OK;
}

SpmvArgs spmv_args(const sable_plan *p, const float *x, float *y, int64_t *cycles) {
    SpmvArgs a;
    memset(&a, 0, sizeof a);
    a.chunks = p->d_chunks;
    a.panel = p->d_panel;
    a.sparse = p->d_sparse;
    a.runs = p->d_runs;
    a.x = x;
    a.y = y;
    a.partial = p->d_partial;
    a.counters = p->d_counters;
    a.ns_out = cycles;
    a.n_chunks = (int)p->n_chunks;
    return a;
}

static int run_spmv(sable_plan *p, const float *x, float *y, int64_t *cycles, void *stream) {
    if (!p || !x || !y) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(p->device);
    if (rc) return rc;
    SpmvArgs a = spmv_args(p, x, y, cycles);
    int e = launch_spmv(a, spmv_smem_bytes(p->max_quads, p->max_runs), cycles != nullptr, stream);
    if (e) return cuda_fail((cudaError_t)e, "spmv launch");
    return SABLE_OK;
}

static int pick_nt(int N) {
    int nt = 4;
    while (nt < N && nt < 128) nt <<= 1;
    return nt;
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
    const int64_t needc = std::max<int64_t>(1, p->n_chunks * n_slices);
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

int spmm_tc_run(sable_plan *p, const float *X, int64_t ldx, float *Y, int64_t ldy, int N, int64_t *cycles,
                void *stream, bool *handled);
void spmm_tc_free(sable_plan *p);

static int run_spmm(sable_plan *p, const float *X, int64_t ldx, float *Y, int64_t ldy, int N, int64_t *cycles,
                    void *stream) {
    if (!p || !X || !Y) return fail(SABLE_ERR_ARG, "null argument");
    if (N <= 0 || (N & 3) || (ldx & 3) || (ldy & 3) || ldx < N || ldy < N)
        return fail(SABLE_ERR_UNSUPPORTED, "SpMM needs N %% 4 == 0 and ld >= N, ld %% 4 == 0 (N=%d ldx=%lld ldy=%lld)", N,
                    (long long)ldx, (long long)ldy);
    if (((uintptr_t)X & 15) || ((uintptr_t)Y & 15)) return fail(SABLE_ERR_UNSUPPORTED, "SpMM operands must be 16-byte aligned");
    int rc = set_device(p->device);
    if (rc) return rc;
    if (p->spmm_tc && N >= 32) {
        bool handled = false;
        rc = spmm_tc_run(p, X, ldx, Y, ldy, N, cycles, stream, &handled);
        if (rc || handled) return rc;
    }
    const int nt = pick_nt(N);
    const int n_slices = (N + nt - 1) / nt;
    rc = ensure_spmm_scratch(p, nt, n_slices);
    if (rc) return rc;
    SpmmArgs a;
    memset(&a, 0, sizeof a);
    a.chunks = p->d_chunks;
    a.panel = p->d_panel;
    a.sparse = p->d_sparse;
    a.runs = p->d_runs;
    a.X = X;
    a.Y = Y;
    a.partial = p->d_spmm_partial;
    a.counters = p->d_spmm_counters;
    a.ns_out = cycles;
    a.ldx = ldx;
    a.ldy = ldy;
    a.N = N;
    a.nt = nt;
    a.n_slices = n_slices;
    a.n_chunks = (int)p->n_chunks;
    a.part_stride = p->n_partial * nt;
    int e = launch_spmm_fp32(a, spmm_smem_bytes(nt, p->max_quads, p->max_runs, p->row_tile), cycles != nullptr, stream);
    if (e) return cuda_fail((cudaError_t)e, "spmm launch");
    return SABLE_OK;
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
    cudaFree(p->d_panel);
    cudaFree(p->d_sparse);
    cudaFree(p->d_runs);
    cudaFree(p->d_chunks);
    cudaFree(p->d_partial);
    cudaFree(p->d_counters);
    cudaFree(p->d_spmm_partial);
    cudaFree(p->d_spmm_counters);
    cudaFree(p->d_x);
    cudaFree(p->d_y);
    spmm_tc_free(p);
    if (prev >= 0) cudaSetDevice(prev);
    delete p;
    return SABLE_OK;
}

int sable_spmv(sable_plan *plan, const float *x_dev, float *y_dev, void *stream) {
    return run_spmv(plan, x_dev, y_dev, nullptr, stream);
}

int sable_spmv_timed(sable_plan *plan, const float *x_dev, float *y_dev, int64_t *cycles_dev, void *stream) {
    if (!cycles_dev) return fail(SABLE_ERR_ARG, "null cycles buffer");
    return run_spmv(plan, x_dev, y_dev, cycles_dev, stream);
}

int sable_spmv_host(sable_plan *p, const float *x_host, float *y_host, void *stream) {
    if (!p || !x_host || !y_host) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(p->device);
    if (rc) return rc;
    if ((rc = ensure_host_staging(p, p->n_cols, p->n_rows))) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(p->d_x, x_host, (size_t)p->n_cols * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "copy x to device");
    if ((rc = run_spmv(p, p->d_x, p->d_y, nullptr, stream))) return rc;
    e = cudaMemcpyAsync(y_host, p->d_y, (size_t)p->n_rows * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "copy y to host");
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
