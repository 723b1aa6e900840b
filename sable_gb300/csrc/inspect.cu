// The inspector steps upstream of the plan, on the GPU:
//
//   sable_vbr_from_csr     VBR construction from a CSR matrix and its
//                          partition (convert_sparse_to_vbr,
//                          utils/convert_real_to_vbr.py:98-199): every
//                          (rpntr x cpntr) block holding a stored entry is
//                          materialised dense, column-major, in block-row
//                          order, ascending block column.
//   sable_similarity_cuts  the row / column partition of cut_indices2 with
//                          similarity2 (src/autopartition.py:34-74, 87-89)
//                          or its numba variant (:91-107).
//
// VBR construction, per block row i (one CTA each, three passes):
//   count    a shared-memory bitmap of the block columns hit by the block
//            row's stored entries (the CSR rows of a block row are one
//            contiguous range of entries); its population count.
//   blocks   after an exclusive scan of the counts (bpntrb / bpntre): the
//            bitmap again, per-word prefix counts, one bindx entry and one
//            block size (h x w) per set bit; then a scan of the sizes (indx).
//   scatter  val zeroed, the bitmap and prefixes again, and one thread per
//            row walks its entries in CSR order adding each value at
//            indx[b] + (col - c0) h + (row - r0): duplicates of an entry sum
//            in CSR order, as the reference's dense materialisation does.
// Block rows without a stored entry get bpntrb = bpntre = -1 (the reference
// asserts that there are none).
//
// Similarity cuts: one warp per pair of adjacent lines (rows from the CSR,
// columns from the CSC given as the CSR of the transpose) computes, in FP64,
// dot0 = a.b, fwd = a[1:].b[:-1], bwd = a[:-1].b[1:] (a's entries looked up
// in b by binary search) and the nonzero counts of a and b.  The reference's
// sequential scan over lines reduces to a per-position predicate: position j
// (1 <= j < n) is a cut iff line j-1 is empty (no stored entry) and line j is
// not, or line j-1 is not empty and similarity(j-1, j) < threshold; 0 and n
// are always cuts.  A scan of the flags compacts the cut positions.
//
// All index arrays are validated on the host before upload, so every kernel
// index stays inside its buffer.  Values are FP32 or FP64 (value_bytes).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace {

constexpr int INSPECT_THREADS = 256;
constexpr int SCAN_CHUNK = 1024;   // elements per CTA of the scan (256 threads x 4)

// ---- exclusive scan of int64 (out[0..n], out[n] = total) ---------------------

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-level exclusive scan of SCAN_CHUNK elements per CTA; chunk totals to sums.
__global__ void scan_chunks_kernel(const int64_t *in, int64_t n, int64_t *out, int64_t *sums) {
    __shared__ int64_t s_warp[INSPECT_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK + (int64_t)tid * 4;
    int64_t v[4], t = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        t += v[i];
    }
    int64_t incl = warp_incl_scan(t, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < INSPECT_THREADS / 32 ? s_warp[lane] : 0;
        w = warp_incl_scan(w, lane);
        if (lane < INSPECT_THREADS / 32) s_warp[lane] = w;
    }
    __syncthreads();
    int64_t run = incl - t + (warp > 0 ? s_warp[warp - 1] : 0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (tid == INSPECT_THREADS - 1) sums[blockIdx.x] = run;
}

__global__ void scan_add_kernel(int64_t *out, int64_t n, const int64_t *offs) {
    const int64_t i = (int64_t)blockIdx.x * SCAN_CHUNK + threadIdx.x * 4;
    const int64_t add = offs[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (i + k < n) out[i + k] += add;
}

__global__ void set_total_kernel(int64_t *out, int64_t n, const int64_t *total) { out[n] = *total; }

// out[0..n] = exclusive scan of in[0..n), out[n] = sum; `tmp` is scratch of
// scan_tmp_len(n) int64.
int64_t scan_tmp_len(int64_t n) {
    int64_t len = 0;
    for (int64_t m = n; m > 1;) {
        const int64_t chunks = (m + SCAN_CHUNK - 1) / SCAN_CHUNK;
        len += 2 * chunks + 1;
        m = chunks;
    }
    return len + 2;
}

cudaError_t scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t s) {
    if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(int64_t), s);
    const int64_t chunks = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    int64_t *sums = tmp, *offs = tmp + chunks;
    scan_chunks_kernel<<<(unsigned)chunks, INSPECT_THREADS, 0, s>>>(in, n, out, sums);
    if (chunks == 1) {
        set_total_kernel<<<1, 1, 0, s>>>(out, n, sums);
        return cudaGetLastError();
    }
    cudaError_t e = scan_i64(sums, offs, chunks, tmp + 2 * chunks + 1, s);
    if (e != cudaSuccess) return e;
    scan_add_kernel<<<(unsigned)chunks, INSPECT_THREADS, 0, s>>>(out, n, offs);
    set_total_kernel<<<1, 1, 0, s>>>(out, n, offs + chunks);
    return cudaGetLastError();
}

// ---- VBR construction ----------------------------------------------------------

// col2bc[c] = block column of column c (binary search over cpntr).
__global__ void col_block_kernel(const int *cpntr, int nbc, int n_cols, int *col2bc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cols) return;
    int lo = 0, hi = nbc;   // last j with cpntr[j] <= c
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (cpntr[mid] <= c) lo = mid; else hi = mid;
    }
    col2bc[c] = lo;
}

// Bitmap of the block columns of block row i in shared memory (words words).
__device__ __forceinline__ void block_row_bitmap(const int64_t *indptr, const int *indices, const int *rpntr,
                                                 const int *col2bc, int i, unsigned *bm, int words) {
    for (int w = threadIdx.x; w < words; w += blockDim.x) bm[w] = 0u;
    __syncthreads();
    const int64_t e0 = indptr[rpntr[i]], e1 = indptr[rpntr[i + 1]];
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const int bc = col2bc[indices[e]];
        atomicOr(&bm[bc >> 5], 1u << (bc & 31));
    }
    __syncthreads();
}

__global__ void vbr_count_kernel(const int64_t *indptr, const int *indices, const int *rpntr, const int *col2bc,
                                 int words, int64_t *counts) {
    extern __shared__ unsigned bm[];
    __shared__ int s_warp[INSPECT_THREADS / 32];
    const int i = blockIdx.x;
    block_row_bitmap(indptr, indices, rpntr, col2bc, i, bm, words);
    int c = 0;
    for (int w = threadIdx.x; w < words; w += blockDim.x) c += __popc(bm[w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += s_warp[k];
        counts[i] = t;
    }
}

// Exclusive prefix of the bitmap words' population counts into pre[words]
// (thread t owns a contiguous range of words).
__device__ __forceinline__ void bitmap_prefix(const unsigned *bm, int words, int *pre) {
    __shared__ int s_part[INSPECT_THREADS];
    const int t = threadIdx.x, per = (words + blockDim.x - 1) / blockDim.x;
    const int w0 = min(words, t * per), w1 = min(words, w0 + per);
    int c = 0;
    for (int w = w0; w < w1; ++w) c += __popc(bm[w]);
    s_part[t] = c;
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            const int v = s_part[k];
            s_part[k] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = s_part[t];
    for (int w = w0; w < w1; ++w) {
        pre[w] = run;
        run += __popc(bm[w]);
    }
    __syncthreads();
}

__global__ void vbr_blocks_kernel(const int64_t *indptr, const int *indices, const int *rpntr, const int *cpntr,
                                  const int *col2bc, int words, const int64_t *bstart, int *bindx, int64_t *bsize,
                                  int *bpntrb, int *bpntre) {
    extern __shared__ unsigned bm[];
    int *pre = reinterpret_cast<int *>(bm + words);
    const int i = blockIdx.x;
    block_row_bitmap(indptr, indices, rpntr, col2bc, i, bm, words);
    bitmap_prefix(bm, words, pre);
    const int64_t b0 = bstart[i];
    const int64_t h = rpntr[i + 1] - rpntr[i];
    for (int w = threadIdx.x; w < words; w += blockDim.x) {
        unsigned bits = bm[w];
        int r = pre[w];
        while (bits) {
            const int bc = 32 * w + __ffs(bits) - 1;
            bits &= bits - 1;
            bindx[b0 + r] = bc;
            bsize[b0 + r] = h * (int64_t)(cpntr[bc + 1] - cpntr[bc]);
            ++r;
        }
    }
    if (threadIdx.x == 0) {
        const bool any = bstart[i + 1] > b0;
        bpntrb[i] = any ? (int)b0 : -1;
        bpntre[i] = any ? (int)bstart[i + 1] : -1;
    }
}

template <typename T>
__global__ void vbr_scatter_kernel(const int64_t *indptr, const int *indices, const T *data, const int *rpntr,
                                   const int *cpntr, const int *col2bc, int words, const int64_t *bstart,
                                   const int64_t *indx, T *val) {
    extern __shared__ unsigned bm[];
    int *pre = reinterpret_cast<int *>(bm + words);
    const int i = blockIdx.x;
    block_row_bitmap(indptr, indices, rpntr, col2bc, i, bm, words);
    bitmap_prefix(bm, words, pre);
    const int r0 = rpntr[i], h = rpntr[i + 1] - r0;
    const int64_t b0 = bstart[i];
    for (int rr = threadIdx.x; rr < h; rr += blockDim.x) {
        const int r = r0 + rr;
        for (int64_t e = indptr[r]; e < indptr[r + 1]; ++e) {
            const int c = indices[e], bc = col2bc[c];
            const unsigned word = bm[bc >> 5];
            const int rank = pre[bc >> 5] + __popc(word & ((1u << (bc & 31)) - 1u));
            const int64_t pos = indx[b0 + rank] + (int64_t)(c - cpntr[bc]) * h + rr;
            val[pos] += data[e];
        }
    }
}

// ---- similarity cuts -----------------------------------------------------------

// First position p in idx[0..n) with idx[p] >= key.
__device__ __forceinline__ int64_t lower_bound_i32(const int *idx, int64_t n, int key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (idx[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <typename T>
__global__ void similarity_flags_kernel(const int64_t *ptr, const int *idx, const T *data, int n_lines,
                                        double threshold, int mode, int64_t *flags) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp == 0 && lane == 0) {
        flags[0] = 1;
        flags[n_lines] = 1;
    }
    const int p = warp;   // pair (p, p + 1) decides position p + 1
    if (p >= n_lines - 1) return;
    const int64_t a0 = ptr[p], a1 = ptr[p + 1], b0 = ptr[p + 1], b1 = ptr[p + 2];
    const int64_t nb = b1 - b0;
    double dot0 = 0.0, fwd = 0.0, bwd = 0.0;
    int cnt_a = 0, cnt_b = 0;
    for (int64_t e = a0 + lane; e < a1; e += 32) {
        const int c = idx[e];
        const double va = (double)data[e];
        cnt_a += va != 0.0;
        int64_t q = lower_bound_i32(idx + b0, nb, c - 1);
        for (; q < nb && idx[b0 + q] <= c + 1; ++q) {
            const int cb = idx[b0 + q];
            const double vb = (double)data[b0 + q];
            if (cb == c - 1) fwd += va * vb;       // a[j+1] b[j]
            else if (cb == c) dot0 += va * vb;     // a[j] b[j]
            else bwd += va * vb;                   // a[j] b[j+1]
        }
    }
    for (int64_t e = b0 + lane; e < b1; e += 32) cnt_b += (double)data[e] != 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dot0 += __shfl_xor_sync(0xffffffffu, dot0, o);
        fwd += __shfl_xor_sync(0xffffffffu, fwd, o);
        bwd += __shfl_xor_sync(0xffffffffu, bwd, o);
        cnt_a += __shfl_xor_sync(0xffffffffu, cnt_a, o);
        cnt_b += __shfl_xor_sync(0xffffffffu, cnt_b, o);
    }
    if (lane != 0) return;
    const bool empty_a = a1 == a0, empty_b = b1 == b0;
    bool cut;
    if (empty_a) {
        cut = !empty_b;   // the end of a run of empty lines
    } else {
        double sim;
        const double best = fmax(fmax(dot0, fwd), bwd);
        const int denom = max(cnt_a, cnt_b);
        if (mode == 1 && (cnt_a == 0 || cnt_b == 0)) sim = 0.0;     // the numba variant
        else sim = best / (double)denom;                              // 0 / 0 is NaN: no cut
        cut = sim < threshold;
    }
    flags[p + 1] = cut ? 1 : 0;
}

__global__ void compact_kernel(const int64_t *flags, const int64_t *pos, int n, int *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j <= n && flags[j]) out[pos[j]] = j;
}

// ---- host helpers --------------------------------------------------------------

struct DevBufs {
    std::vector<void *> ptrs;
    ~DevBufs() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T>
    int alloc(T **p, size_t n, const char *what) {
        *p = nullptr;
        const size_t bytes = std::max<size_t>(16, n * sizeof(T));
        cudaError_t e = cudaMalloc((void **)p, bytes);
        if (e != cudaSuccess)
            return sable::fail(SABLE_ERR_NOMEM, "cudaMalloc %s (%zu bytes): %s", what, bytes, cudaGetErrorString(e));
        ptrs.push_back(*p);
        return SABLE_OK;
    }
    template <typename T>
    int upload(T **p, const T *h, size_t n, const char *what) {
        int rc = alloc(p, n, what);
        if (rc) return rc;
        if (n) {
            cudaError_t e = cudaMemcpy(*p, h, n * sizeof(T), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return sable::cuda_fail(e, what);
        }
        return SABLE_OK;
    }
};

int check_csr(const sable_csr_desc *m, const char *what) {
    if (!m) return sable::fail(SABLE_ERR_ARG, "%s: null descriptor", what);
    if (m->n_rows < 0 || m->n_cols < 0 || m->nnz < 0) return sable::fail(SABLE_ERR_INVALID, "%s: negative size", what);
    if (m->value_bytes != 4 && m->value_bytes != 8)
        return sable::fail(SABLE_ERR_ARG, "%s: value_bytes %d (4 or 8)", what, m->value_bytes);
    if (!m->indptr || (m->nnz > 0 && (!m->indices || !m->data)))
        return sable::fail(SABLE_ERR_ARG, "%s: null array", what);
    if (m->indptr[0] != 0 || m->indptr[m->n_rows] != m->nnz)
        return sable::fail(SABLE_ERR_INVALID, "%s: indptr must run from 0 to nnz", what);
    for (int32_t r = 0; r < m->n_rows; ++r) {
        if (m->indptr[r + 1] < m->indptr[r]) return sable::fail(SABLE_ERR_INVALID, "%s: indptr decreases at %d", what, r);
        for (int64_t e = m->indptr[r]; e < m->indptr[r + 1]; ++e) {
            const int32_t c = m->indices[e];
            if (c < 0 || c >= m->n_cols) return sable::fail(SABLE_ERR_INVALID, "%s: column %d out of range", what, c);
        }
    }
    return SABLE_OK;
}

int check_partition(const int32_t *p, int32_t nb, int32_t n, const char *what) {
    if (!p || nb < 0) return sable::fail(SABLE_ERR_ARG, "%s: null or negative", what);
    if (p[0] != 0 || p[nb] != n) return sable::fail(SABLE_ERR_INVALID, "%s must run from 0 to %d", what, n);
    for (int32_t i = 0; i < nb; ++i)
        if (p[i + 1] <= p[i]) return sable::fail(SABLE_ERR_INVALID, "%s must increase strictly (at %d)", what, i);
    return SABLE_OK;
}

}  // namespace

struct sable_vbr_build {
    int device = 0;
    int value_bytes = 8;
    int64_t n_blocks = 0, n_val = 0;
    int32_t n_block_rows = 0;
    void *d_val = nullptr;
    int64_t *d_indx = nullptr;
    int *d_bindx = nullptr, *d_bpntrb = nullptr, *d_bpntre = nullptr;
};

using namespace sable;

extern "C" {

int sable_vbr_from_csr(const sable_csr_desc *csr, int32_t n_block_rows, const int32_t *rpntr, int32_t n_block_cols,
                       const int32_t *cpntr, int32_t device, sable_vbr_build **out) {
    if (!out) return fail(SABLE_ERR_ARG, "null output pointer");
    *out = nullptr;
    int rc = check_csr(csr, "CSR");
    if (rc) return rc;
    if ((rc = check_partition(rpntr, n_block_rows, csr->n_rows, "rpntr"))) return rc;
    if ((rc = check_partition(cpntr, n_block_cols, csr->n_cols, "cpntr"))) return rc;
    const int words = (n_block_cols + 31) / 32;
    const size_t smem = (size_t)words * 8;   // bitmap + word prefixes
    int dev = device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(SABLE_ERR_CUDA, "no current device");
    if ((rc = set_device(dev))) return rc;
    int smem_max = 0;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem + 2 * INSPECT_THREADS * 4 > (size_t)smem_max)
        return fail(SABLE_ERR_UNSUPPORTED, "%d block columns: the per-block-row bitmap exceeds shared memory",
                    n_block_cols);
    const int n_rows = csr->n_rows, n_cols = csr->n_cols, vb = csr->value_bytes;
    DevBufs tmp;
    int64_t *d_indptr = nullptr, *d_counts = nullptr, *d_bstart = nullptr, *d_bsize = nullptr, *d_scan = nullptr;
    int *d_indices = nullptr, *d_rpntr = nullptr, *d_cpntr = nullptr, *d_col2bc = nullptr;
    unsigned char *d_data = nullptr;
    if ((rc = tmp.upload(&d_indptr, csr->indptr, (size_t)n_rows + 1, "indptr")) ||
        (rc = tmp.upload(&d_indices, csr->indices, (size_t)csr->nnz, "indices")) ||
        (rc = tmp.upload(&d_data, static_cast<const unsigned char *>(csr->data), (size_t)csr->nnz * vb, "values")) ||
        (rc = tmp.upload(&d_rpntr, rpntr, (size_t)n_block_rows + 1, "rpntr")) ||
        (rc = tmp.upload(&d_cpntr, cpntr, (size_t)n_block_cols + 1, "cpntr")) ||
        (rc = tmp.alloc(&d_col2bc, (size_t)n_cols, "column map")) ||
        (rc = tmp.alloc(&d_counts, (size_t)n_block_rows, "block counts")) ||
        (rc = tmp.alloc(&d_bstart, (size_t)n_block_rows + 1, "block starts")))
        return rc;
    const int64_t scan_len = scan_tmp_len(std::max<int64_t>(n_block_rows, 1));
    cudaStream_t s = 0;
    sable_vbr_build *b = new (std::nothrow) sable_vbr_build();
    if (!b) return fail(SABLE_ERR_NOMEM, "host allocation");
    b->device = dev;
    b->value_bytes = vb;
    b->n_block_rows = n_block_rows;
    auto bail = [&](int code) {
        sable_vbr_build_destroy(b);
        return code;
    };
    cudaError_t e = cudaSuccess;
    if (n_cols > 0) col_block_kernel<<<(n_cols + 255) / 256, 256, 0, s>>>(d_cpntr, n_block_cols, n_cols, d_col2bc);
    if (n_block_rows > 0) {
        cudaFuncSetAttribute(vbr_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        vbr_count_kernel<<<n_block_rows, INSPECT_THREADS, words * 4, s>>>(d_indptr, d_indices, d_rpntr, d_col2bc, words,
                                                                          d_counts);
    }
    if ((rc = tmp.alloc(&d_scan, (size_t)scan_len, "scan scratch"))) return bail(rc);
    if ((e = scan_i64(d_counts, d_bstart, n_block_rows, d_scan, s)) != cudaSuccess) return bail(cuda_fail(e, "block scan"));
    int64_t n_blocks = 0;
    if ((e = cudaMemcpy(&n_blocks, d_bstart + n_block_rows, sizeof n_blocks, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return bail(cuda_fail(e, "block count"));
    b->n_blocks = n_blocks;
    if ((rc = tmp.alloc(&d_bsize, (size_t)n_blocks, "block sizes"))) return bail(rc);
    if (cudaMalloc((void **)&b->d_bindx, std::max<size_t>(16, (size_t)n_blocks * 4)) != cudaSuccess ||
        cudaMalloc((void **)&b->d_indx, (size_t)(n_blocks + 1) * 8) != cudaSuccess ||
        cudaMalloc((void **)&b->d_bpntrb, std::max<size_t>(16, (size_t)n_block_rows * 4)) != cudaSuccess ||
        cudaMalloc((void **)&b->d_bpntre, std::max<size_t>(16, (size_t)n_block_rows * 4)) != cudaSuccess)
        return bail(fail(SABLE_ERR_NOMEM, "VBR index arrays"));
    if (n_block_rows > 0) {
        cudaFuncSetAttribute(vbr_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        vbr_blocks_kernel<<<n_block_rows, INSPECT_THREADS, smem, s>>>(d_indptr, d_indices, d_rpntr, d_cpntr, d_col2bc,
                                                                      words, d_bstart, b->d_bindx, d_bsize,
                                                                      b->d_bpntrb, b->d_bpntre);
    }
    int64_t *d_scan2 = nullptr;
    if ((rc = tmp.alloc(&d_scan2, (size_t)scan_tmp_len(std::max<int64_t>(n_blocks, 1)), "scan scratch"))) return bail(rc);
    if ((e = scan_i64(d_bsize, b->d_indx, n_blocks, d_scan2, s)) != cudaSuccess) return bail(cuda_fail(e, "size scan"));
    int64_t n_val = 0;
    if ((e = cudaMemcpy(&n_val, b->d_indx + n_blocks, sizeof n_val, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return bail(cuda_fail(e, "value count"));
    b->n_val = n_val;
    if (cudaMalloc(&b->d_val, std::max<size_t>(16, (size_t)n_val * vb)) != cudaSuccess)
        return bail(fail(SABLE_ERR_NOMEM, "VBR values (%lld)", (long long)n_val));
    if ((e = cudaMemsetAsync(b->d_val, 0, (size_t)n_val * vb, s)) != cudaSuccess) return bail(cuda_fail(e, "zero values"));
    if (n_block_rows > 0) {
        if (vb == 8) {
            cudaFuncSetAttribute(vbr_scatter_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            vbr_scatter_kernel<double><<<n_block_rows, 128, smem, s>>>(
                d_indptr, d_indices, reinterpret_cast<const double *>(d_data), d_rpntr, d_cpntr, d_col2bc, words,
                d_bstart, b->d_indx, static_cast<double *>(b->d_val));
        } else {
            cudaFuncSetAttribute(vbr_scatter_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            vbr_scatter_kernel<float><<<n_block_rows, 128, smem, s>>>(
                d_indptr, d_indices, reinterpret_cast<const float *>(d_data), d_rpntr, d_cpntr, d_col2bc, words,
                d_bstart, b->d_indx, static_cast<float *>(b->d_val));
        }
    }
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return bail(cuda_fail(e, "VBR construction"));
    *out = b;
    return SABLE_OK;
}

int sable_vbr_build_sizes(const sable_vbr_build *b, int64_t *n_blocks, int64_t *n_val) {
    if (!b || !n_blocks || !n_val) return fail(SABLE_ERR_ARG, "null argument");
    *n_blocks = b->n_blocks;
    *n_val = b->n_val;
    return SABLE_OK;
}

int sable_vbr_build_copy(const sable_vbr_build *b, void *val, int64_t *indx, int32_t *bindx, int32_t *bpntrb,
                         int32_t *bpntre) {
    if (!b || !val || !indx || !bindx || !bpntrb || !bpntre) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(b->device);
    if (rc) return rc;
    cudaError_t e;
    if ((e = cudaMemcpy(val, b->d_val, (size_t)b->n_val * b->value_bytes, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(indx, b->d_indx, (size_t)(b->n_blocks + 1) * 8, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(bindx, b->d_bindx, (size_t)b->n_blocks * 4, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(bpntrb, b->d_bpntrb, (size_t)b->n_block_rows * 4, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(bpntre, b->d_bpntre, (size_t)b->n_block_rows * 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "copy VBR arrays");
    return SABLE_OK;
}

int sable_vbr_build_destroy(sable_vbr_build *b) {
    if (!b) return SABLE_OK;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    cudaFree(b->d_val);
    cudaFree(b->d_indx);
    cudaFree(b->d_bindx);
    cudaFree(b->d_bpntrb);
    cudaFree(b->d_bpntre);
    if (prev >= 0) cudaSetDevice(prev);
    delete b;
    return SABLE_OK;
}

// Cut positions of the lines of one matrix (rows of `m`) into out[0..*n_out).
static int line_cuts(const sable_csr_desc *m, double threshold, int32_t mode, int32_t *out, int32_t *n_out) {
    const int n = m->n_rows, vb = m->value_bytes;
    if (n == 0) {
        out[0] = 0;
        *n_out = 1;
        return SABLE_OK;
    }
    DevBufs tmp;
    int64_t *d_ptr = nullptr, *d_flags = nullptr, *d_pos = nullptr, *d_scan = nullptr;
    int *d_idx = nullptr, *d_out = nullptr;
    unsigned char *d_data = nullptr;
    int rc;
    if ((rc = tmp.upload(&d_ptr, m->indptr, (size_t)n + 1, "indptr")) ||
        (rc = tmp.upload(&d_idx, m->indices, (size_t)m->nnz, "indices")) ||
        (rc = tmp.upload(&d_data, static_cast<const unsigned char *>(m->data), (size_t)m->nnz * vb, "values")) ||
        (rc = tmp.alloc(&d_flags, (size_t)n + 1, "cut flags")) || (rc = tmp.alloc(&d_pos, (size_t)n + 2, "cut positions")) ||
        (rc = tmp.alloc(&d_scan, (size_t)scan_tmp_len(n + 1), "scan scratch")) ||
        (rc = tmp.alloc(&d_out, (size_t)n + 1, "cuts")))
        return rc;
    const int pairs = std::max(1, n - 1);
    const unsigned grid = (unsigned)(((int64_t)pairs * 32 + INSPECT_THREADS - 1) / INSPECT_THREADS);
    if (vb == 8)
        similarity_flags_kernel<double><<<grid, INSPECT_THREADS>>>(d_ptr, d_idx, reinterpret_cast<const double *>(d_data),
                                                                   n, threshold, mode, d_flags);
    else
        similarity_flags_kernel<float><<<grid, INSPECT_THREADS>>>(d_ptr, d_idx, reinterpret_cast<const float *>(d_data),
                                                                  n, threshold, mode, d_flags);
    cudaError_t e = scan_i64(d_flags, d_pos, n + 1, d_scan, 0);
    if (e != cudaSuccess) return cuda_fail(e, "cut scan");
    compact_kernel<<<(n + 1 + 255) / 256, 256>>>(d_flags, d_pos, n, d_out);
    int64_t cnt = 0;
    if ((e = cudaMemcpy(&cnt, d_pos + n + 1, sizeof cnt, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(out, d_out, (size_t)cnt * 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(e, "copy cuts");
    *n_out = (int32_t)cnt;
    return SABLE_OK;
}

int sable_similarity_cuts(const sable_csr_desc *csr, const sable_csr_desc *csc, double threshold, int32_t mode,
                          int32_t device, int32_t *rpntr_out, int32_t *n_rpntr, int32_t *cpntr_out, int32_t *n_cpntr) {
    if (!rpntr_out || !n_rpntr || !cpntr_out || !n_cpntr) return fail(SABLE_ERR_ARG, "null output pointer");
    if (mode != 0 && mode != 1) return fail(SABLE_ERR_ARG, "mode %d (0: similarity2, 1: its numba variant)", mode);
    int rc = check_csr(csr, "CSR");
    if (rc) return rc;
    if ((rc = check_csr(csc, "CSC"))) return rc;
    if (csc->n_rows != csr->n_cols || csc->n_cols != csr->n_rows || csc->nnz != csr->nnz)
        return fail(SABLE_ERR_INVALID, "the CSC is not the transpose of the CSR (shape or nnz)");
    for (const sable_csr_desc *m : {csr, csc})
        for (int32_t r = 0; r < m->n_rows; ++r)
            for (int64_t e = m->indptr[r] + 1; e < m->indptr[r + 1]; ++e)
                if (m->indices[e] <= m->indices[e - 1])
                    return fail(SABLE_ERR_INVALID, "indices must increase strictly within each line (line %d)", r);
    if ((rc = set_device(device))) return rc;
    if ((rc = line_cuts(csr, threshold, mode, rpntr_out, n_rpntr))) return rc;
    return line_cuts(csc, threshold, mode, cpntr_out, n_cpntr);
}

}  // extern "C"
