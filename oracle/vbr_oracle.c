/*
 * ORACLE — test infrastructure only.  Nothing in the shipped package links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py do.
 *
 * A host FP64 restatement of the executor that SABLE's code generator emits
 * (reference: src/codegen.py).  Each function names the generator it follows.
 *
 *   oracle_spmv_vbrc   gen_single_threaded_spmv   src/codegen.py:293-452
 *                      kernels spmv_kernel / _2 / _3 src/codegen.py:263-291
 *                      MKL call (beta = 0, before the dense blocks)
 *                      src/codegen.py:407-411, 420
 *   oracle_spmm_vbr    gen_single_threaded_spmm   src/codegen.py:827-937
 *                      spmm_kernel (i-j-k)         src/codegen.py:851-859
 *                      DSL-unrolled sparse blocks  src/codegen.py:150-163, 906-922
 *   cpu_spmv_timed     the generated timed loop of gen_single/multi_threaded_spmv
 *                      (src/codegen.py:412-439, 567-637), block rows split over
 *                      threads by greedy LPT (split_chunks, src/codegen.py:165-186)
 *   cpu_spmm_timed     gen_single/multi_threaded_spmm timed region
 *                      (src/codegen.py:906-928, 939-1064)
 *
 * The MKL sparse BLAS call of the reference (closed library, version unpinned)
 * is restated as a plain CSR row loop: y[i] = sum_k csr_val[k] * x[indices[k]]
 * over k in [indptr[i], indptr[i+1]) in index order.
 *
 * Besides y, every oracle also returns |A|.|x| per output, the scale of the
 * per-row parity tolerance.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Mark which block columns of block row a are stored; the generator walks
 * b = 0..nbc-1 and emits a call when b is in bindx[bpntrb[a]:bpntre[a]]
 * (src/codegen.py:421-426). */
static void mark_row(const int32_t *bindx, int32_t b0, int32_t b1, uint8_t *mark, int32_t nbc, int on) {
    for (int32_t k = b0; k < b1; ++k) {
        int32_t b = bindx[k];
        if (b >= 0 && b < nbc) mark[b] = (uint8_t)on;
    }
}

static int is_ublock(const int32_t *ublocks, int64_t n_ublocks, int64_t ordinal) {
    /* `nnz_block not in ublocks` (src/codegen.py:427); ublocks is ascending. */
    int64_t lo = 0, hi = n_ublocks;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (ublocks[mid] < ordinal) lo = mid + 1; else hi = mid;
    }
    return lo < n_ublocks && ublocks[lo] == ordinal;
}

/*
 * y = A x for a compressed VBR (.vbrc) matrix.
 * val/indx hold the dense blocks only (indx has n_dense+1 entries);
 * ublocks lists the ordinals (over all stored blocks, in generator order) of
 * the blocks moved to the global CSR (indptr/indices/csr_val, may be NULL).
 * Returns 0, or -1 when the arrays are inconsistent.
 */
int oracle_spmv_vbrc(int32_t n_rows, int32_t n_cols, int32_t nbr, int32_t nbc,
                     const int32_t *rpntr, const int32_t *cpntr,
                     const int32_t *bpntrb, const int32_t *bpntre, const int32_t *bindx,
                     const int64_t *indx, int64_t n_dense, const double *val,
                     const int32_t *ublocks, int64_t n_ublocks,
                     const int64_t *indptr, const int32_t *indices, const double *csr_val,
                     const double *x, double *y, double *yabs) {
    (void)n_cols;
    memset(y, 0, sizeof(double) * (size_t)n_rows);
    if (yabs) memset(yabs, 0, sizeof(double) * (size_t)n_rows);
    /* MKL part first, beta = 0 (src/codegen.py:419-420). */
    if (n_ublocks > 0 && indptr) {
        for (int32_t i = 0; i < n_rows; ++i) {
            double s = 0.0, sa = 0.0;
            for (int64_t k = indptr[i]; k < indptr[i + 1]; ++k) {
                s += csr_val[k] * x[indices[k]];
                sa += fabs(csr_val[k]) * fabs(x[indices[k]]);
            }
            y[i] = s;
            if (yabs) yabs[i] = sa;
        }
    }
    uint8_t *mark = (uint8_t *)calloc((size_t)nbc + 1, 1);
    if (!mark) return -1;
    int64_t count = 0, nnz_block = 0;
    for (int32_t a = 0; a < nbr; ++a) {
        if (bpntrb[a] == -1) continue;
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 1);
        int32_t i0 = rpntr[a], i1 = rpntr[a + 1];
        for (int32_t b = 0; b < nbc; ++b) {
            if (!mark[b]) continue;
            if (!is_ublock(ublocks, n_ublocks, nnz_block)) {
                if (count >= n_dense) { free(mark); return -1; }
                const double *blk = val + indx[count];
                int32_t j0 = cpntr[b], j1 = cpntr[b + 1];
                /* spmv_kernel: j outer, i inner, column-major block
                 * (src/codegen.py:263-272); the 1-row / 1-column variants
                 * (:274-291) compute the same sums in the same order. */
                for (int32_t j = j0; j < j1; ++j)
                    for (int32_t i = i0; i < i1; ++i) {
                        double v = blk[(int64_t)(j - j0) * (i1 - i0) + (i - i0)];
                        y[i] += v * x[j];
                        if (yabs) yabs[i] += fabs(v) * fabs(x[j]);
                    }
                ++count;
            }
            ++nnz_block;
        }
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 0);
    }
    free(mark);
    return 0;
}

/*
 * Y = A X for an uncompressed VBR matrix, X row-major n_cols x N, Y row-major
 * n_rows x N (the reference fixes N = 512; here N is a parameter).
 * `density` follows gen_single_threaded_spmm: when density > 0, blocks whose
 * density% <= density are emitted as unrolled per-nonzero statements, which
 * skip the zero entries; the others go through spmm_kernel.  Sums run in the
 * generator's order: blocks in row/column order, i, then j, then k.
 */
int oracle_spmm_vbr(int32_t n_rows, int32_t n_cols, int32_t nbr, int32_t nbc,
                    const int32_t *rpntr, const int32_t *cpntr,
                    const int32_t *bpntrb, const int32_t *bpntre, const int32_t *bindx,
                    const int64_t *indx, int64_t n_blocks, const double *val,
                    int32_t density, int32_t N,
                    const double *X, double *Y, double *Yabs) {
    (void)n_cols;
    memset(Y, 0, sizeof(double) * (size_t)n_rows * (size_t)N);
    if (Yabs) memset(Yabs, 0, sizeof(double) * (size_t)n_rows * (size_t)N);
    uint8_t *mark = (uint8_t *)calloc((size_t)nbc + 1, 1);
    if (!mark) return -1;
    int64_t count = 0;
    for (int32_t a = 0; a < nbr; ++a) {
        if (bpntrb[a] == -1) continue;
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 1);
        int32_t i0 = rpntr[a], i1 = rpntr[a + 1], h = i1 - i0;
        for (int32_t b = 0; b < nbc; ++b) {
            if (!mark[b]) continue;
            if (count >= n_blocks) { free(mark); return -1; }
            const double *blk = val + indx[count];
            int32_t j0 = cpntr[b], j1 = cpntr[b + 1], w = j1 - j0;
            int skip_zeros = 0;
            if (density > 0) {
                int64_t nz = 0;
                for (int64_t e = 0; e < (int64_t)h * w; ++e) nz += blk[e] != 0.0;
                double pct = (double)nz / (double)((int64_t)h * w) * 100.0;
                skip_zeros = !(pct > (double)density);
            }
            for (int32_t i = i0; i < i1; ++i)
                for (int32_t j = j0; j < j1; ++j) {
                    double v = blk[(int64_t)(j - j0) * h + (i - i0)];
                    if (skip_zeros && v == 0.0) continue;
                    const double *xr = X + (int64_t)j * N;
                    double *yr = Y + (int64_t)i * N;
                    for (int32_t k = 0; k < N; ++k) yr[k] += v * xr[k];
                    if (Yabs) {
                        double *ya = Yabs + (int64_t)i * N;
                        for (int32_t k = 0; k < N; ++k) ya[k] += fabs(v) * fabs(xr[k]);
                    }
                }
            ++count;
        }
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 0);
    }
    free(mark);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Timed CPU port of the generated executor (the cpu_baseline).              */
/* ------------------------------------------------------------------------ */

static int64_t now_ns(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (int64_t)t.tv_sec * 1000000000LL + t.tv_nsec;
}

/* One dense block as the generator emits it: a call with baked-in bounds. */
typedef struct { int32_t i0, i1, j0, j1; int64_t off; } blk_call;

/* Greedy LPT over block rows by h*w work (split_chunks, src/codegen.py:165-186):
 * rows sorted by work descending (stable), each to the currently lightest
 * thread.  Returns the number of threads that received work. */
static int lpt_split(const int64_t *work, int32_t nbr, int threads, int32_t *owner) {
    int32_t nz = 0;
    for (int32_t a = 0; a < nbr; ++a) nz += work[a] != 0;
    if (nz < threads) threads = nz;
    for (int32_t a = 0; a < nbr; ++a) owner[a] = -1;
    if (threads <= 0) return 0;
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nz ? nz : 1));
    int32_t m = 0;
    for (int32_t a = 0; a < nbr; ++a) if (work[a]) order[m++] = a;
    /* stable insertion-free sort: simple merge via qsort on (work desc, index asc) */
    for (int32_t p = 1; p < m; ++p) {
        int32_t v = order[p], q = p - 1;
        while (q >= 0 && work[order[q]] < work[v]) { order[q + 1] = order[q]; --q; }
        order[q + 1] = v;
    }
    int64_t *sums = (int64_t *)calloc((size_t)threads, sizeof(int64_t));
    for (int32_t p = 0; p < m; ++p) {
        int t = 0;
        for (int u = 1; u < threads; ++u) if (sums[u] < sums[t]) t = u;
        owner[order[p]] = t;
        sums[t] += work[order[p]];
    }
    free(sums);
    free(order);
    return threads;
}

/*
 * Runs `iters` timed iterations of the generated SpMV executor over a .vbrc
 * matrix on `threads` host threads (1 = gen_single_threaded_spmv).  Per
 * iteration: memset y, CSR part (beta = 0), dense blocks.  times_ns receives
 * one duration per iteration.  Returns the number of threads used.
 */
int cpu_spmv_timed(int32_t n_rows, int32_t nbr, int32_t nbc,
                   const int32_t *rpntr, const int32_t *cpntr,
                   const int32_t *bpntrb, const int32_t *bpntre, const int32_t *bindx,
                   const int64_t *indx, int64_t n_dense, const double *val,
                   const int32_t *ublocks, int64_t n_ublocks,
                   const int64_t *indptr, const int32_t *indices, const double *csr_val,
                   const double *x, double *y, int threads, int iters, int64_t *times_ns) {
    /* Build the call list the generator would emit. */
    blk_call *calls = (blk_call *)malloc(sizeof(blk_call) * (size_t)(n_dense ? n_dense : 1));
    int32_t *row_first = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nbr + 1));
    int64_t *work = (int64_t *)calloc((size_t)nbr, sizeof(int64_t));
    uint8_t *mark = (uint8_t *)calloc((size_t)nbc + 1, 1);
    int64_t count = 0, nnz_block = 0;
    for (int32_t a = 0; a < nbr; ++a) {
        row_first[a] = (int32_t)count;
        if (bpntrb[a] == -1) continue;
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 1);
        for (int32_t b = 0; b < nbc; ++b) {
            if (!mark[b]) continue;
            if (!is_ublock(ublocks, n_ublocks, nnz_block) && count < n_dense) {
                blk_call c = {rpntr[a], rpntr[a + 1], cpntr[b], cpntr[b + 1], indx[count]};
                calls[count++] = c;
                work[a] += (int64_t)(c.i1 - c.i0) * (c.j1 - c.j0);
            }
            ++nnz_block;
        }
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 0);
    }
    row_first[nbr] = (int32_t)count;
    free(mark);
    int32_t *owner = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nbr ? nbr : 1));
    int used = lpt_split(work, nbr, threads < 1 ? 1 : threads, owner);
    if (used < 1) used = 1;
#ifdef _OPENMP
    omp_set_num_threads(threads < 1 ? 1 : threads);
#endif
    for (int it = 0; it < iters; ++it) {
        memset(y, 0, sizeof(double) * (size_t)n_rows);
        int64_t t1 = now_ns();
        if (n_ublocks > 0 && indptr) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (threads > 1)
#endif
            for (int32_t i = 0; i < n_rows; ++i) {
                double s = 0.0;
                for (int64_t k = indptr[i]; k < indptr[i + 1]; ++k) s += csr_val[k] * x[indices[k]];
                y[i] = s;
            }
        }
#ifdef _OPENMP
#pragma omp parallel for schedule(static, 1) if (threads > 1)
#endif
        for (int t = 0; t < used; ++t) {
            for (int32_t a = 0; a < nbr; ++a) {
                if (used > 1 && owner[a] != t) continue;
                for (int32_t c = row_first[a]; c < row_first[a + 1]; ++c) {
                    const blk_call bc = calls[c];
                    const double *restrict blk = val + bc.off;
                    const int32_t h = bc.i1 - bc.i0;
                    double *restrict yy = y + bc.i0;
                    for (int32_t j = bc.j0; j < bc.j1; ++j) {
                        const double xj = x[j];
                        const double *restrict col = blk + (int64_t)(j - bc.j0) * h;
                        for (int32_t i = 0; i < h; ++i) yy[i] += col[i] * xj;
                    }
                }
            }
        }
        times_ns[it] = now_ns() - t1;
    }
    free(owner);
    free(work);
    free(row_first);
    free(calls);
    return used;
}

/*
 * Timed SpMM port: gen_single/multi_threaded_spmm, FP32 like the reference
 * (src/codegen.py:851-859 uses float), width N instead of the literal 512.
 * Blocks whose density% <= density (density > 0) skip zero entries as the
 * unrolled code does.  Returns the number of threads used.
 */
int cpu_spmm_timed(int32_t n_rows, int32_t nbr, int32_t nbc,
                   const int32_t *rpntr, const int32_t *cpntr,
                   const int32_t *bpntrb, const int32_t *bpntre, const int32_t *bindx,
                   const int64_t *indx, int64_t n_blocks, const float *val,
                   int32_t density, int32_t N, const float *X, float *Y,
                   int threads, int iters, int64_t *times_ns) {
    blk_call *calls = (blk_call *)malloc(sizeof(blk_call) * (size_t)(n_blocks ? n_blocks : 1));
    uint8_t *sparse = (uint8_t *)calloc((size_t)(n_blocks ? n_blocks : 1), 1);
    int32_t *row_first = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nbr + 1));
    int64_t *work = (int64_t *)calloc((size_t)nbr, sizeof(int64_t));
    uint8_t *mark = (uint8_t *)calloc((size_t)nbc + 1, 1);
    int64_t count = 0;
    for (int32_t a = 0; a < nbr; ++a) {
        row_first[a] = (int32_t)count;
        if (bpntrb[a] == -1) continue;
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 1);
        for (int32_t b = 0; b < nbc; ++b) {
            if (!mark[b] || count >= n_blocks) continue;
            blk_call c = {rpntr[a], rpntr[a + 1], cpntr[b], cpntr[b + 1], indx[count]};
            int64_t hw = (int64_t)(c.i1 - c.i0) * (c.j1 - c.j0);
            if (density > 0) {
                int64_t nz = 0;
                for (int64_t e = 0; e < hw; ++e) nz += val[c.off + e] != 0.0f;
                sparse[count] = !((double)nz / (double)hw * 100.0 > (double)density);
            }
            if (!sparse[count]) work[a] += hw;
            calls[count++] = c;
        }
        mark_row(bindx, bpntrb[a], bpntre[a], mark, nbc, 0);
    }
    row_first[nbr] = (int32_t)count;
    free(mark);
    int32_t *owner = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nbr ? nbr : 1));
    /* The pthread split assigns only rows with dense work (work_per_br,
     * src/codegen.py:966-988); rows holding only unrolled blocks go to the
     * thread owning the fewest rows so that no work is lost. */
    int used = lpt_split(work, nbr, threads < 1 ? 1 : threads, owner);
    if (used < 1) used = 1;
    for (int32_t a = 0; a < nbr; ++a) if (owner[a] < 0) owner[a] = a % used;
#ifdef _OPENMP
    omp_set_num_threads(threads < 1 ? 1 : threads);
#endif
    for (int it = 0; it < iters; ++it) {
        memset(Y, 0, sizeof(float) * (size_t)n_rows * (size_t)N);
        int64_t t1 = now_ns();
#ifdef _OPENMP
#pragma omp parallel for schedule(static, 1) if (threads > 1)
#endif
        for (int t = 0; t < used; ++t) {
            for (int32_t a = 0; a < nbr; ++a) {
                if (used > 1 && owner[a] != t) continue;
                for (int32_t c = row_first[a]; c < row_first[a + 1]; ++c) {
                    const blk_call bc = calls[c];
                    const float *restrict blk = val + bc.off;
                    const int32_t h = bc.i1 - bc.i0;
                    const int skip = sparse[c];
                    for (int32_t i = bc.i0; i < bc.i1; ++i)
                        for (int32_t j = bc.j0; j < bc.j1; ++j) {
                            const float v = blk[(int64_t)(j - bc.j0) * h + (i - bc.i0)];
                            if (skip && v == 0.0f) continue;
                            const float *restrict xr = X + (int64_t)j * N;
                            float *restrict yr = Y + (int64_t)i * N;
                            for (int32_t k = 0; k < N; ++k) yr[k] += v * xr[k];
                        }
                }
            }
        }
        times_ns[it] = now_ns() - t1;
    }
    free(owner);
    free(work);
    free(row_first);
    free(sparse);
    free(calls);
    return used;
}
