/* ORACLE harness only: plain CSR loop behind the MKL names that SABLE's
 * generated SpMV executor calls.  y = alpha*A*x + beta*y, entries of a row in
 * index order; rows split over mkl_set_num_threads() OpenMP threads, as MKL's
 * threaded CSR product does (each row's sum keeps its order, so the result
 * does not depend on the thread count). */
#include <stdlib.h>
#include "mkl.h"
struct sable_standin_csr { int rows, cols, base; int *rs, *re, *ci; double *v; };
static int g_threads = 1;
void mkl_set_num_threads(int n) { g_threads = n > 0 ? n : 1; }
sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, sparse_index_base_t base, int rows, int cols,
                                        int *rows_start, int *rows_end, int *col_indx, double *values) {
    struct sable_standin_csr *m = (struct sable_standin_csr *)malloc(sizeof *m);
    m->rows = rows; m->cols = cols; m->base = (int)base;
    m->rs = rows_start; m->re = rows_end; m->ci = col_indx; m->v = values;
    *A = m;
    return SPARSE_STATUS_SUCCESS;
}
sparse_status_t mkl_sparse_d_mv(sparse_operation_t op, double alpha, const sparse_matrix_t A,
                                struct matrix_descr descr, const double *x, double beta, double *y) {
    (void)op; (void)descr;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < A->rows; ++i) {
        double s = 0.0;
        for (int k = A->rs[i] - A->base; k < A->re[i] - A->base; ++k) s += A->v[k] * x[A->ci[k] - A->base];
        y[i] = alpha * s + (beta == 0.0 ? 0.0 : beta * y[i]);
    }
    return SPARSE_STATUS_SUCCESS;
}
