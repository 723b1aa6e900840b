/* ORACLE harness only: the subset of mkl_spblas.h used by SABLE's generated C. */
#ifndef SABLE_ORACLE_MKL_SPBLAS_STANDIN_H
#define SABLE_ORACLE_MKL_SPBLAS_STANDIN_H
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10 } sparse_operation_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20 } sparse_matrix_type_t;
typedef enum { SPARSE_STATUS_SUCCESS = 0 } sparse_status_t;
struct matrix_descr { sparse_matrix_type_t type; int mode; int diag; };
typedef struct sable_standin_csr *sparse_matrix_t;
sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, sparse_index_base_t base, int rows, int cols,
                                        int *rows_start, int *rows_end, int *col_indx, double *values);
sparse_status_t mkl_sparse_d_mv(sparse_operation_t op, double alpha, const sparse_matrix_t A,
                                struct matrix_descr descr, const double *x, double beta, double *y);
#endif
