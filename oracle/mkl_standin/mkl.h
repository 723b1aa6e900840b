/* ORACLE harness only: stand-in for the three Intel MKL sparse-BLAS entry
 * points that SABLE's generated SpMV executor calls (src/codegen.py:407-411,
 * 420).  MKL is not installed here; the stand-in is a plain CSR row loop. */
#ifndef SABLE_ORACLE_MKL_STANDIN_H
#define SABLE_ORACLE_MKL_STANDIN_H
#include "mkl_spblas.h"
void mkl_set_num_threads(int n);
#endif
