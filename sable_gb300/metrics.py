"""Algorithmic byte and flop counts used for GB/s, GFLOP/s and the roofline.

SpMV bytes B = sum over stored blocks of min(4*h*w, 8*nnz + 4*(h+1))
               + 4*n_cols + 4*n_rows
Each block is charged its cheaper FP32 encoding (dense values, or CSR values
+ int32 columns + row pointers); x is read once and y written once.  The
count does not depend on which representation a plan chose, so a poor
dense / sparse choice costs time, not bytes.

SpMM flops F = 2 * N * nnz(A) (true nonzeros); the bytes of its memory bound
are the SpMV matrix term + 4 * N * (n_cols + n_rows).
"""
from __future__ import annotations

import numpy as np

from . import convert


def block_stats(m):
    """(block table, nnz per block) of a VbrMatrix-like object."""
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    return bt, convert.block_nnz(m.val, bt)


def spmv_matrix_bytes(bt, nnz) -> int:
    return int(np.minimum(4 * bt.size, 8 * nnz + 4 * (bt.h + 1)).sum())


def spmv_bytes(m) -> int:
    bt, nnz = block_stats(m)
    return spmv_matrix_bytes(bt, nnz) + 4 * int(m.rpntr[-1]) + 4 * int(m.cpntr[-1])


def spmm_flops(m, N: int) -> int:
    _, nnz = block_stats(m)
    return int(2 * N * int(nnz.sum()))


def spmm_bytes(m, N: int) -> int:
    bt, nnz = block_stats(m)
    return spmv_matrix_bytes(bt, nnz) + 4 * N * (int(m.rpntr[-1]) + int(m.cpntr[-1]))
