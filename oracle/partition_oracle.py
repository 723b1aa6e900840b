"""ORACLE — test infrastructure only (tests/ use it as the checker; the
product never imports it).

Plain restatements of the reference's partitioning steps, loop for loop, on
dense line vectors, for small matrices:

  cut_indices2 + similarity2        src/autopartition.py:34-68, 87-89
  similarity2_numba                 src/autopartition.py:91-107
  convert_sparse_to_vbr             utils/convert_real_to_vbr.py:130-175
                                    (every block with a stored entry, dense,
                                    column-major, block-row order)
"""
from __future__ import annotations

import numpy as np
import scipy.sparse


def similarity2(a: np.ndarray, b: np.ndarray) -> float:
    """src/autopartition.py:87-89 (NumPy float64 semantics: 0 / 0 is NaN)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.float64(max(a.dot(b), a[1:].dot(b[:-1]), a[:-1].dot(b[1:]))) / np.float64(
            max(np.count_nonzero(a), np.count_nonzero(b)))


def similarity2_numba(a: np.ndarray, b: np.ndarray) -> float:
    """src/autopartition.py:91-107."""
    ca, cb = np.count_nonzero(a), np.count_nonzero(b)
    if ca == 0 or cb == 0:
        return 0.0
    a, b = a.astype(np.float64), b.astype(np.float64)
    best = np.dot(a, b)
    if len(a) > 1 and len(b) > 1:
        best = max(best, np.dot(a[1:], b[:-1]), np.dot(a[:-1], b[1:]))
    return best / max(ca, cb)


def cut_indices2(A, cut_threshold: float, similarity=similarity2):
    """src/autopartition.py:34-68 -> (col_indices, row_indices)."""
    A = scipy.sparse.csc_matrix(A)
    R = scipy.sparse.csr_matrix(A)
    n_rows, n_cols = A.shape

    def cuts(n, line_nnz, line):
        out = [0]
        i = 0
        while i < n - 1:
            if line_nnz(i) == 0:
                while i < n - 1 and line_nnz(i + 1) == 0:
                    i += 1
                out.append(i + 1)
            elif similarity(line(i), line(i + 1)) < cut_threshold:
                out.append(i + 1)
            i += 1
        if out[-1] != n:
            out.append(n)
        return out

    col = cuts(n_cols, lambda i: A[:, [i]].nnz, lambda i: A[:, [i]].toarray().ravel())
    row = cuts(n_rows, lambda i: R[[i], :].nnz, lambda i: R[[i], :].toarray().ravel())
    return col, row


def sparse_to_vbr(mat, rpntr, cpntr):
    """utils/convert_real_to_vbr.py:130-175 -> (val, indx, bindx, bpntrb,
    bpntre); a block row without blocks gets -1 / -1."""
    A = scipy.sparse.csc_matrix(mat)
    vals, sizes, bindx, counts = [], [], [], []
    for ri in range(len(rpntr) - 1):
        c = 0
        for ci in range(len(cpntr) - 1):
            blk = A[rpntr[ri]:rpntr[ri + 1], cpntr[ci]:cpntr[ci + 1]]
            if blk.nnz > 0:
                vals.append(np.asarray(blk.todense()).flatten(order="F"))
                sizes.append(blk.shape[0] * blk.shape[1])
                bindx.append(ci)
                c += 1
        counts.append(c)
    val = np.concatenate(vals) if vals else np.zeros(0)
    indx = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    ends = np.cumsum(counts)
    counts = np.asarray(counts)
    bpntrb = np.where(counts > 0, ends - counts, -1)
    bpntre = np.where(counts > 0, ends, -1)
    return val.astype(np.float64), indx, np.asarray(bindx, dtype=np.int64), bpntrb, bpntre
