"""The inspector steps upstream of the plan, on the GPU (reference:
src/autopartition.py, utils/convert_real_to_vbr.py).

  cut_indices2(A, cut_threshold, similarity)      src/autopartition.py:34-68
      row / column cuts by the similarity of adjacent lines (similarity2,
      :87-89, or similarity2_numba, :91-107), computed by
      sable_similarity_cuts; returns (col_indices, row_indices) like the
      reference.
  convert_sparse_to_vbr(mat, rpntr, cpntr, fname, dst_dir)
                                                   utils/convert_real_to_vbr.py:98-199
      VBR arrays of a sparse matrix for a given partition, built by
      sable_vbr_from_csr; writes <dst_dir>/<fname>.vbr.
  my_convert_dense_to_vbrc((src_path, dest_path), cut_threshold, cut_indices, similarity)
                                                   src/autopartition.py:194-205
      MatrixMarket file -> cuts -> VBR -> compressed VBR (.vbrc).

The block choice of the compression stays on the host (convert.py); the
scans over every stored entry run on the GPU.
"""
from __future__ import annotations

import ctypes
import os
import pathlib

import numpy as np
import scipy.sparse

from . import _lib, convert, fileio
from .vbr import VBR

SIMILARITY_MODES = {"similarity2": 0, "similarity2_numba": 1}


def _csr_desc(m: scipy.sparse.csr_array, keep: list, dtype=np.float64) -> _lib.CsrDesc:
    indptr = np.ascontiguousarray(m.indptr, dtype=np.int64)
    indices = np.ascontiguousarray(m.indices, dtype=np.int32)
    data = np.ascontiguousarray(m.data, dtype=dtype)
    keep += [indptr, indices, data]
    d = _lib.CsrDesc()
    d.n_rows, d.n_cols = int(m.shape[0]), int(m.shape[1])
    d.indptr, d.indices, d.data = indptr.ctypes.data, _lib.ptr(indices), _lib.ptr(data)
    d.value_bytes = data.dtype.itemsize
    d.nnz = int(indptr[-1])
    return d


def _canonical_csr(A) -> scipy.sparse.csr_array:
    m = scipy.sparse.csr_array(A)
    if not m.has_canonical_format:
        m = m.copy()
        m.sum_duplicates()
    return m


def _mode(similarity) -> int:
    name = similarity if isinstance(similarity, str) else getattr(similarity, "__name__", "similarity2")
    if name not in SIMILARITY_MODES:
        raise ValueError(f"similarity {name!r}: one of {sorted(SIMILARITY_MODES)}")
    return SIMILARITY_MODES[name]


def cut_indices2(A, cut_threshold: float, similarity="similarity2", device: int | None = None):
    """src/autopartition.py:34-68 -> (col_indices, row_indices) as lists.

    `similarity` names the reference's similarity function ("similarity2" or
    "similarity2_numba", or a function of that name).  A line is a row (of
    the CSR) or a column (of the CSC); duplicate entries are summed first."""
    csr = _canonical_csr(A)
    csc = _canonical_csr(csr.T)       # the CSC as the CSR of the transpose
    keep: list = []
    d_r, d_c = _csr_desc(csr, keep), _csr_desc(csc, keep)
    rp = np.zeros(csr.shape[0] + 1, dtype=np.int32)
    cp = np.zeros(csr.shape[1] + 1, dtype=np.int32)
    nr, nc = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(_lib.load().sable_similarity_cuts(ctypes.byref(d_r), ctypes.byref(d_c), float(cut_threshold),
                                                 _mode(similarity), -1 if device is None else int(device),
                                                 rp.ctypes.data, ctypes.byref(nr), cp.ctypes.data, ctypes.byref(nc)),
               "sable_similarity_cuts")
    return cp[: nc.value].tolist(), rp[: nr.value].tolist()


def vbr_from_csr(mat, rpntr, cpntr, dtype=np.float64, device: int | None = None):
    """(val, indx, bindx, bpntrb, bpntre) of `mat` partitioned by rpntr /
    cpntr, built on the GPU (sable_vbr_from_csr); val has `dtype` (float64 as
    in the reference, or float32)."""
    m = scipy.sparse.csr_array(mat)    # duplicates are kept: the kernel sums them in CSR order
    rpntr = np.ascontiguousarray(rpntr, dtype=np.int32)
    cpntr = np.ascontiguousarray(cpntr, dtype=np.int32)
    keep: list = []
    d = _csr_desc(m, keep, dtype=np.dtype(dtype))
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(lib.sable_vbr_from_csr(ctypes.byref(d), len(rpntr) - 1, rpntr.ctypes.data, len(cpntr) - 1,
                                      cpntr.ctypes.data, -1 if device is None else int(device), ctypes.byref(h)),
               "sable_vbr_from_csr")
    try:
        nb, nv = ctypes.c_int64(), ctypes.c_int64()
        _lib.check(lib.sable_vbr_build_sizes(h, ctypes.byref(nb), ctypes.byref(nv)), "sable_vbr_build_sizes")
        val = np.zeros(max(nv.value, 1), dtype=dtype)
        indx = np.zeros(nb.value + 1, dtype=np.int64)
        bindx = np.zeros(max(nb.value, 1), dtype=np.int32)
        bpntrb = np.zeros(max(len(rpntr) - 1, 1), dtype=np.int32)
        bpntre = np.zeros(max(len(rpntr) - 1, 1), dtype=np.int32)
        _lib.check(lib.sable_vbr_build_copy(h, val.ctypes.data, indx.ctypes.data, bindx.ctypes.data,
                                            bpntrb.ctypes.data, bpntre.ctypes.data), "sable_vbr_build_copy")
    finally:
        lib.sable_vbr_build_destroy(h)
    nbr = len(rpntr) - 1
    return (val[: nv.value], indx, bindx[: nb.value].astype(np.int64), bpntrb[:nbr].astype(np.int64),
            bpntre[:nbr].astype(np.int64))


def convert_sparse_to_vbr(mat, rpntr, cpntr, fname, dst_dir, write: bool = True):
    """utils/convert_real_to_vbr.py:98-199 on the GPU: returns (val, indx,
    bindx, bpntrb, bpntre) and writes <dst_dir>/<fname>.vbr (unless
    write=False)."""
    val, indx, bindx, bpntrb, bpntre = vbr_from_csr(mat, rpntr, cpntr)
    if write:
        fileio.write_vbr_matrix(fname, VBR(val, indx, bindx, np.asarray(rpntr), np.asarray(cpntr), bpntrb, bpntre),
                                str(dst_dir))
    return val, indx, bindx, bpntrb, bpntre


def my_convert_dense_to_vbrc(file_info, cut_threshold: float, cut_indices=None, similarity="similarity2"):
    """src/autopartition.py:194-205: read a MatrixMarket file, cut it
    (cut_indices2 on the GPU), build its VBR form on the GPU and compress it
    (host), writing <dest dir>/<stem>.vbr and .vbrc; returns (val, rpntr,
    cpntr, indx, bindx, bpntrb, bpntre, ublocks, indptr, indices, csr_val)."""
    import scipy.io
    src_path, dest_path = file_info
    A = scipy.sparse.csc_matrix(scipy.io.mmread(src_path))
    cpntr, rpntr = cut_indices2(A, cut_threshold, similarity)
    stem = pathlib.Path(src_path).resolve().stem
    dst = pathlib.Path(dest_path).resolve().parent
    os.makedirs(dst, exist_ok=True)
    val, indx, bindx, bpntrb, bpntre = convert_sparse_to_vbr(A, rpntr, cpntr, stem, dst)
    val2, indx2, bindx, bpntrb, bpntre, ublocks, indptr, indices, csr_val = convert.convert_vbr_to_compressed(
        val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, stem, dst)
    return val2, rpntr, cpntr, indx2, bindx, bpntrb, bpntre, ublocks, indptr, indices, csr_val
