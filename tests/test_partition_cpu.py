"""The partitioning steps upstream of the plan, on the host: the oracle's
restatements of cut_indices2 / similarity2 (src/autopartition.py:34-107)
and convert_sparse_to_vbr (utils/convert_real_to_vbr.py:98-199) against
the reference's own outputs (tests/golden, made by running the reference),
the product's numpy convert_sparse_to_vbr against the oracle, and the
argument checks of the GPU entry points that run before any CUDA call."""
import ctypes
import hashlib
import os
import pathlib

import numpy as np
import pytest
import scipy.sparse

from oracle import partition_oracle as po
from sable_gb300 import _lib, convert, partition, synth

CASES = [c for c in synth.PARTITION_CASES]


def _fix(golden, name, key):
    return golden.arr(name, key)


@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_oracle_cuts_match_reference(golden, case):
    A = synth.partition_case(*case)
    name = f"part_{case[0]}"
    col, row = po.cut_indices2(A, 0.2, po.similarity2)
    np.testing.assert_array_equal(col, _fix(golden, name, "col"))
    np.testing.assert_array_equal(row, _fix(golden, name, "row"))
    col, row = po.cut_indices2(A, 0.2, po.similarity2_numba)
    np.testing.assert_array_equal(col, _fix(golden, name, "col_numba"))
    np.testing.assert_array_equal(row, _fix(golden, name, "row_numba"))


@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_vbr_construction_host_vs_oracle_vs_reference(golden, case):
    A = synth.partition_case(*case)
    name = f"part_{case[0]}"
    rp, cp = _fix(golden, name, "row"), _fix(golden, name, "col")
    want = po.sparse_to_vbr(A, rp, cp)
    got = convert.convert_sparse_to_vbr(scipy.sparse.csc_matrix(A), rp, cp, "x", "", write=False)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(np.asarray(g), np.asarray(w))
    if golden.meta(name)["vbr_ok"]:
        for k, w in zip(("val", "indx", "bindx", "bpntrb", "bpntre"), want):
            np.testing.assert_array_equal(w, _fix(golden, name, k))
    else:
        assert (want[3] == -1).any()   # a block row without blocks (the reference asserts)


def test_partition_kat_oracle(golden):
    """test.py:122-142: the oracle restatement on example2's dense matrix."""
    ex2 = golden.arrays("example2_arrays")
    dense = convert.vbr_to_dense(*ex2)
    got = po.sparse_to_vbr(scipy.sparse.csc_matrix(dense), ex2[3], ex2[4])
    for g, w in zip(got, (ex2[0], ex2[1], ex2[2], ex2[5], ex2[6])):
        np.testing.assert_array_equal(g, w)


def test_manual_mtx_cuts_when_available(golden):
    """The reference's manual_mtx matrices, read by path when its root is
    named in SABLE_REFERENCE_ROOT: the oracle's cuts equal the reference's."""
    root = os.environ.get("SABLE_REFERENCE_ROOT")
    if not root:
        pytest.skip("SABLE_REFERENCE_ROOT not set")
    import scipy.io
    done = 0
    for name, meta in golden.index.items():
        if not name.startswith("mtx_"):
            continue
        path = pathlib.Path(root) / meta["file"]
        if not path.exists() or hashlib.sha256(path.read_bytes()).hexdigest() != meta["file_sha"]:
            continue
        A = scipy.sparse.csc_matrix(scipy.io.mmread(str(path)))
        col, row = po.cut_indices2(A, 0.2, po.similarity2)
        np.testing.assert_array_equal(col, golden.arr(name, "col"))
        np.testing.assert_array_equal(row, golden.arr(name, "row"))
        done += 1
    assert done > 0


def _desc(indptr, indices, data, n_rows, n_cols, keep):
    keep += [indptr, indices, data]
    d = _lib.CsrDesc()
    d.n_rows, d.n_cols = n_rows, n_cols
    d.indptr, d.indices, d.data = indptr.ctypes.data, indices.ctypes.data, data.ctypes.data
    d.value_bytes, d.nnz = data.dtype.itemsize, int(indptr[-1])
    return d


def test_inspector_argument_checks():
    lib = _lib.load()
    keep = []
    ip = np.array([0, 2, 3], np.int64)
    ix = np.array([1, 0, 2], np.int32)        # row 0 not increasing
    dt = np.ones(3)
    csr = _desc(ip, ix, dt, 2, 3, keep)
    csc_ip = np.array([0, 1, 2, 3], np.int64)
    csc = _desc(csc_ip, np.array([0, 0, 1], np.int32), dt, 3, 2, keep)
    out = np.zeros(8, np.int32)
    n1, n2 = ctypes.c_int32(), ctypes.c_int32()
    rc = lib.sable_similarity_cuts(ctypes.byref(csr), ctypes.byref(csc), 0.2, 0, -1, out.ctypes.data,
                                   ctypes.byref(n1), out.ctypes.data, ctypes.byref(n2))
    assert rc == _lib.SABLE_ERR_INVALID and b"increase" in lib.sable_last_error()
    rc = lib.sable_similarity_cuts(ctypes.byref(csr), ctypes.byref(csc), 0.2, 7, -1, out.ctypes.data,
                                   ctypes.byref(n1), out.ctypes.data, ctypes.byref(n2))
    assert rc == _lib.SABLE_ERR_ARG
    bad_col = _desc(ip, np.array([0, 5, 2], np.int32), dt, 2, 3, keep)
    h = ctypes.c_void_p()
    rp = np.array([0, 2], np.int32)
    cp = np.array([0, 1, 3], np.int32)
    assert lib.sable_vbr_from_csr(ctypes.byref(bad_col), 1, rp.ctypes.data, 2, cp.ctypes.data, -1,
                                  ctypes.byref(h)) == _lib.SABLE_ERR_INVALID
    ok = _desc(ip, np.array([0, 1, 2], np.int32), dt, 2, 3, keep)
    bad_rp = np.array([0, 3], np.int32)
    assert lib.sable_vbr_from_csr(ctypes.byref(ok), 1, bad_rp.ctypes.data, 2, cp.ctypes.data, -1,
                                  ctypes.byref(h)) == _lib.SABLE_ERR_INVALID
    with pytest.raises(ValueError):
        partition._mode("similarity3")
