"""GPU similarity cuts (sable_similarity_cuts; src/autopartition.py:34-107)
and GPU VBR construction (sable_vbr_from_csr; utils/convert_real_to_vbr.py:
98-199) against the reference's own outputs (tests/golden) and the oracle's
restatements: integer and index results exactly, values bit for bit."""
import os

import numpy as np
import pytest
import scipy.sparse

from oracle import partition_oracle as po
from sable_gb300 import convert, fileio, partition, synth

pytestmark = pytest.mark.gpu
CASES = list(synth.PARTITION_CASES)


@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_gpu_cuts_match_reference(golden, cuda, case):
    A = synth.partition_case(*case)
    name = f"part_{case[0]}"
    for sim, suffix in (("similarity2", ""), ("similarity2_numba", "_numba")):
        col, row = partition.cut_indices2(scipy.sparse.csc_matrix(A), 0.2, sim)
        np.testing.assert_array_equal(col, golden.arr(name, "col" + suffix))
        np.testing.assert_array_equal(row, golden.arr(name, "row" + suffix))


@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_gpu_vbr_matches_reference_and_oracle(golden, cuda, case):
    A = synth.partition_case(*case)
    name = f"part_{case[0]}"
    rp, cp = golden.arr(name, "row"), golden.arr(name, "col")
    got = partition.vbr_from_csr(A, rp, cp)
    want = po.sparse_to_vbr(A, rp, cp)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    if golden.meta(name)["vbr_ok"]:
        for k, g in zip(("val", "indx", "bindx", "bpntrb", "bpntre"), got):
            np.testing.assert_array_equal(g, golden.arr(name, k))
    val32 = partition.vbr_from_csr(A, rp, cp, dtype=np.float32)[0]
    np.testing.assert_array_equal(val32, want[0].astype(np.float32))


def test_gpu_vbr_kat_example(golden, cuda):
    """test.py:122-142 on the GPU: example2's dense matrix."""
    ex2 = golden.arrays("example2_arrays")
    dense = convert.vbr_to_dense(*ex2)
    got = partition.vbr_from_csr(scipy.sparse.csc_matrix(dense), ex2[3], ex2[4])
    for g, w in zip(got, (ex2[0], ex2[1], ex2[2], ex2[5], ex2[6])):
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("shape,nbc_parts", [((1, 1), 1), ((40, 3000), 700), ((3000, 40), 7), ((257, 257), 257)])
def test_gpu_vbr_edges(cuda, shape, nbc_parts):
    """Single entries, many block columns (multi-word bitmaps, 1-column
    partitions), long columns, empty block rows; duplicates summed in order."""
    rng = np.random.default_rng(sum(shape))
    n_rows, n_cols = shape
    k = max(1, n_rows * n_cols // 50)
    r = rng.integers(0, n_rows, k)
    c = rng.integers(0, n_cols, k)
    v = rng.integers(-8, 9, k).astype(np.float64)
    A = scipy.sparse.coo_array((v, (r, c)), shape=shape).tocsr()   # duplicates kept, unsorted columns sorted
    A.sort_indices()
    cuts_c = np.unique(np.concatenate([[0, n_cols], rng.choice(np.arange(1, n_cols), min(nbc_parts, n_cols) - 1,
                                                                replace=False) if n_cols > 1 else []])).astype(int)
    cuts_r = np.unique(np.concatenate([[0, n_rows], rng.choice(np.arange(1, n_rows), min(9, n_rows - 1),
                                                                replace=False) if n_rows > 1 else []])).astype(int)
    got = partition.vbr_from_csr(A, cuts_r, cuts_c)
    want = po.sparse_to_vbr(A, cuts_r, cuts_c)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


def test_gpu_cuts_edges(cuda):
    """One line, all-empty lines, an empty matrix, a dense matrix."""
    for A in (scipy.sparse.csr_array(np.ones((1, 5))), scipy.sparse.csr_array((4, 6)),
              scipy.sparse.csr_array(np.ones((7, 9))), scipy.sparse.csr_array(np.eye(12))):
        for sim in ("similarity2", "similarity2_numba"):
            got = partition.cut_indices2(A, 0.2, sim)
            want = po.cut_indices2(A, 0.2, po.similarity2 if sim == "similarity2" else po.similarity2_numba)
            assert list(got[0]) == list(want[0]) and list(got[1]) == list(want[1]), (A.shape, sim, got, want)


def test_mtx_to_vbrc_pipeline(cuda, tmp_path):
    """my_convert_dense_to_vbrc (src/autopartition.py:194-205): a MatrixMarket
    file cut and converted on the GPU gives the same .vbr / .vbrc files as
    the host restatement."""
    import scipy.io
    A = synth.partition_case(3002, 500, 420, "quarters", False)
    src = tmp_path / "m.mtx"
    scipy.io.mmwrite(str(src), scipy.sparse.coo_array(A))
    out = partition.my_convert_dense_to_vbrc((str(src), str(tmp_path / "vbr" / "m.vbrc")), 0.2)
    B = scipy.sparse.csc_matrix(scipy.io.mmread(str(src)))
    col, row = po.cut_indices2(B, 0.2, po.similarity2)
    assert list(out[1]) == list(row) and list(out[2]) == list(col)
    val, indx, bindx, bpntrb, bpntre = po.sparse_to_vbr(B, row, col)
    text = fileio.read_vbr(os.path.join(tmp_path, "vbr", "m.vbr"))
    for g, w in zip((text[0], text[1], text[2], text[5], text[6]), (val, indx, bindx, bpntrb, bpntre)):
        np.testing.assert_array_equal(g, w)
    assert os.path.exists(os.path.join(tmp_path, "vbr", "m.vbrc"))
