"""The oracle and the host-side format / block-split code, pinned against the
reference's own outputs (tests/golden, made by tests/golden/make_golden.py
from the reference's generator and its generated C)."""
import hashlib

import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import blockmodel, convert, fileio, synth
from sable_gb300.vbr import VBR


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(np.asarray(a))
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def compressed(arrays, density=None, model=None):
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = arrays
    bt = convert.block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx)
    dense = convert.choose_dense(np.asarray(val, np.float64), rpntr, cpntr, indx, bindx, bpntrb, bpntre,
                                 density=density, model=model, bt=bt)
    return convert.compress(np.asarray(val, np.float64), rpntr, cpntr, indx, bindx, bpntrb, bpntre, dense, bt=bt,
                            value_dtype=np.float64)


def test_example_spmv_canon(golden):
    """oracle(example.vbr, x = 1) == output_spmv_canon.txt and the reference C output."""
    ex = golden.arrays("example_arrays")
    c = compressed(ex, density=0)
    y, ya = oracle.spmv_vbrc(c, np.ones(11))
    np.testing.assert_array_equal(y, golden.arr("example_canon", "spmv"))
    np.testing.assert_array_equal(y, golden.arr("example_d0", "y"))
    assert np.all(ya >= np.abs(y))


def test_example2_compression_kat(golden):
    """convert_vbr_to_compressed(density=80) reproduces the reference's
    ublocks / indx / CSR arrays exactly (test.py:80-105) and the oracle
    reproduces output_spmv_canon_sparse.txt (x = 1)."""
    ex2 = golden.arrays("example2_arrays")
    ref = golden.arrays("example2_vbrc", ("val", "indx", "ublocks", "indptr", "indices", "csr_val"))
    c = compressed(ex2, density=80)
    np.testing.assert_array_equal(c.val, ref[0])
    np.testing.assert_array_equal(c.indx, ref[1])
    np.testing.assert_array_equal(c.ublocks, ref[2])
    np.testing.assert_array_equal(c.indptr, ref[3])
    np.testing.assert_array_equal(c.indices, ref[4])
    np.testing.assert_array_equal(c.csr_val, ref[5])
    y, _ = oracle.spmv_vbrc(c, np.ones(11))
    canon = golden.arr("example_canon", "spmv_sparse")
    np.testing.assert_array_equal(y[: len(canon)], canon)
    np.testing.assert_array_equal(y, golden.arr("example2_d80", "y"))


def test_partition_kat(golden):
    """convert_sparse_to_vbr of example2's dense matrix gives the reference arrays (test.py:122-142)."""
    ex2 = golden.arrays("example2_arrays")
    dense = convert.vbr_to_dense(*ex2)
    import scipy.sparse
    val, indx, bindx, bpntrb, bpntre = convert.convert_sparse_to_vbr(scipy.sparse.csc_matrix(dense), ex2[3], ex2[4],
                                                                     "e2", "/tmp", write=False)
    for got, want in zip((val, indx, bindx, bpntrb, bpntre), (ex2[0], ex2[1], ex2[2], ex2[5], ex2[6])):
        np.testing.assert_array_equal(got, want)


def test_compression_full_dense(golden):
    ex = golden.arrays("example_arrays")
    c = compressed(ex, density=0)
    assert len(c.ublocks) == 0 and c.indptr is None
    np.testing.assert_array_equal(c.val, ex[0])
    np.testing.assert_array_equal(c.indx, ex[1])


@pytest.mark.parametrize("case,density", [("spmv1000_d0", 0), ("spmv1000_d50", 50), ("spmv1000_rf", None)])
def test_spmv1000_against_reference_c(golden, case, density):
    """Seeded 1000^2 matrix: block split identical to the reference's, FP64
    oracle within 1e-13 (|A||x|-scaled) of the reference's generated C."""
    meta = golden.meta(case)
    m = synth.spmv_1000(meta["seed"])
    x = synth.vector(m.n_cols, meta["x_seed"])
    assert sha(*m.arrays(), x) == meta["sha"], "generator drifted from the fixture"
    arrays = (m.val.astype(np.float64), *m.arrays()[1:])
    model = blockmodel.RFTableModel() if density is None else None
    c = compressed(arrays, density=density, model=model)
    np.testing.assert_array_equal(c.ublocks, golden.arr(case, "ublocks"))
    np.testing.assert_array_equal(c.indx, golden.arr(case, "indx2"))
    if len(golden.arr(case, "indptr")):
        np.testing.assert_array_equal(c.indptr, golden.arr(case, "indptr"))
        np.testing.assert_array_equal(c.indices, golden.arr(case, "indices"))
        np.testing.assert_array_equal(c.csr_val, golden.arr(case, "csr_val"))
    assert sha(np.asarray(c.val, np.float64)) == meta["val2_sha"]
    y, ya = oracle.spmv_vbrc(c, x)
    r = oracle.report(y, golden.arr(case, "y"), ya)
    assert r["max"] < 1e-13, r


@pytest.mark.parametrize("case", ["spmm400_N32_d0", "spmm400_N8_d30"])
def test_spmm_against_reference_c(golden, case):
    """FP64 SpMM oracle vs the reference's generated FP32 C: within the
    parity tolerance (the reference rounds every product to FP32)."""
    meta = golden.meta(case)
    m = synth.spmm_50k(meta["seed"], n=meta["n"], parts=meta["parts"], p=meta["p"])
    X = synth.dense_operand(m.n_cols, meta["N"], meta["x_seed"])
    assert sha(*m.arrays(), X) == meta["sha"]
    Y, Ya = oracle.spmm_vbr(m, X, density=meta["density"])
    r = oracle.report(Y, golden.arr(case, "Y"), Ya)
    assert r["pass"], r


def test_example_spmm_canon(golden):
    ex = golden.arrays("example_arrays")
    m = synth.VbrMatrix(*ex)
    Y, _ = oracle.spmm_vbr(m, np.ones((11, 512)))
    assert golden.meta("example_canon")["spmm_rows_constant"]
    np.testing.assert_array_equal(Y[:, 0], golden.arr("example_canon", "spmm_rows"))
    np.testing.assert_array_equal(Y, golden.arr("example_spmm512", "Y"))


def test_rf_table_sanity_points():
    """The printed expectations of studies/find_threshold.py:65-73."""
    rf = blockmodel.RFTableModel()
    X = [[50, 50, 1], [153, 9, 0.65], [125, 8, 1], [465, 2, 1], [1000, 1, 100.0], [1139, 1, 100.0],
         [150, 150, 100], [1, 9996, 100.0], [9996, 1, 100.0]]
    np.testing.assert_array_equal(rf.predict(X), [0, 0, 0, 0, 0, 0, 1, 1, 1])


def test_vbr_file_round_trip(tmp_path, golden):
    ex = golden.arrays("example_arrays")
    fileio.write_vbr_matrix("ex", VBR(*[a.tolist() for a in ex]), str(tmp_path))
    text = (tmp_path / "ex.vbr").read_text().splitlines()
    assert text[0].startswith("val=[4.0,1.0,2.0,5.0,") and text[3] == "rpntr=[0,2,5,6,9,11]"
    back = fileio.read_vbr(str(tmp_path / "ex.vbr"))
    for a, b in zip(back, ex):
        np.testing.assert_array_equal(a, b)


def test_vbrc_file_round_trip(tmp_path, golden):
    ex2 = golden.arrays("example2_arrays")
    out = convert.convert_vbr_to_compressed(*[np.asarray(a) for a in (ex2[0], ex2[3], ex2[4], ex2[1], ex2[2], ex2[5],
                                                                      ex2[6])], "e2", str(tmp_path), density=80)
    back = fileio.read_vbrc(str(tmp_path / "e2.vbrc"))
    ref = golden.arrays("example2_vbrc", ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre", "ublocks",
                                          "indptr", "indices", "csr_val"))
    for a, b in zip(back, ref):
        np.testing.assert_array_equal(a, b)
    assert len(out) == 9


def test_oracle_planted_mistake_is_caught():
    """A wrong value planted in the oracle's input is visible in report()."""
    m = synth.spmv_1000()
    x = synth.vector(m.n_cols, 2000)
    arrays = (m.val.astype(np.float64), *m.arrays()[1:])
    c = compressed(arrays, density=0)
    y, ya = oracle.spmv_vbrc(c, x)
    c.val = c.val.copy()
    c.val[len(c.val) // 2] += 0.5
    y2, _ = oracle.spmv_vbrc(c, x)
    assert not oracle.report(y2, y, ya)["pass"]


def test_partition_sizes_infeasible_total_raises():
    with pytest.raises(ValueError):
        synth.sizes_with_sum(np.random.default_rng(0), 30, 20, 80, 3000)
