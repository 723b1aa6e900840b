"""The reference-named entry points end to end, the way a caller of the
reference's src/codegen.py uses them: write a .vbr file, compress it to
.vbrc, run the *_codegen inspector, execute the registered plan, and compare
with the FP64 oracle (and, for the example matrix, the reference's canonical
output)."""
import os

import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import codegen, convert, fileio, synth
from sable_gb300.vbr import VBR

pytestmark = pytest.mark.gpu


def test_spmv_codegen_from_files(cuda, tmp_path):
    m = synth.spmv_1000()
    vbr_dir, gen_dir = str(tmp_path / "vbr"), str(tmp_path / "gen")
    os.makedirs(vbr_dir)
    arrays = [np.asarray(a) for a in m.arrays()]
    fileio.write_vbr_matrix("m1000", VBR(*[a.tolist() for a in arrays]), vbr_dir)
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(os.path.join(vbr_dir, "m1000.vbr"))
    convert.convert_vbr_to_compressed(val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, "m1000", vbr_dir, density=30)
    ms = codegen.vbr_spmv_codegen("m1000", gen_dir, vbr_dir, threads=1, bench=3)
    assert ms >= 0 and os.path.exists(os.path.join(gen_dir, "m1000.sable.json"))
    x = synth.vector(m.n_cols, 5)
    times, y = codegen.run_spmv(gen_dir, "m1000", x)
    assert len(times) == 3
    comp = codegen._compressed_from_vbrc(*fileio.read_vbrc(os.path.join(vbr_dir, "m1000.vbrc")))
    comp.val = comp.val.astype(np.float64)
    y_ref, ya = oracle.spmv_vbrc(comp, x)
    r = oracle.report(y, y_ref, ya)
    assert r["pass"], r
    assert codegen.load_plan(gen_dir, "m1000").plan.schedule == codegen.SPMV_SHAPE["schedule"]


def test_spmm_codegen_example(golden, cuda, tmp_path):
    """vbr_spmm_codegen on the reference's example matrix, X = ones(11 x 512):
    every column equals the canonical SpMM output."""
    ex = golden.arrays("example_arrays")
    vbr_dir, gen_dir = str(tmp_path / "vbr"), str(tmp_path / "gen")
    os.makedirs(vbr_dir)
    fileio.write_vbr_matrix("example", VBR(*[a.tolist() for a in ex]), vbr_dir)
    codegen.vbr_spmm_codegen("example", 0, gen_dir, vbr_dir, threads=1)
    times, Y = codegen.run_spmm(gen_dir, "example", X=np.ones((11, 512), np.float32))
    np.testing.assert_allclose(Y[:, 0], golden.arr("example_canon", "spmm_rows"), rtol=1e-6)
    assert np.all(Y == Y[:, :1])


def test_only_nonzeros_baselines(golden, cuda, tmp_path):
    """The reference's per-nonzero baselines (src/baseline.py) on its example
    matrix: every block CSR, the canonical SpMV (x = 1) and SpMM (X = ones)
    outputs; and on a generated matrix against the FP64 oracle."""
    ex = golden.arrays("example_arrays")
    vbr_dir, gen_dir = str(tmp_path / "vbr"), str(tmp_path / "gen")
    os.makedirs(vbr_dir)
    fileio.write_vbr_matrix("example", VBR(*[a.tolist() for a in ex]), vbr_dir)
    codegen.only_nonzeros_spmv("example", gen_dir, vbr_dir)
    rec = codegen.load_plan(gen_dir, "example")
    assert rec.plan.stats()["dense_values"] == 0
    _, y = codegen.run_spmv(gen_dir, "example", np.ones(11, np.float32))
    np.testing.assert_allclose(y, golden.arr("example_canon", "spmv"), rtol=1e-6)
    codegen.only_nonzeros_spmm("example", gen_dir, vbr_dir)
    _, Y = codegen.run_spmm(gen_dir, "example", X=np.ones((11, 512), np.float32))
    np.testing.assert_allclose(Y[:, 0], golden.arr("example_canon", "spmm_rows"), rtol=1e-6)
    # a generated matrix (the reference generator's drop-in), random x
    import random
    random.seed(5)
    name = synth.vbr_matrix_gen(240, 200, "uniform", 8, 10, 20, 30, 15, False, vbr_dir=vbr_dir)
    codegen.only_nonzeros_spmv(name, gen_dir, vbr_dir + "_Sparse")
    x = synth.vector(200, 6)
    _, y = codegen.run_spmv(gen_dir, name, x)
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(os.path.join(vbr_dir + "_Sparse", name + ".vbr"))
    m = synth.VbrMatrix(np.asarray(val), np.asarray(indx), np.asarray(bindx), np.asarray(rpntr), np.asarray(cpntr),
                        np.asarray(bpntrb), np.asarray(bpntre))
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, np.zeros(m.n_blocks, bool))
    y_ref, ya = oracle.spmv_vbrc(comp, x)
    r = oracle.report(y, y_ref, ya)
    assert r["pass"], r


def _write_example(golden, vbr_dir):
    ex = golden.arrays("example_arrays")
    fileio.write_vbr_matrix("example", VBR(*[a.tolist() for a in ex]), vbr_dir)


def test_cuda_codegen_entry_points_example(golden, cuda, tmp_path):
    """vbr_spmv_cuda_codegen / vbr_spmm_cuda_codegen (src/codegen.py:1077-1195,
    1312-1436; the integer density rule of :1158) on the reference's example:
    x = 1 gives the canonical SpMV output, X = ones(11 x 512) the canonical
    SpMM rows, for an all-dense and a mostly-sparse choice."""
    vbr_dir, gen_dir = str(tmp_path / "vbr"), str(tmp_path / "gen")
    os.makedirs(vbr_dir)
    _write_example(golden, vbr_dir)
    for density in (0, 80):
        us = codegen.vbr_spmv_cuda_codegen("example", gen_dir, vbr_dir, density)
        assert us >= 0
        _, y = codegen.run_spmv(gen_dir, "example", np.ones(11, np.float32))
        np.testing.assert_allclose(y, golden.arr("example_canon", "spmv"), rtol=1e-6)
        codegen.vbr_spmm_cuda_codegen("example", gen_dir, vbr_dir, density)
        _, Y = codegen.run_spmm(gen_dir, "example", X=np.ones((11, 512), np.float32))
        np.testing.assert_allclose(Y[:, 0], golden.arr("example_canon", "spmm_rows"), rtol=1e-6)
        assert np.all(Y == Y[:, :1])


def test_cuda_codegen_entry_points_vs_reference_c(golden, cuda, tmp_path):
    """The same entry points on the seeded 1000^2 SpMV and 400^2 SpMM cases,
    against the outputs of the reference's own generated C."""
    vbr_dir, gen_dir = str(tmp_path / "vbr"), str(tmp_path / "gen")
    meta = golden.meta("spmv1000_d50")
    m = synth.spmv_1000(meta["seed"])
    fileio.write_vbr_matrix("m1000", VBR(*[np.asarray(a).tolist() for a in m.arrays()]), vbr_dir)
    codegen.vbr_spmv_cuda_codegen("m1000", gen_dir, vbr_dir, 50)
    x = synth.vector(m.n_cols, meta["x_seed"])
    _, y = codegen.run_spmv(gen_dir, "m1000", x)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, np.ones(m.n_blocks, bool),
                            value_dtype=np.float64)
    _, ya = oracle.spmv_vbrc(comp, x)
    r = oracle.report(y, golden.arr("spmv1000_d50", "y"), ya)
    assert r["pass"], r
    meta = golden.meta("spmm400_N32_d0")
    m = synth.spmm_50k(meta["seed"], n=meta["n"], parts=meta["parts"], p=meta["p"])
    fileio.write_vbr_matrix("m400", VBR(*[np.asarray(a).tolist() for a in m.arrays()]), vbr_dir)
    codegen.vbr_spmm_cuda_codegen("m400", gen_dir, vbr_dir, 0)
    X = synth.dense_operand(m.n_cols, meta["N"], meta["x_seed"])
    _, Y = codegen.run_spmm(gen_dir, "m400", X=X)
    r = oracle.report(Y, golden.arr("spmm400_N32_d0", "Y"), oracle.spmm_vbr(m, X)[1])
    assert r["pass"], r


def test_multi_threaded_generators(golden, cuda, tmp_path):
    """gen_multi_threaded_spmv / gen_multi_threaded_spmm (src/codegen.py:454-643,
    939-1075): the OpenMP split becomes GPU parallelism; the thread count is
    recorded, the result matches the reference's generated C."""
    vbr_dir, gen_dir = str(tmp_path / "vbr"), str(tmp_path / "gen")
    os.makedirs(vbr_dir)
    meta = golden.meta("spmv1000_d50")
    m = synth.spmv_1000(meta["seed"])
    val2, indx2, bindx, bpntrb, bpntre, ublocks, indptr, indices, csr_val = convert.convert_vbr_to_compressed(
        m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, "m1000", vbr_dir, density=50)
    np.testing.assert_array_equal(ublocks, golden.arr("spmv1000_d50", "ublocks"))
    ms = codegen.gen_multi_threaded_spmv(4, val2, indx2, bindx, m.rpntr, m.cpntr, bpntrb, bpntre, ublocks, indptr,
                                         indices, csr_val, gen_dir, "m1000", vbr_dir, bench=2)
    assert ms >= 0 and codegen.load_plan(gen_dir, "m1000").info["threads"] == 4
    x = synth.vector(m.n_cols, meta["x_seed"])
    times, y = codegen.run_spmv(gen_dir, "m1000", x)
    assert len(times) == 2
    comp = codegen._compressed_from_vbrc(*fileio.read_vbrc(os.path.join(vbr_dir, "m1000.vbrc")))
    comp.val = comp.val.astype(np.float64)
    _, ya = oracle.spmv_vbrc(comp, x)
    r = oracle.report(y, golden.arr("spmv1000_d50", "y"), ya)
    assert r["pass"], r
    meta = golden.meta("spmm400_N8_d30")
    m = synth.spmm_50k(meta["seed"], n=meta["n"], parts=meta["parts"], p=meta["p"])
    rec = codegen.gen_multi_threaded_spmm(8, m.val, m.indx, m.bindx, m.rpntr, m.cpntr, m.bpntrb, m.bpntre,
                                          meta["density"], gen_dir, "m400", vbr_dir)
    assert rec.info["threads"] == 8
    X = synth.dense_operand(m.n_cols, meta["N"], meta["x_seed"])
    _, Y = codegen.run_spmm(gen_dir, "m400", X=X)
    r = oracle.report(Y, golden.arr("spmm400_N8_d30", "Y"), oracle.spmm_vbr(m, X)[1])
    assert r["pass"], r


def test_codegen_from_binary_files(cuda, tmp_path):
    """The drop-in entry points read the binary forms (.vbrcb / .vbrb) when
    the text files are absent, with results identical to the text path."""
    m = synth.spmv_1000(1000)
    text_dir, bin_dir = str(tmp_path / "text"), str(tmp_path / "bin")
    vbr = VBR(*[np.asarray(a) for a in m.arrays()])
    fileio.write_vbr_matrix("m", VBR(*[np.asarray(a).tolist() for a in m.arrays()]), text_dir)
    fileio.write_vbr_binary("m", vbr, bin_dir)
    for d, binary in ((text_dir, False), (bin_dir, True)):
        convert.convert_vbr_to_compressed(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, "m", d,
                                          density=30, binary=binary)
    assert not os.path.exists(os.path.join(bin_dir, "m.vbrc")) and not os.path.exists(os.path.join(bin_dir, "m.vbr"))
    x = synth.vector(m.n_cols, 3)
    X = synth.dense_operand(m.n_cols, 32, 4)
    out = {}
    for tag, d in (("t", text_dir), ("b", bin_dir)):
        gen = str(tmp_path / ("gen" + tag))
        codegen.vbr_spmv_codegen("m", gen, d, threads=1)
        _, y = codegen.run_spmv(gen, "m", x)
        codegen.vbr_spmm_codegen("m", 30, gen + "mm", d, threads=1)
        _, Y = codegen.run_spmm(gen + "mm", "m", X=X)
        out[tag] = (y, Y)
    np.testing.assert_array_equal(out["t"][0], out["b"][0])
    np.testing.assert_array_equal(out["t"][1], out["b"][1])
