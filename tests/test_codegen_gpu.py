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
