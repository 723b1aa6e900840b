"""SpMM parity on the GPU (FP32 CUDA-core form, and split-BF16 tensor-core
forms when the plan enables them) against the FP64 oracle and the reference's
generated C.  Tolerance: |Y_gpu - Y_ref| <= 1e-5 * (|A||X|) per entry for FP32
and the three-term split ("split3", six products); the two-term split
("split2", three products) keeps 16 bits per operand and is held to its bound
3 * 2^-16 * (|A||X|)."""
import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import convert, synth
from sable_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def random_vbr(seed, rsizes, csizes, p, dense_frac=0.5):
    rng = np.random.default_rng(seed)
    present = rng.random((len(rsizes), len(csizes))) < p

    def fill(rng, h, w, a, b):
        v = rng.uniform(-1, 1, (h, w)).astype(np.float32)
        if rng.random() < dense_frac:
            return v
        return v * synth.block_pattern(rng, h, w, rng.uniform(0.02, 0.5), "uniform")

    return synth.assemble(rng, np.asarray(rsizes), np.asarray(csizes), present, fill)


def tol_of(tc):
    return oracle.TOL_SPLIT2 if tc == "split2" else oracle.TOL


def spmm_check(m, dense, X, tc=False, **opts):
    import torch
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    plan = Plan(comp, spmm_tc=tc, **opts)
    Y = plan.spmm(torch.as_tensor(X).cuda()).cpu().numpy()
    Yr, Ya = oracle.spmm_vbr(m, X)
    r = oracle.report(Y, Yr, Ya, tol_of(tc))
    plan.close()
    return Y, r


@pytest.mark.parametrize("case", ["spmm400_N32_d0", "spmm400_N8_d30"])
@pytest.mark.parametrize("tc", [False, "split2", "split3"])
def test_vs_reference_c(golden, cuda, case, tc):
    meta = golden.meta(case)
    m = synth.spmm_50k(meta["seed"], n=meta["n"], parts=meta["parts"], p=meta["p"])
    X = synth.dense_operand(m.n_cols, meta["N"], meta["x_seed"])
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    dense = np.ones(m.n_blocks, bool) if meta["density"] == 0 else \
        convert.block_density_pct(convert.block_nnz(m.val, bt), bt) > meta["density"]
    Y, r = spmm_check(m, dense, X, tc=tc)
    rc = oracle.report(Y, golden.arr(case, "Y"), oracle.spmm_vbr(m, X)[1], tol_of(tc))
    assert r["pass"] and rc["pass"], (r, rc)


@pytest.mark.parametrize("N", [4, 8, 32, 64, 128, 256, 512])
def test_widths(cuda, N):
    m = random_vbr(3, [23, 64, 130, 5, 48], [17, 40, 96, 3, 128, 9], 0.7)
    X = synth.dense_operand(m.n_cols, N, 4)
    rng = np.random.default_rng(5)
    Y, r = spmm_check(m, rng.random(m.n_blocks) < 0.5, X)
    assert r["pass"], r


@pytest.mark.parametrize("chunk_bytes", [0, 4096])
@pytest.mark.parametrize("tc", [False, "split2", "split3"])
@pytest.mark.parametrize("split_layout", ["mixed", "separate"])
def test_split_tiles_and_edges(cuda, chunk_bytes, tc, split_layout):
    m = random_vbr(6, [1, 300, 64, 2, 100], [1, 250, 3, 64, 77, 2, 31], 0.8)
    X = synth.dense_operand(m.n_cols, 64, 7)
    rng = np.random.default_rng(8)
    Y, r = spmm_check(m, rng.random(m.n_blocks) < 0.5, X, tc=tc, chunk_bytes=chunk_bytes, split_layout=split_layout)
    assert r["pass"], r


def test_spmm_host_entry(cuda):
    import torch
    m = random_vbr(9, np.full(12, 40), np.full(12, 40), 0.4)
    X = synth.dense_operand(m.n_cols, 32, 10)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, np.ones(m.n_blocks, bool))
    plan = Plan(comp)
    Yd = plan.spmm(torch.as_tensor(X).cuda()).cpu().numpy()
    Yh = plan.spmm_host(X)
    np.testing.assert_array_equal(Yd, Yh)


@pytest.mark.parametrize("N", [32, 128])
@pytest.mark.parametrize("tc", [False, "split3"])
def test_large_items_spmm_only(cuda, N, tc):
    """Work items above the shared-memory staging size (256 KB: whole block
    rows per item, long K loops, no split tiles): SpMM parity, and SpMV and
    the batch's staged executors refuse the plan instead of staging records
    that do not fit; a batch takes it when its matrix runs on the tcgen05
    kernel (split BF16, which streams records), with the plan's own bits."""
    import torch
    from sable_gb300 import _lib
    from sable_gb300.batch import Batch
    m = random_vbr(61, np.full(12, 120), np.full(20, 40), 0.5, dense_frac=0.7)  # ~0.1-0.2 MB per block row
    X = synth.dense_operand(m.n_cols, N, 62)
    rng = np.random.default_rng(63)
    dense = rng.random(m.n_blocks) < 0.7
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    plan = Plan(comp, spmm_tc=tc, chunk_bytes=262144, split_layout="separate")
    assert plan.stats()["scratch_floats"] == 0  # no tile is split
    Y = plan.spmm(torch.as_tensor(X).cuda()).cpu().numpy()
    Yr, Ya = oracle.spmm_vbr(m, X)
    r = oracle.report(Y, Yr, Ya, tol_of(tc))
    assert r["pass"], r
    with pytest.raises(_lib.SableError, match="SpMM-only"):
        plan.spmv(torch.zeros(m.n_cols, device="cuda"))
    if tc:
        b = Batch([plan], [N])
        Xd = torch.as_tensor(X).cuda()
        Yb = torch.empty(m.n_rows, N, device="cuda")
        b.run([Xd], [Yb])
        b.check()
        np.testing.assert_array_equal(Yb.cpu().numpy(), Y)
        b.close()
    else:
        with pytest.raises(_lib.SableError, match="staging"):
            Batch([plan], [N])
    with pytest.raises(_lib.SableError, match="staging"):
        Batch([plan], [1])
    plan.close()
