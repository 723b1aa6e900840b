"""Batched SpMV / SpMM (one persistent kernel for many matrices) against the
FP64 oracle, against the per-matrix entry points, with and without a CUDA
graph, and the batch's argument checks."""
import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import _lib, convert, synth
from sable_gb300.batch import Batch
from sable_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def random_vbr(seed, n, lo=4, hi=128, p=0.05):
    rng = np.random.default_rng(seed)
    rs = synth.sizes_until(rng, lo, hi, n)
    cs = synth.sizes_until(rng, lo, hi, n)
    present = rng.random((len(rs), len(cs))) < p
    present[0, 0] = True

    def fill(rng, h, w, a, b):
        v = rng.uniform(-1, 1, (h, w)).astype(np.float32)
        return v if rng.random() < 0.5 else v * synth.block_pattern(rng, h, w, rng.uniform(0.02, 0.4), "uniform")

    return synth.assemble(rng, rs, cs, present, fill)


def make(seed, n, width, tc=False, chunk_bytes=0):
    m = random_vbr(seed, n)
    dense = np.random.default_rng(seed + 1).random(m.n_blocks) < 0.6
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    return m, comp, Plan(comp, spmm_tc=tc, chunk_bytes=chunk_bytes)


CASES = [  # (n, width, tc, chunk_bytes)
    (300, 1, False, 0), (2000, 1, False, 4096), (1500, 64, False, 0), (900, 64, "split3", 4096),
    (700, 32, "split2", 0), (1200, 8, False, 0), (500, 128, "split3", 0), (4000, 1, False, 0),
    (64, 4, False, 0), (2500, 96, False, 8192), (800, 16, False, 0), (3000, 1, False, 16384),
]


def build_batch(use_graph, seed0=10):
    import torch
    mats, plans, xs = [], [], []
    for k, (n, w, tc, cb) in enumerate(CASES):
        m, comp, p = make(seed0 + k, n, w, tc, cb)
        mats.append((m, comp))
        plans.append(p)
        rng = np.random.default_rng(100 + k)
        x = rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)
        xs.append(torch.as_tensor(x).cuda())
    b = Batch(plans, [c[1] for c in CASES], use_graph=use_graph)
    return b, mats, plans, xs


def check_outputs(mats, xs, ys):
    for k, ((m, comp), x, y) in enumerate(zip(mats, xs, ys)):
        w, tc = CASES[k][1], CASES[k][2]
        xn = x.cpu().numpy()
        if w == 1:
            yr, ya = oracle.spmv_vbrc(comp, xn)
        else:
            yr, ya = oracle.spmm_vbr(m, xn)
        tol = oracle.TOL_SPLIT2 if tc == "split2" else oracle.TOL
        r = oracle.report(y.cpu().numpy(), yr, ya, tol)
        assert r["pass"], (k, CASES[k], r)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_oracle(cuda, use_graph):
    b, mats, plans, xs = build_batch(use_graph)
    ys = b.outputs()
    b.run(xs, ys)
    b.check()
    check_outputs(mats, xs, ys)
    info = b.info()
    assert info["n_mats"] == len(CASES) and info["n_units"] >= sum(p.stats()["n_chunks"] for p in plans)


def test_batch_spmv_bitwise_equals_single_plan(cuda):
    """SpMV units run the per-item body: identical bits to sable_spmv."""
    import torch
    b, mats, plans, xs = build_batch(True)
    ys = b.outputs()
    b.run(xs, ys)
    torch.cuda.synchronize()
    for k, (p, x, y) in enumerate(zip(plans, xs, ys)):
        if CASES[k][1] == 1:
            assert torch.equal(p.spmv(x), y), k


def test_batch_repeat_and_new_pointers(cuda):
    import torch
    b, mats, plans, xs = build_batch(True, seed0=40)
    for p in plans:
        p.close()  # the batch keeps its own copy of the records
    ys1 = b.outputs()
    b.run(xs, ys1)
    ys2 = b.outputs()
    b.run(xs, ys2)          # new result pointers: the table is re-uploaded
    b.run(xs, ys2)          # and replayed as is
    xs3 = [x.clone() * 2 for x in xs]
    ys3 = b.outputs()
    b.run(xs3, ys3)
    b.check()
    torch.cuda.synchronize()
    for a, c, d in zip(ys1, ys2, ys3):
        assert torch.equal(a, c)
        assert torch.equal(a * 2, d)


def test_batch_one_ctas_per_sm(cuda):
    b, mats, plans, xs = build_batch(False, seed0=70)
    b2 = Batch(plans, [c[1] for c in CASES], ctas_per_sm=1, use_graph=False)
    ys = b2.outputs()
    b2.run(xs, ys)
    b2.check()
    check_outputs(mats, xs, ys)
    import torch
    assert b2.info()["n_ctas"] <= torch.cuda.get_device_properties(0).multi_processor_count


def test_batch_argument_checks(cuda):
    m, comp, p = make(5, 200, 1)
    with pytest.raises(_lib.SableError) as e:
        Batch([p], [6])
    assert e.value.code == -4
    with pytest.raises(ValueError):
        Batch([p], [1, 4])
    b = Batch([p], [1])
    import torch
    with pytest.raises(ValueError):
        b.run([torch.zeros(3, device="cuda")], [torch.zeros(m.n_rows, device="cuda")])


def test_batch_256_generator_distribution(cuda):
    """40 matrices from the 256-matrix batch workload's generator (rows
    log-uniform in [1000, 20000], partitions U[4,128], block p = 0.02, SpMM
    width 64 for every second matrix), each with the learned block choice at
    its width, SpMM matrices in split BF16 (three terms) on the tcgen05 kernel
    with whole block rows per item, all in one CUDA-graph launch; every
    output against the FP64 oracle."""
    import torch
    from sable_gb300 import blockmodel
    mats, widths = synth.batch_256(count=40)
    model = blockmodel.MLPModel.load()
    plans, comps, xs = [], [], []
    rng = np.random.default_rng(256)
    for m, w in zip(mats, widths):
        bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
        dense = model.choose_dense(convert.block_features(m.val, bt, w))
        comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense, bt=bt)
        comps.append(comp)
        shape = {} if w == 1 else {"row_tile": 128, "chunk_bytes": 262144}   # whole block rows (tcgen05)
        plans.append(Plan(comp, spmm_tc="split3", split_layout="mixed" if w == 1 else "separate", **shape))
        xs.append(torch.as_tensor(rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)).cuda())
    b = Batch(plans, widths, use_graph=True)
    ys = b.outputs()
    b.run(xs, ys)
    b.check()
    worst = 0.0
    for k, (m, comp, w, x, y) in enumerate(zip(mats, comps, widths, xs, ys)):
        xn = x.cpu().numpy()
        yr, ya = oracle.spmv_vbrc(comp, xn) if w == 1 else oracle.spmm_vbr(m, xn)
        r = oracle.report(y.cpu().numpy(), yr, ya)
        assert r["pass"], (k, w, r)
        worst = max(worst, r["max"])
    assert worst <= oracle.TOL


def test_batch_tcgen05_spmm_bitwise_equals_single_plan(cuda):
    """Split-BF16 SpMM matrices whose plans hold tcgen05 panel terms run on the
    tcgen05 kernel inside the batch (one launch per N-slice width, widths 32
    to 256, a 96-wide matrix sharing the 128-wide group's launch): identical
    bits to each plan's own sable_spmm, next to a plan on the mma.sync kernel
    (in the persistent kernel's queue) and SpMV matrices, all within the
    tolerance of FP64."""
    import torch
    cases = [(900, 64, "split3", "umma", 4096), (700, 32, "split3", "umma", 0), (600, 96, "split3", "umma", 0),
             (500, 128, "split3", "umma", 8192), (400, 256, "split3", "umma", 0), (800, 64, "split2", "umma", 0),
             (650, 64, "split3", "mma_sync", 0), (1500, 1, False, "umma", 0), (300, 8, False, "umma", 0)]
    mats, plans, xs = [], [], []
    for k, (n, w, tc, kern, cb) in enumerate(cases):
        m = random_vbr(500 + k, n)
        dense = np.random.default_rng(600 + k).random(m.n_blocks) < 0.7
        comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
        mats.append((m, comp))
        plans.append(Plan(comp, spmm_tc=tc, chunk_bytes=cb, tc_kernel=kern,
                          split_layout="mixed" if w == 1 else "separate"))
        rng = np.random.default_rng(700 + k)
        xs.append(torch.as_tensor(rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)).cuda())
    widths = [c[1] for c in cases]
    for use_graph in (False, True):
        b = Batch(plans, widths, use_graph=use_graph)
        ys = b.outputs()
        b.run(xs, ys)
        b.run(xs, ys)
        b.check()
        torch.cuda.synchronize()
        for k, ((m, comp), p, x, y, c) in enumerate(zip(mats, plans, xs, ys, cases)):
            w, tc, kern = c[1], c[2], c[3]
            xn = x.cpu().numpy()
            yr, ya = oracle.spmv_vbrc(comp, xn) if w == 1 else oracle.spmm_vbr(m, xn)
            r = oracle.report(y.cpu().numpy(), yr, ya, oracle.TOL_SPLIT2 if tc == "split2" else oracle.TOL)
            assert r["pass"], (k, c, r)
            if w >= 32 and kern == "umma":
                assert torch.equal(p.spmm(x), y), (k, c)
        b.close()


def test_batch_per_warp_spmv_plans(cuda):
    """SpMV matrices whose plans hold compact records (the per-warp executor)
    run on the per-warp kernel inside the batch, with a per-item matrix
    table and split tiles combined in the kernel: identical bits to each
    plan's own sable_spmv, next to SpMV matrices on the batch's ring and SpMM
    matrices on the tcgen05 kernel; with and without a graph, twice."""
    import torch
    cases = [(3000, 1, "warp_items", 16, 8192), (1200, 1, "warp_items", 8, 4096), (5000, 1, "warp_items", 32, 32768),
             (200, 1, "warp_items", 64, 4096), (2000, 1, "items", 128, 4096), (900, 64, "items", 128, 0),
             (4000, 1, "warp_items", 16, 32768)]
    mats, plans, xs = [], [], []
    for k, (n, w, sched, rt, cb) in enumerate(cases):
        m = random_vbr(800 + k, n)
        dense = np.random.default_rng(900 + k).random(m.n_blocks) < 0.5
        comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
        mats.append((m, comp))
        plans.append(Plan(comp, schedule=sched, row_tile=rt, chunk_bytes=cb, spmm_tc="split3" if w > 1 else False))
        rng = np.random.default_rng(1000 + k)
        xs.append(torch.as_tensor(rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)).cuda())
    assert any(p.stats()["scratch_floats"] > 0 for p, c in zip(plans, cases) if c[2] == "warp_items")
    widths = [c[1] for c in cases]
    for use_graph in (False, True):
        b = Batch(plans, widths, use_graph=use_graph)
        ys = b.outputs()
        for _ in range(2):
            b.run(xs, ys)
        b.check()
        torch.cuda.synchronize()
        for k, ((m, comp), p, x, y, c) in enumerate(zip(mats, plans, xs, ys, cases)):
            xn = x.cpu().numpy()
            yr, ya = oracle.spmv_vbrc(comp, xn) if c[1] == 1 else oracle.spmm_vbr(m, xn)
            r = oracle.report(y.cpu().numpy(), yr, ya)
            assert r["pass"], (k, c, r)
            if c[1] == 1:
                assert torch.equal(p.spmv(x), y), (k, c)
        b.close()


def test_tune_batch_picks_a_shape_per_class(cuda):
    """The batch autotuner times whole batches over the SpMV executors and
    item shapes and the SpMM item sizes; the batch it returns gives the FP64
    oracle's results."""
    import torch
    from sable_gb300 import autotune
    mats, widths = synth.batch_256(count=12)
    rng = np.random.default_rng(12)
    comps, xs, ys = [], [], []
    for m, w in zip(mats, widths):
        dense = rng.random(m.n_blocks) < 0.6
        comps.append(convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense))
        xs.append(torch.as_tensor(rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)).cuda())
        ys.append(torch.empty(m.n_rows if w == 1 else (m.n_rows, w), device="cuda"))
    b, table = autotune.tune_batch(comps, widths, xs, ys, reps=3)
    assert len([t for t in table if t["ms"] is not None]) >= len(autotune.BATCH_SPMV_SHAPES)
    b.run(xs, ys)
    b.check()
    for m, comp, w, x, y in zip(mats, comps, widths, xs, ys):
        xn = x.cpu().numpy()
        yr, ya = oracle.spmv_vbrc(comp, xn) if w == 1 else oracle.spmm_vbr(m, xn)
        r = oracle.report(y.cpu().numpy(), yr, ya)
        assert r["pass"], (w, r)
    b.close()
