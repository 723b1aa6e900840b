"""SpMV parity on the GPU (libsable through its C ABI) against the FP64
oracle and the reference's generated C.  Tolerance: per row
|y_gpu - y_ref| <= 1e-5 * (|A||x|)_row."""
import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import blockmodel, convert, synth
from sable_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def plan_and_ref(m, dense_mask, x, **opts):
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense_mask)
    plan = Plan(comp, **opts)
    y_ref, yabs = oracle.spmv_vbrc(comp, x.astype(np.float64))
    return plan, comp, y_ref, yabs


def run(plan, x):
    import torch
    xd = torch.as_tensor(x).cuda()
    y = plan.spmv(xd)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def random_vbr(seed, rsizes, csizes, p, dense_frac=0.5, empty_rows=()):
    rng = np.random.default_rng(seed)
    rsizes, csizes = np.asarray(rsizes), np.asarray(csizes)
    present = rng.random((len(rsizes), len(csizes))) < p
    for a in empty_rows:
        present[a, :] = False

    def fill(rng, h, w, a, b):
        v = rng.uniform(-1, 1, (h, w)).astype(np.float32)
        if rng.random() < dense_frac:
            return v
        return v * synth.block_pattern(rng, h, w, rng.uniform(0.02, 0.5), "uniform")

    return synth.assemble(rng, rsizes, csizes, present, fill)


def test_example_canon(golden, cuda):
    ex = synth.VbrMatrix(*[np.asarray(a) for a in golden.arrays("example_arrays")])
    ex.val = ex.val.astype(np.float32)
    plan, comp, y_ref, yabs = plan_and_ref(ex, np.ones(ex.n_blocks, bool), np.ones(11, np.float32))
    y = run(plan, np.ones(11, np.float32))
    np.testing.assert_array_equal(y, golden.arr("example_canon", "spmv"))


def test_example2_density80_canon(golden, cuda):
    ex2 = synth.VbrMatrix(*[np.asarray(a) for a in golden.arrays("example2_arrays")])
    ex2.val = ex2.val.astype(np.float32)
    bt = convert.block_table(ex2.rpntr, ex2.cpntr, ex2.bpntrb, ex2.bpntre, ex2.bindx, ex2.indx)
    dense = convert.block_density_pct(convert.block_nnz(ex2.val, bt), bt) > 80
    plan, comp, y_ref, yabs = plan_and_ref(ex2, dense, np.ones(11, np.float32))
    np.testing.assert_array_equal(comp.ublocks, golden.arr("example2_vbrc", "ublocks"))
    y = run(plan, np.ones(11, np.float32))
    canon = golden.arr("example_canon", "spmv_sparse")
    np.testing.assert_array_equal(y[: len(canon)], canon)


@pytest.mark.parametrize("case,density", [("spmv1000_d0", 0), ("spmv1000_d50", 50), ("spmv1000_rf", None)])
def test_spmv1000_vs_reference_c(golden, cuda, case, density):
    meta = golden.meta(case)
    m = synth.spmv_1000(meta["seed"])
    x = synth.vector(m.n_cols, meta["x_seed"])
    model = blockmodel.RFTableModel() if density is None else None
    dense = convert.choose_dense(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, density=density,
                                 model=model)
    plan, comp, y_ref, yabs = plan_and_ref(m, dense, x)
    y = run(plan, x)
    r_c = oracle.report(y, golden.arr(case, "y"), yabs)
    r_o = oracle.report(y, y_ref, yabs)
    assert r_c["pass"] and r_o["pass"], (r_c, r_o)


@pytest.mark.parametrize("row_tile", [128, 64, 17])
@pytest.mark.parametrize("chunk_bytes", [0, 4096])
@pytest.mark.parametrize("schedule,split_layout", [("persistent", "mixed"), ("items", "mixed"), ("items", "separate"),
                                                   ("warp_items", "mixed"), ("warp_items", "separate")])
def test_edge_shapes(cuda, row_tile, chunk_bytes, schedule, split_layout):
    """Tall block rows (tile splits), width-1 / height-1 partitions, empty
    block rows, tiny work items (split tiles combined by the combine launch)."""
    rs = [1, 300, 5, 1, 64, 129, 7, 2, 40]
    cs = [1, 3, 200, 1, 9, 33, 128, 2, 4, 77]
    m = random_vbr(7, rs, cs, 0.6, empty_rows=(2,))
    x = synth.vector(m.n_cols, 8)
    rng = np.random.default_rng(9)
    dense = rng.random(m.n_blocks) < 0.5
    plan, comp, y_ref, yabs = plan_and_ref(m, dense, x, row_tile=row_tile, chunk_bytes=chunk_bytes, schedule=schedule,
                                           split_layout=split_layout)
    y = run(plan, x)
    r = oracle.report(y, y_ref, yabs)
    assert r["pass"], r
    assert np.all(y[m.rpntr[2]:m.rpntr[3]] == 0)


@pytest.mark.parametrize("dense_all", [True, False])
def test_all_dense_all_sparse(cuda, dense_all):
    m = random_vbr(11, np.full(20, 37), np.full(25, 29), 0.3)
    x = synth.vector(m.n_cols, 12)
    plan, comp, y_ref, yabs = plan_and_ref(m, np.full(m.n_blocks, dense_all), x)
    y = run(plan, x)
    assert oracle.report(y, y_ref, yabs)["pass"]


@pytest.mark.parametrize("schedule", ["items", "warp_items"])
def test_one_huge_block_row(cuda, schedule):
    """One block row with many blocks: dozens of work items on one tile."""
    m = random_vbr(13, [96], np.full(400, 50), 0.9, dense_frac=0.7)
    x = synth.vector(m.n_cols, 14)
    rng = np.random.default_rng(15)
    plan, comp, y_ref, yabs = plan_and_ref(m, rng.random(m.n_blocks) < 0.6, x, schedule=schedule)
    assert plan.stats()["n_chunks"] > 20
    y = run(plan, x)
    assert oracle.report(y, y_ref, yabs)["pass"]


ROW_LENGTHS = [0, 1, 2, 3, 7, 8, 9, 15, 16, 17, 31, 32, 33, 63, 64, 65, 255, 256, 257, 300, 0, 0, 5, 1]


@pytest.mark.parametrize("row_tile", [8, 17, 32, 64, 128])
@pytest.mark.parametrize("chunk_bytes", [4096, 32768])
@pytest.mark.parametrize("dense_frac", [0.0, 0.5])
def test_compact_csr_row_lengths(cuda, row_tile, chunk_bytes, dense_frac):
    """The per-warp executor's CSR pass (8 entries per lane, 256 per warp
    step, rows summed by a segmented scan over the lanes) on rows whose
    lengths straddle the lane and step boundaries, with empty rows and rows
    longer than a step; tiles of up to 64 rows (128 is capped)."""
    rng = np.random.default_rng(41)
    rs, cs = [64, 40, 3, 64], [600, 700, 350]

    def fill(r, h, w, a, b):
        v = r.uniform(-1, 1, (h, w)).astype(np.float32)
        if r.random() < dense_frac:
            return v
        keep = np.zeros((h, w), bool)
        for i in range(h):
            n = min(ROW_LENGTHS[(i + 7 * a + 3 * b) % len(ROW_LENGTHS)], w)
            keep[i, r.choice(w, n, replace=False)] = True
        return v * keep

    m = synth.assemble(rng, np.array(rs), np.array(cs), np.ones((len(rs), len(cs)), bool), fill)
    x = synth.vector(m.n_cols, 42)
    dense = np.zeros(m.n_blocks, bool) if dense_frac == 0 else rng.random(m.n_blocks) < dense_frac
    plan, comp, y_ref, yabs = plan_and_ref(m, dense, x, row_tile=row_tile, chunk_bytes=chunk_bytes,
                                           schedule="warp_items")
    y = run(plan, x)
    r = oracle.report(y, y_ref, yabs)
    assert r["pass"], r
    y2 = run(plan, x)  # split-tile counters reset themselves; same bits again
    np.testing.assert_array_equal(y, y2)
    plan.check()


def test_compact_plan_is_spmv_only(cuda):
    """A plan of the per-warp executor holds compact records: SpMM, and a
    batch asked for a width above 1, refuse it with SABLE_ERR_UNSUPPORTED
    instead of misreading them."""
    import torch
    from sable_gb300 import _lib
    from sable_gb300.batch import Batch
    m = synth.spmv_1000()
    plan, comp, y_ref, yabs = plan_and_ref(m, np.ones(m.n_blocks, bool), synth.vector(m.n_cols, 1),
                                           schedule="warp_items")
    X = torch.zeros(m.n_cols, 8, device="cuda")
    with pytest.raises(_lib.SableError, match="SpMV only"):
        plan.spmm(X)
    with pytest.raises(_lib.SableError, match="SpMV only"):
        Batch([plan], [4])


def test_deterministic_and_host_entry(cuda):
    import torch
    m = synth.spmv_1000()
    x = synth.vector(m.n_cols, 21)
    rng = np.random.default_rng(22)
    plan, comp, y_ref, yabs = plan_and_ref(m, rng.random(m.n_blocks) < 0.5, x, chunk_bytes=4096)
    xd = torch.as_tensor(x).cuda()
    y1 = plan.spmv(xd).cpu().numpy()
    y2 = plan.spmv(xd).cpu().numpy()
    np.testing.assert_array_equal(y1, y2)
    y3 = plan.spmv_host(x)
    np.testing.assert_array_equal(y1, y3)
    assert oracle.report(y1, y_ref, yabs)["pass"]
    plan.check()  # no bounded device wait ran out


@pytest.mark.parametrize("schedule", ["items", "warp_items"])
def test_host_entry_pinned_buffers(cuda, schedule):
    """sable_spmv_host with pinned host buffers (read and written by the
    kernels themselves, no copy-engine transfer), 16-byte aligned and not:
    the same bits as the device-buffer SpMV, call after call."""
    import torch
    from sable_gb300 import _lib
    m = synth.spmv_1000()
    rng = np.random.default_rng(23)
    plan, comp, y_ref, yabs = plan_and_ref(m, rng.random(m.n_blocks) < 0.5, synth.vector(m.n_cols, 24),
                                           schedule=schedule, chunk_bytes=4096)
    x = synth.vector(m.n_cols, 24)
    y_dev = plan.spmv(torch.as_tensor(x).cuda()).cpu().numpy()
    stream = torch.cuda.current_stream().cuda_stream
    for off in (0, 1):
        xh = torch.zeros(m.n_cols + off, dtype=torch.float32).pin_memory()
        yh = torch.full((m.n_rows + off,), float("nan"), dtype=torch.float32).pin_memory()
        xh[off:] = torch.as_tensor(x)
        for _ in range(2):
            _lib.check(_lib.load().sable_spmv_host(plan.handle, xh[off:].data_ptr(), yh[off:].data_ptr(), stream),
                       "sable_spmv_host")
            np.testing.assert_array_equal(yh[off:].numpy(), y_dev)
    assert oracle.report(y_dev, y_ref, yabs)["pass"]
    plan.check()


@pytest.mark.parametrize("schedule", ["items", "warp_items"])
def test_host_entry_graph_follows_buffers(cuda, schedule):
    """With both buffers pinned, sable_spmv_host replays a graph of the x
    copy and the SpMV kept for the last (x, y) pair: alternating between two
    pinned pairs (the graph is captured again at every change), new x values
    in the same buffer (replayed as is), a pinned x with a pageable y and a
    pageable pair (the copy path): always the device-buffer SpMV's bits."""
    import torch
    from sable_gb300 import _lib
    m = synth.spmv_1000()
    rng = np.random.default_rng(25)
    plan, comp, y_ref, yabs = plan_and_ref(m, rng.random(m.n_blocks) < 0.5, synth.vector(m.n_cols, 26),
                                           schedule=schedule, chunk_bytes=4096)
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    pairs = [(torch.zeros(m.n_cols).pin_memory(), torch.zeros(m.n_rows).pin_memory()) for _ in range(2)]
    for k in range(6):
        xh, yh = pairs[k % 2]
        x = synth.vector(m.n_cols, 100 + k)
        xh.copy_(torch.as_tensor(x))
        yh.fill_(float("nan"))
        _lib.check(lib.sable_spmv_host(plan.handle, xh.data_ptr(), yh.data_ptr(), stream), "sable_spmv_host")
        np.testing.assert_array_equal(yh.numpy(), plan.spmv(torch.as_tensor(x).cuda()).cpu().numpy())
    x = synth.vector(m.n_cols, 200)
    xp = torch.as_tensor(x).pin_memory()
    yq = np.full(m.n_rows, np.nan, np.float32)          # pageable
    _lib.check(lib.sable_spmv_host(plan.handle, xp.data_ptr(), yq.ctypes.data, stream), "sable_spmv_host")
    y_dev = plan.spmv(torch.as_tensor(x).cuda()).cpu().numpy()
    np.testing.assert_array_equal(yq, y_dev)
    np.testing.assert_array_equal(plan.spmv_host(x), y_dev)
    plan.check()


def test_spmv_100k_full_size(cuda):
    """The 100000^2 workload (~20k blocks, ~5e7 stored values) at full size
    against the FP64 oracle, with the learned-form split (dense where the
    dense encoding is cheaper) and the all-CSR split of the reference RF."""
    import torch
    m = synth.spmv_100k()
    x = synth.vector(m.n_cols, 31)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    nnz = convert.block_nnz(m.val, bt)
    cheaper_dense = 4 * bt.size <= 8 * nnz + 4 * (bt.h + 1)
    for dense, schedule in ((cheaper_dense, "persistent"), (np.zeros(m.n_blocks, bool), "persistent"),
                            (cheaper_dense, "items"), (cheaper_dense, "warp_items"),
                            (np.ones(m.n_blocks, bool), "warp_items")):
        plan, comp, y_ref, yabs = plan_and_ref(m, dense, x, schedule=schedule)
        y = run(plan, x)
        r = oracle.report(y, y_ref, yabs)
        assert r["pass"], r
        # linearity: A(2x) == 2 A(x) exactly (scaling by 2 is exact in FP32)
        y2 = plan.spmv(torch.as_tensor(2 * x).cuda()).cpu().numpy()
        np.testing.assert_array_equal(y2, 2 * y)
        plan.close()
