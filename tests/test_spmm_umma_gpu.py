"""Split-BF16 SpMM on the tcgen05 tensor cores (TMEM accumulators) against the
FP64 oracle, next to the warp-level mma.sync kernel on the same plans.

Edge shapes of the transposed product: tile heights 1..128 (the MMA's N is
the height rounded up to 16), panel widths that leave a partial last K step,
N-slices narrower than the 128-row MMA (N = 32, 64, 96) and several slices
(N = 256), items without a dense panel (CSR only), tiles split over several
items (partial sums), and whole-block-row items with long K loops.
Tolerance: 1e-5 * (|A||X|) per entry for split3 (six products), the split2
bound 3 * 2^-16 * (|A||X|) for split2 (three products)."""
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


def run(m, dense, X, tc, kernel, **opts):
    import torch
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    plan = Plan(comp, spmm_tc=tc, tc_kernel=kernel, **opts)
    Xd = torch.as_tensor(X).cuda()
    Y1 = plan.spmm(Xd).cpu().numpy()
    Y2 = plan.spmm(Xd).cpu().numpy()
    plan.check()
    plan.close()
    assert np.array_equal(Y1, Y2), "two calls differ"
    Yr, Ya = oracle.spmm_vbr(m, X)
    return Y1, oracle.report(Y1, Yr, Ya, oracle.TOL_SPLIT2 if tc == "split2" else oracle.TOL)


HEIGHTS = [1, 7, 16, 17, 33, 64, 100, 128, 130]
WIDTHS = [1, 3, 15, 16, 17, 40, 77, 128]


@pytest.mark.parametrize("N", [32, 64, 96, 128, 256])
@pytest.mark.parametrize("tc", ["split2", "split3"])
@pytest.mark.parametrize("kernel", ["umma", "mma_sync"])
def test_heights_widths_slices(cuda, N, tc, kernel):
    m = random_vbr(71, HEIGHTS, WIDTHS, 0.6)
    X = synth.dense_operand(m.n_cols, N, 72)
    rng = np.random.default_rng(73)
    _, r = run(m, rng.random(m.n_blocks) < 0.6, X, tc, kernel)
    assert r["pass"], r


@pytest.mark.parametrize("chunk_bytes", [4096, 16384, 262144])
@pytest.mark.parametrize("split_layout", ["mixed", "separate"])
def test_items_and_split_tiles(cuda, chunk_bytes, split_layout):
    m = random_vbr(74, [128, 96, 1, 50, 128, 20], [64, 3, 128, 90, 17, 128, 40], 0.8, dense_frac=0.7)
    X = synth.dense_operand(m.n_cols, 128, 75)
    rng = np.random.default_rng(76)
    _, r = run(m, rng.random(m.n_blocks) < 0.7, X, "split3", "umma", chunk_bytes=chunk_bytes,
               split_layout=split_layout)
    assert r["pass"], r


@pytest.mark.parametrize("frac", [0.0, 1.0])
def test_all_csr_and_all_dense(cuda, frac):
    m = random_vbr(77, [40, 128, 7, 64], [33, 128, 16, 90], 0.8)
    X = synth.dense_operand(m.n_cols, 64, 78)
    _, r = run(m, np.full(m.n_blocks, frac > 0.5), X, "split3", "umma")
    assert r["pass"], r


def test_umma_matches_mma_sync_closely(cuda):
    """The two tensor-core kernels compute the same split products in a
    different order: both within the parity tolerance of FP64, and within
    a few FP32 rounding steps of each other."""
    m = random_vbr(79, [50, 80, 20, 64, 128], [60, 30, 128, 45, 20, 77], 0.7, dense_frac=0.8)
    X = synth.dense_operand(m.n_cols, 128, 80)
    dense = np.random.default_rng(81).random(m.n_blocks) < 0.8
    Yu, ru = run(m, dense, X, "split3", "umma")
    Ym, rm = run(m, dense, X, "split3", "mma_sync")
    assert ru["pass"] and rm["pass"], (ru, rm)
    _, Ya = oracle.spmm_vbr(m, X)
    assert np.max(np.abs(Yu - Ym) / np.maximum(Ya, 1e-30)) < 5e-6


def test_spmm_50k_shape_sample(cuda):
    """A 5000^2 matrix from the 50000^2 SpMM workload's generator (partition
    sizes 20..80, 60 % dense blocks), N = 128, with the SpMM entry point's
    launch shape (whole block rows per item)."""
    m = synth.spmm_50k(seed=1015, n=5000, parts=100, p=0.05)
    X = synth.dense_operand(m.n_cols, 128, 82)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    dense = convert.block_density_pct(convert.block_nnz(m.val, bt), bt) > 30
    _, r = run(m, dense, X, "split3", "umma", chunk_bytes=262144, split_layout="separate", row_tile=128)
    assert r["pass"], r


@pytest.mark.parametrize("N", [32, 128])
def test_spmm_50k_full_size(cuda, N):
    """The full 50000^2 SpMM workload (1000 x 1000 partitions of 20..80, block
    p = 0.01, 60 % dense blocks) at N = 32 and 128, with the learned block
    choice and the entry point's launch shape, against the FP64 oracle on
    every output."""
    from sable_gb300 import blockmodel
    m = synth.spmm_50k()
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    dense = blockmodel.MLPModel.load().choose_dense(convert.block_features(m.val, bt, N))
    X = synth.dense_operand(m.n_cols, N, 7)
    _, r = run(m, dense, X, "split3", "umma", chunk_bytes=262144, split_layout="separate", row_tile=128)
    assert r["pass"] and r["rows"] == m.n_rows * N, r


@pytest.mark.parametrize("N", [36, 100, 132, 260])
@pytest.mark.parametrize("tc", ["split2", "split3"])
def test_widths_strides_and_the_entry_without_allocation(cuda, N, tc):
    """Widths that are not multiples of 8 or of the N-slice width, X and Y
    inside wider rows (leading dimensions above N): within the tolerance of
    FP64, nothing written past column N of Y, and bit-identical to the entry
    point without allocation, which runs the same kernel with its split-tile
    scratch in the library's fixed array."""
    import torch
    from sable_gb300 import _lib
    m = random_vbr(83, [40, 128, 7, 64, 100], [33, 128, 16, 90, 5], 0.8, dense_frac=0.8)
    dense = np.random.default_rng(84).random(m.n_blocks) < 0.8
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    plan = Plan(comp, spmm_tc=tc, tc_kernel="umma")
    Xw = torch.as_tensor(synth.dense_operand(m.n_cols, N + 12, 85)).cuda()
    X = Xw[:, :N]                      # leading dimension N + 12
    Yw = torch.full((m.n_rows, N + 8), float("nan"), device="cuda")
    Y = Yw[:, :N]
    plan.spmm(X, Y)
    Yn = torch.full((m.n_rows, N), float("nan"), device="cuda")
    lib = _lib.load()
    _lib.check(lib.sable_spmm_noalloc(plan.handle, X.data_ptr(), X.stride(0), Yn.data_ptr(), N, N,
                                      torch.cuda.current_stream().cuda_stream), "sable_spmm_noalloc")
    plan.check()
    Yh = Y.cpu().numpy()
    assert np.array_equal(Yh, Yn.cpu().numpy())
    assert torch.isnan(Yw[:, N:]).all()          # nothing written past N
    Yr, Ya = oracle.spmm_vbr(m, X.cpu().numpy())
    r = oracle.report(Yh, Yr, Ya, oracle.TOL_SPLIT2 if tc == "split2" else oracle.TOL)
    assert r["pass"], r
    plan.close()
