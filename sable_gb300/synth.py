"""Seeded synthetic VBR workloads.

The reference's generator (synthesize_matrices/vbr_matrices_gen.py:36-113)
draws partitions with random_splits (:24-34), picks dense and "sparse"
blocks at random and fills every stored entry with 1.0.  The workloads here
follow the same structure with FP32 values and x drawn from U(-1, 1):

  spmv_1000      1000 x 1000, 10 x 10 random partitions, block p = 0.2,
                 half of the stored blocks fully dense, the rest 10 % dense.
  spmv_100k      100000 x 100000, 2000 x 2000 partitions of size U[10,100]
                 (adjusted to sum to 100000), block p = 0.005, density 1.0
                 w.p. 0.4 else U[0.05, 0.5], uniform or row-clustered.
  spmm_50k       50000 x 50000, 1000 x 1000 partitions in [20,80], block
                 p = 0.01, 60 % dense blocks, rest density U[0.05, 0.3].
  batch_256      256 square matrices, n log-uniform in [1000, 20000],
                 partitions U[4,128], block p = 0.02, dense fraction
                 U[0.2, 0.8], sparse density U[0.02, 0.4]; width 64 for half.
  blocks_200k    standalone blocks for the block model: h, w log-uniform in
                 [2, 256], density U[0.01, 1], uniform / banded /
                 row-clustered, N in {1, 8, 32, 128}.
Every generator is deterministic in its seed (numpy default_rng).

vbr_matrix_gen is the reference generator's drop-in: same signature, same
semantics, a .vbr file written, values 1.0 (see its docstring).
"""
from __future__ import annotations

import random
from dataclasses import dataclass, field

import numpy as np

SEED_BASE = 1000


@dataclass
class VbrMatrix:
    val: np.ndarray      # float32, all stored blocks, column-major each
    indx: np.ndarray     # int64
    bindx: np.ndarray    # int64
    rpntr: np.ndarray
    cpntr: np.ndarray
    bpntrb: np.ndarray
    bpntre: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n_rows(self) -> int:
        return int(self.rpntr[-1])

    @property
    def n_cols(self) -> int:
        return int(self.cpntr[-1])

    @property
    def n_blocks(self) -> int:
        return len(self.bindx)

    def arrays(self):
        return self.val, self.indx, self.bindx, self.rpntr, self.cpntr, self.bpntrb, self.bpntre


def random_splits(rng, n: int, parts: int) -> np.ndarray:
    """n split into `parts` positive sizes at distinct uniform cut points
    (the rule of random_splits, vbr_matrices_gen.py:24-34)."""
    cuts = np.sort(rng.choice(np.arange(1, n), size=parts - 1, replace=False))
    return np.diff(np.concatenate([[0], cuts, [n]])).astype(np.int64)


def sizes_with_sum(rng, parts: int, lo: int, hi: int, total: int) -> np.ndarray:
    """`parts` sizes drawn U[lo, hi], then random unit steps (decrements of
    sizes > lo, or increments of sizes < hi) until they sum to `total`."""
    if not parts * lo <= total <= parts * hi:
        raise ValueError(f"{parts} sizes in [{lo}, {hi}] cannot sum to {total}")
    s = rng.integers(lo, hi + 1, size=parts).astype(np.int64)
    diff = int(s.sum()) - total
    while diff != 0:
        if diff > 0:
            elig = np.nonzero(s > lo)[0]
            k = min(diff, len(elig))
            pick = rng.choice(elig, size=k, replace=False)
            s[pick] -= 1
            diff -= k
        else:
            elig = np.nonzero(s < hi)[0]
            k = min(-diff, len(elig))
            pick = rng.choice(elig, size=k, replace=False)
            s[pick] += 1
            diff += k
    return s


def sizes_until(rng, lo: int, hi: int, total: int) -> np.ndarray:
    """Sizes drawn U[lo, hi] until they cover `total`; the last one is cut to
    fit and merged into its neighbour when that would leave it below lo."""
    out = []
    acc = 0
    while acc < total:
        v = int(rng.integers(lo, hi + 1))
        out.append(v)
        acc += v
    out[-1] -= acc - total
    if out[-1] < lo and len(out) > 1:
        out[-2] += out.pop()
    return np.asarray(out, dtype=np.int64)


def block_pattern(rng, h: int, w: int, density: float, pattern: str) -> np.ndarray:
    """Boolean h x w nonzero mask (column-major flattening is applied later)."""
    hw = h * w
    k = int(round(density * hw))
    k = min(max(k, 1), hw)
    if k == hw:
        return np.ones((h, w), dtype=bool)
    m = np.zeros(hw, dtype=bool)
    if pattern == "uniform":
        m[rng.choice(hw, size=k, replace=False)] = True
        return m.reshape(h, w)
    if pattern == "row_clustered":
        r = min(h, max(1, -(-k // w)))
        r0 = int(rng.integers(0, h - r + 1))
        sub = np.zeros(r * w, dtype=bool)
        sub[rng.choice(r * w, size=k, replace=False)] = True
        mm = np.zeros((h, w), dtype=bool)
        mm[r0:r0 + r, :] = sub.reshape(r, w)
        return mm
    if pattern == "banded":
        # a diagonal band of the block wide enough to hold k entries
        ii, jj = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
        dist = np.abs(ii * (w / h) - jj).ravel()
        order = np.argsort(dist, kind="stable")
        band = order[: min(hw, int(k * 1.5) + 1)]
        m[rng.choice(band, size=k, replace=False)] = True
        return m.reshape(h, w)
    raise ValueError(pattern)


def assemble(rng, rsizes, csizes, present: np.ndarray, block_fill) -> VbrMatrix:
    """Build the VBR arrays from partition sizes and a block presence mask.
    block_fill(rng, h, w, a, b) returns the h x w float32 block (zeros allowed)."""
    rpntr = np.concatenate([[0], np.cumsum(rsizes)]).astype(np.int64)
    cpntr = np.concatenate([[0], np.cumsum(csizes)]).astype(np.int64)
    nbr = len(rsizes)
    rows, cols = np.nonzero(present)
    counts = np.bincount(rows, minlength=nbr)
    ends = np.cumsum(counts)
    bpntrb = np.where(counts > 0, ends - counts, -1).astype(np.int64)
    bpntre = np.where(counts > 0, ends, -1).astype(np.int64)
    h = rsizes[rows]
    w = csizes[cols]
    size = h * w
    indx = np.concatenate([[0], np.cumsum(size)]).astype(np.int64)
    val = np.empty(int(indx[-1]), dtype=np.float32)
    for k in range(len(rows)):
        blk = block_fill(rng, int(h[k]), int(w[k]), int(rows[k]), int(cols[k]))
        val[indx[k]: indx[k + 1]] = np.asarray(blk, dtype=np.float32).ravel(order="F")
    return VbrMatrix(val, indx, cols.astype(np.int64), rpntr, cpntr, bpntrb, bpntre)


def _values(rng, h, w):
    return rng.uniform(-1.0, 1.0, size=(h, w)).astype(np.float32)


def spmv_1000(seed: int = SEED_BASE + 0) -> VbrMatrix:
    rng = np.random.default_rng(seed)
    rs = random_splits(rng, 1000, 10)
    cs = random_splits(rng, 1000, 10)
    present = rng.random((10, 10)) < 0.2
    dense = rng.random((10, 10)) < 0.5

    def fill(rng, h, w, a, b):
        v = _values(rng, h, w)
        if not dense[a, b]:
            v = v * block_pattern(rng, h, w, 0.10, "uniform")
        return v

    m = assemble(rng, rs, cs, present, fill)
    m.meta = {"workload": "spmv_1000", "seed": seed}
    return m


def spmv_100k(seed: int = SEED_BASE + 1, n: int = 100000, parts: int = 2000, p: float = 0.005) -> VbrMatrix:
    rng = np.random.default_rng(seed)
    rs = sizes_with_sum(rng, parts, 10, 100, n)
    cs = sizes_with_sum(rng, parts, 10, 100, n)
    present = rng.random((parts, parts)) < p

    def fill(rng, h, w, a, b):
        v = _values(rng, h, w)
        if rng.random() < 0.4:
            return v
        d = rng.uniform(0.05, 0.5)
        pat = "uniform" if rng.random() < 0.5 else "row_clustered"
        return v * block_pattern(rng, h, w, d, pat)

    m = assemble(rng, rs, cs, present, fill)
    m.meta = {"workload": "spmv_100k", "seed": seed, "n": n, "parts": parts, "p": p}
    return m


def spmm_50k(seed: int = SEED_BASE + 2, n: int = 50000, parts: int = 1000, p: float = 0.01) -> VbrMatrix:
    rng = np.random.default_rng(seed)
    rs = sizes_with_sum(rng, parts, 20, 80, n)
    cs = sizes_with_sum(rng, parts, 20, 80, n)
    present = rng.random((parts, parts)) < p

    def fill(rng, h, w, a, b):
        v = _values(rng, h, w)
        if rng.random() < 0.6:
            return v
        return v * block_pattern(rng, h, w, rng.uniform(0.05, 0.3), "uniform")

    m = assemble(rng, rs, cs, present, fill)
    m.meta = {"workload": "spmm_50k", "seed": seed, "n": n, "parts": parts, "p": p}
    return m


def batch_256(seed: int = SEED_BASE + 3, count: int = 256, n_lo: int = 1000, n_hi: int = 20000):
    """Returns (matrices, widths): widths[i] = 64 for odd i (half of them), 1 otherwise."""
    rng = np.random.default_rng(seed)
    mats, widths = [], []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        rs = sizes_until(rng, 4, 128, n)
        cs = sizes_until(rng, 4, 128, n)
        present = rng.random((len(rs), len(cs))) < 0.02
        dense_frac = rng.uniform(0.2, 0.8)

        def fill(rng, h, w, a, b, dense_frac=dense_frac):
            v = _values(rng, h, w)
            if rng.random() < dense_frac:
                return v
            return v * block_pattern(rng, h, w, rng.uniform(0.02, 0.4), "uniform")

        m = assemble(rng, rs, cs, present, fill)
        m.meta = {"workload": "batch_256", "index": i, "seed": seed, "n": n}
        mats.append(m)
        widths.append(64 if i % 2 == 1 else 1)
    return mats, widths


@dataclass
class BlockSample:
    h: int
    w: int
    density: float
    pattern: str
    N: int
    block: np.ndarray  # float32 h x w


def blocks_200k(seed: int = SEED_BASE + 4, count: int = 200000, lo: int = 2, hi: int = 256):
    """Standalone blocks for the block model (structure only; values U(-1,1))."""
    rng = np.random.default_rng(seed)
    pats = ("uniform", "banded", "row_clustered")
    Ns = (1, 8, 32, 128)
    hs = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    ws = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    ds = rng.uniform(0.01, 1.0, size=count)
    ps = rng.integers(0, 3, size=count)
    nsel = rng.integers(0, 4, size=count)
    for k in range(count):
        h, w = int(hs[k]), int(ws[k])
        mask = block_pattern(rng, h, w, float(ds[k]), pats[ps[k]])
        yield BlockSample(h, w, float(ds[k]), pats[ps[k]], Ns[nsel[k]], _values(rng, h, w) * mask)


def vector(n: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-1.0, 1.0, size=n).astype(np.float32)


def dense_operand(n: int, N: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-1.0, 1.0, size=(n, N)).astype(np.float32)


# ---------------------------------------------------------------------------
# Drop-in for the reference's generator
# ---------------------------------------------------------------------------
def _sample_splits(n: int, parts: int) -> list[int]:
    """`parts` positive sizes summing to n: the gaps between parts - 1 cut
    points drawn without replacement from 1..n-1 (random_splits,
    synthesize_matrices/vbr_matrices_gen.py:24-34; Python's `random`)."""
    if n <= 0 or parts <= 0:
        raise ValueError("Both n and a must be positive integers.")
    cuts = sorted(random.sample(range(1, n), parts - 1))
    bounds = [0, *cuts, n]
    return [bounds[k + 1] - bounds[k] for k in range(parts)]


def vbr_matrix_gen(m: int, n: int, partitioning: str, row_split: int, col_split: int, num_dense: int,
                   perc_dense_zeros: int, num_sparse: int, dense_blocks_only: bool,
                   vbr_dir: str = "Generated_VBR") -> str:
    """Synthetic m x n VBR matrix written to <vbr_dir>/<name>.vbr (dense_blocks_only) or
    <vbr_dir>_Sparse/<name>.vbr; returns <name>.  The reference generator's signature and
    semantics (synthesize_matrices/vbr_matrices_gen.py:36-113): row_split x col_split
    partitions, uniform or drawn by random cuts ("nonuniform"); num_dense blocks at random
    with perc_dense_zeros % of their entries zero, then num_sparse of the remaining blocks
    with 10 nonzeros each; every nonzero is 1.0.  The draws come from Python's `random`
    module in the reference's order (partitions, dense blocks, sparse blocks, then the zero
    positions of every stored block in block order), so a call after random.seed(s)
    produces the reference's matrix for the same seed."""
    from .fileio import write_vbr_matrix
    from .vbr import VBR
    assert m % row_split == 0 and n % col_split == 0
    if partitioning == "nonuniform":
        rsz, csz = _sample_splits(m, row_split), _sample_splits(n, col_split)
    elif partitioning == "uniform":
        rsz, csz = [m // row_split] * row_split, [n // col_split] * col_split
    else:
        raise ValueError(f"partitioning {partitioning!r}: 'uniform' or 'nonuniform'")
    rpntr = np.concatenate([[0], np.cumsum(rsz)]).astype(np.int64)
    cpntr = np.concatenate([[0], np.cumsum(csz)]).astype(np.int64)
    n_blocks = row_split * col_split
    dense = random.sample(range(n_blocks), num_dense)
    dense_set = set(dense)
    sparse = random.sample([b for b in range(n_blocks) if b not in dense_set], num_sparse)
    stored = sorted(dense + sparse)
    nonzeros_in_sparse = 10
    vals, indx, bindx = [], [0], []
    bpntrb = np.full(row_split, -1, np.int64)
    bpntre = np.full(row_split, -1, np.int64)
    for k, b in enumerate(stored):
        a, c = divmod(b, col_split)
        size = int((rpntr[a + 1] - rpntr[a]) * (cpntr[c + 1] - cpntr[c]))
        n_zero = size * perc_dense_zeros // 100 if b in dense_set else size - nonzeros_in_sparse
        block = np.ones(size)
        block[random.sample(range(size), n_zero)] = 0.0
        vals.append(block)
        indx.append(indx[-1] + size)
        bindx.append(c)
        if bpntrb[a] == -1:
            bpntrb[a] = k
        bpntre[a] = k + 1
    val = np.concatenate(vals) if vals else np.zeros(0)
    matrix = VBR(val, np.asarray(indx, np.int64), np.asarray(bindx, np.int64), rpntr, cpntr, bpntrb, bpntre)
    if dense_blocks_only:
        name = f"Matrix_{m}_{n}_{row_split}_{col_split}_{num_dense}_{perc_dense_zeros}_{partitioning}"
        write_vbr_matrix(name, matrix, vbr_dir)
    else:
        name = f"Matrix_{m}_{n}_{row_split}_{col_split}_{num_dense}_{perc_dense_zeros}_{num_sparse}_{partitioning}"
        write_vbr_matrix(name, matrix, vbr_dir + "_Sparse")
    return name


def partition_case(seed: int, n_rows: int, n_cols: int, values: str = "quarters", empty_lines: bool = True,
                   explicit_zeros: bool = True):
    """A sparse matrix with hidden block structure for the partitioning steps
    (similarity cuts, VBR construction): blocks of 1..24 rows / columns, 15 %
    of them present with density U[0.3, 1], a few scattered entries, runs of
    empty rows and columns (first and last lines included) and stored zeros.
    values "quarters": multiples of 1/4 in [-2.25, 2.25] (every product and sum
    exact in FP64, so any summation order agrees); "uniform": U(-1, 1).
    Returns a canonical scipy CSR array (explicit zeros kept)."""
    import scipy.sparse
    rng = np.random.default_rng(seed)
    rs = sizes_until(rng, 1, 24, n_rows)
    cs = sizes_until(rng, 1, 24, n_cols)
    rp = np.concatenate([[0], np.cumsum(rs)])
    cp = np.concatenate([[0], np.cumsum(cs)])
    mask = np.zeros((n_rows, n_cols), dtype=bool)
    for i in range(len(rs)):
        for j in range(len(cs)):
            if rng.random() < 0.15:
                d = rng.uniform(0.3, 1.0)
                mask[rp[i]:rp[i + 1], cp[j]:cp[j + 1]] = rng.random((rs[i], cs[j])) < d
    mask |= rng.random((n_rows, n_cols)) < 0.002
    if empty_lines:
        for k in rng.choice(n_rows, size=max(1, n_rows // 40), replace=False):
            mask[k: k + int(rng.integers(1, 4)), :] = False
        for k in rng.choice(n_cols, size=max(1, n_cols // 40), replace=False):
            mask[:, k: k + int(rng.integers(1, 4))] = False
        mask[0, :] = False
        mask[:, -1] = False
    r, c = np.nonzero(mask)
    if values == "quarters":
        v = rng.integers(-9, 10, size=len(r)).astype(np.float64) / 4.0
        v[v == 0] = 0.25
    else:
        v = rng.uniform(-1.0, 1.0, size=len(r))
    if explicit_zeros and len(v):
        v[rng.random(len(v)) < 0.02] = 0.0
    A = scipy.sparse.csr_array((v, (r, c)), shape=(n_rows, n_cols))
    A.sum_duplicates()
    return A


# (seed, n_rows, n_cols, values, empty_lines) of the partition fixtures
PARTITION_CASES = [(3001, 300, 260, "quarters", True), (3002, 500, 420, "quarters", False),
                   (3003, 240, 300, "uniform", False), (3004, 160, 150, "quarters", True),
                   (3005, 700, 640, "quarters", False)]
