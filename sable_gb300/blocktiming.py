"""Device timings of the dense and the sparse form of individual blocks — the
training data of the learned block cost model.

The reference times every candidate block on the CPU, once as a dense
kernel and once as CSR (studies/threshold.py:32-86), and fits its
RandomForest to the faster label (studies/find_threshold.py:22-62).  Here
the timings come from this library's own GPU kernels.  A set of blocks is
laid out so that sample block k has block row k to itself, together with a
dense companion block of COMPANION_COLS columns in its own block column: in
a real matrix a block shares its row tile with other blocks, and a work
item's fixed cost (record copy, x loads, barriers) is shared by everything in
it, so a block's cost only means something next to other work.  The matrix is
planned twice, the sample blocks dense and the sample blocks sparse (the
companions always dense), and run with sable_spmv_timed / sable_spmm_timed,
which record the SM cycles of every work item; a block's cost in one form is
the sum over the items of its block row (median of `reps` launches).  The
companion adds the same work to both forms, so the comparison of the forms
includes what the sparse form really adds to a tile: a CSR part beside the
dense panel.  Summed cycles are additive like the kernel's total time: the
time of the items divided by the number of them that run at once.
"""
from __future__ import annotations

import numpy as np

from . import convert, synth
from .plan import Plan

SPMM_TILE = 128       # widest N-slice of the SpMM kernels
COMPANION_COLS = 64   # dense companion block beside every sample block


def diag_vbr(blocks, companion_cols: int = 0, seed: int = 0) -> synth.VbrMatrix:
    """VBR matrix with sample block k alone in block row k (block column 2k
    when companions are on, k otherwise), plus, with companion_cols > 0, a
    dense h x companion_cols block of U(-1, 1) values in block column 2k + 1."""
    nb = len(blocks)
    hs = np.array([b.shape[0] for b in blocks], dtype=np.int64)
    ws = np.array([b.shape[1] for b in blocks], dtype=np.int64)
    rpntr = np.concatenate([[0], np.cumsum(hs)]).astype(np.int64)
    if companion_cols <= 0:
        cpntr = np.concatenate([[0], np.cumsum(ws)]).astype(np.int64)
        indx = np.concatenate([[0], np.cumsum(hs * ws)]).astype(np.int64)
        val = (np.concatenate([np.asarray(b, np.float32).ravel(order="F") for b in blocks]) if nb
               else np.zeros(0, np.float32))
        ar = np.arange(nb, dtype=np.int64)
        return synth.VbrMatrix(val, indx, ar.copy(), rpntr, cpntr, ar.copy(), ar + 1)
    rng = np.random.default_rng(seed)
    widths = np.stack([ws, np.full(nb, companion_cols, np.int64)], 1).ravel()
    cpntr = np.concatenate([[0], np.cumsum(widths)]).astype(np.int64)
    sizes = np.stack([hs * ws, hs * companion_cols], 1).ravel()
    indx = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    parts = []
    for b in blocks:
        parts.append(np.asarray(b, np.float32).ravel(order="F"))
        parts.append(rng.uniform(-1, 1, b.shape[0] * companion_cols).astype(np.float32))
    val = np.concatenate(parts) if nb else np.zeros(0, np.float32)
    bindx = np.arange(2 * nb, dtype=np.int64)
    bpntrb = 2 * np.arange(nb, dtype=np.int64)
    return synth.VbrMatrix(val, indx, bindx, rpntr, cpntr, bpntrb, bpntrb + 2)


def block_stats(blocks, N: int) -> np.ndarray:
    """Feature rows (rows, cols, nnz, density, variance of nnz per row, N)."""
    out = np.zeros((len(blocks), 6), dtype=np.float32)
    for k, b in enumerate(blocks):
        rn = (b != 0).sum(axis=1)
        nnz = int(rn.sum())
        out[k] = (b.shape[0], b.shape[1], nnz, nnz / b.size, rn.var(), N)
    return out


def _slices(N: int) -> int:
    nt = 4
    while nt < N and nt < SPMM_TILE:
        nt <<= 1
    return (N + nt - 1) // nt


def _form_cycles(m: synth.VbrMatrix, dense: bool, N: int, reps: int, spmm_tc, chunk_bytes: int,
                 companions: bool, schedule: str = "items", row_tile: int = 128) -> np.ndarray:
    """Cycles of every block row (= sample block) with the samples in one form."""
    import torch
    nb = len(m.rpntr) - 1
    mask = np.full(m.n_blocks, dense, dtype=bool)
    if companions:
        mask[1::2] = True
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, mask)
    plan = Plan(comp, chunk_bytes=chunk_bytes, spmm_tc=spmm_tc, split_layout="mixed" if N == 1 else "separate",
                schedule=schedule if N == 1 else "items", row_tile=row_tile if N == 1 else 128)
    try:
        n_items = plan.stats()["n_chunks"]
        tile_of = plan.chunk_tiles()
        h = np.diff(m.rpntr)
        rt = row_tile if N == 1 else 128
        tile_block = np.repeat(np.arange(nb), (h + rt - 1) // rt)   # tiles of block row k
        item_block = tile_block[tile_of]
        rng = np.random.default_rng(nb)
        if N == 1:
            x = torch.as_tensor(rng.uniform(-1, 1, m.n_cols).astype(np.float32)).cuda()
            y = torch.empty(m.n_rows, device="cuda")
            cyc = torch.zeros(n_items, dtype=torch.int64, device="cuda")
            run = lambda: plan.spmv_timed(x, y, cyc)  # noqa: E731
        else:
            X = torch.as_tensor(rng.uniform(-1, 1, (m.n_cols, N)).astype(np.float32)).cuda()
            Y = torch.empty(m.n_rows, N, device="cuda")
            cyc = torch.zeros(_slices(N) * n_items, dtype=torch.int64, device="cuda")
            run = lambda: plan.spmm_timed(X, Y, cyc)  # noqa: E731
        run()
        torch.cuda.synchronize()
        samples = []
        for _ in range(reps):
            run()
            samples.append(cyc.view(-1, n_items).sum(0).cpu().numpy())
        plan.check()
        per_item = np.median(np.stack(samples), axis=0)
        return np.bincount(item_block, weights=per_item, minlength=nb)
    finally:
        plan.close()


# SpMV blocks are timed in the shape the autotuner picks for large matrices:
# one warp per 32 KB work item (compact records), 32-row tiles.
SPMV_SCHEDULE = "warp_items"
SPMV_ROW_TILE = 32
SPMV_CHUNK = 32768


def time_blocks(blocks, N: int, reps: int = 5, spmm_tc="split3", chunk_bytes: int = 0,
                companion_cols: int = COMPANION_COLS):
    """(dense cycles, sparse cycles) of every block in its block row (with its
    companion), float64 [n_blocks] each."""
    m = diag_vbr(blocks, companion_cols)
    c = companion_cols > 0
    if N == 1:
        kw = {"schedule": SPMV_SCHEDULE, "row_tile": SPMV_ROW_TILE}
        cb = chunk_bytes or SPMV_CHUNK
    else:
        kw, cb = {}, chunk_bytes
    return (_form_cycles(m, True, N, reps, spmm_tc, cb, c, **kw),
            _form_cycles(m, False, N, reps, spmm_tc, cb, c, **kw))


def matrix_blocks(m: synth.VbrMatrix):
    """The stored blocks of a VBR matrix as h x w arrays (bindx order)."""
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    val = np.asarray(m.val, np.float32)
    return [val[o:o + s].reshape(w, h).T for o, s, h, w in zip(bt.off, bt.size, bt.h, bt.w)]


def time_matrix_blocks(m: synth.VbrMatrix, N: int, batch: int = 10000, **kw):
    """Per-block (dense, sparse) cycles and features of a matrix's own blocks."""
    blocks = matrix_blocks(m)
    d, s, f = [], [], []
    for i in range(0, len(blocks), batch):
        part = blocks[i:i + batch]
        a, b = time_blocks(part, N, **kw)
        d.append(a)
        s.append(b)
        f.append(block_stats(part, N))
    return np.concatenate(d), np.concatenate(s), np.concatenate(f)


def timing_set(seed: int = synth.SEED_BASE + 4, count: int = 200000, batch: int = 10000, log=None, **kw):
    """Time the synthetic block set (synth.blocks_200k): features [count, 6]
    and dense / sparse cycles [count], in generator order."""
    feats = np.zeros((count, 6), dtype=np.float32)
    cd = np.zeros(count)
    cs = np.zeros(count)
    pend = {}

    def flush(N):
        idx, blks = pend.pop(N)
        a, b = time_blocks(blks, N, **kw)
        cd[idx], cs[idx] = a, b
        feats[idx] = block_stats(blks, N)
        if log:
            log(f"timed {len(blks)} blocks at N={N}")

    for k, smp in enumerate(synth.blocks_200k(seed, count)):
        ent = pend.setdefault(smp.N, ([], []))
        ent[0].append(k)
        ent[1].append(smp.block)
        if len(ent[0]) >= batch:
            flush(smp.N)
    for N in list(pend):
        flush(N)
    return feats, cd, cs
