"""Device timings of the dense and the sparse form of individual blocks — the
training data of the learned block cost model.

The reference times every candidate block on the CPU, once as a dense
kernel and once as CSR (studies/threshold.py:32-86), and fits its
RandomForest to the faster label (studies/find_threshold.py:22-62).  Here
the timings come from this library's own GPU kernels: a set of blocks is laid
out as a block-diagonal VBR matrix (block k alone in block row k and block
column k), so every work item of a plan belongs to exactly one block.  The
matrix is planned twice, all blocks dense and all blocks sparse, and run with
sable_spmv_timed / sable_spmm_timed, which record the SM cycles of every work
item; a block's cost in one form is the sum over its items (median of
`reps` launches).  Summed cycles are additive in the same way as the
kernel's total time: it is the time of the items divided by the number of
them that run at once.
"""
from __future__ import annotations

import numpy as np

from . import convert, synth
from .plan import Plan

SPMM_TILE = 128  # widest N-slice of the SpMM kernels


def diag_vbr(blocks) -> synth.VbrMatrix:
    """Block-diagonal VBR matrix of the given dense h x w float32 blocks."""
    hs = np.array([b.shape[0] for b in blocks], dtype=np.int64)
    ws = np.array([b.shape[1] for b in blocks], dtype=np.int64)
    nb = len(blocks)
    rpntr = np.concatenate([[0], np.cumsum(hs)]).astype(np.int64)
    cpntr = np.concatenate([[0], np.cumsum(ws)]).astype(np.int64)
    indx = np.concatenate([[0], np.cumsum(hs * ws)]).astype(np.int64)
    val = np.concatenate([np.asarray(b, np.float32).ravel(order="F") for b in blocks]) if nb else np.zeros(0, np.float32)
    ar = np.arange(nb, dtype=np.int64)
    return synth.VbrMatrix(val, indx, ar.copy(), rpntr, cpntr, ar.copy(), ar + 1)


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


def _form_cycles(m: synth.VbrMatrix, dense: bool, N: int, reps: int, spmm_tc, chunk_bytes: int) -> np.ndarray:
    import torch
    nb = m.n_blocks
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre,
                            np.full(nb, dense, dtype=bool))
    plan = Plan(comp, chunk_bytes=chunk_bytes, spmm_tc=spmm_tc)
    try:
        n_items = plan.stats()["n_chunks"]
        tile_of = plan.chunk_tiles()
        h = np.diff(m.rpntr)
        tile_block = np.repeat(np.arange(nb), (h + 127) // 128)   # tiles of block row k (row tile 128)
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


def time_blocks(blocks, N: int, reps: int = 5, spmm_tc="split3", chunk_bytes: int = 0):
    """(dense cycles, sparse cycles) of every block, float64 [n_blocks] each."""
    m = diag_vbr(blocks)
    return (_form_cycles(m, True, N, reps, spmm_tc, chunk_bytes),
            _form_cycles(m, False, N, reps, spmm_tc, chunk_bytes))


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
