"""Sharding of the VBR path over ranks (one process per GPU).

The path has no exchange step: y = A x splits by block rows, each rank
keeping the whole x (or the columns its blocks touch) and writing a disjoint
slice of y, and a batch splits by matrix.  So ranks share work, not data:

  shard_block_rows   contiguous block-row ranges with near-equal algorithmic
                     bytes (prefix sums of per-block-row bytes cut at k/world),
                     the contiguous counterpart of the reference's greedy
                     block-row split over threads (split_chunks,
                     src/codegen.py:165-186)
  sub_block_rows     the VBR arrays of one block-row range (rows renumbered
                     from 0, columns kept), ready for a plan on that rank
  shard_matrices     greedy LPT assignment of a batch's matrices to ranks
"""
from __future__ import annotations

import numpy as np

from . import convert, metrics, synth


def block_row_bytes(m) -> np.ndarray:
    """Algorithmic bytes of every block row (each block at its cheaper FP32 encoding)."""
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    nnz = convert.block_nnz(m.val, bt)
    per_block = np.minimum(4 * bt.size, 8 * nnz + 4 * (bt.h + 1))
    nbr = len(m.rpntr) - 1
    out = np.bincount(bt.row, weights=per_block, minlength=nbr).astype(np.float64)
    return out + 4 * np.diff(np.asarray(m.rpntr))   # y rows


def shard_block_rows(m, world: int) -> list[tuple[int, int]]:
    """[a0, a1) block-row ranges, one per rank, covering all block rows."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = block_row_bytes(m)
    c = np.concatenate([[0.0], np.cumsum(w)])
    nbr = len(w)
    cuts = [0]
    for k in range(1, world):
        cuts.append(int(np.clip(np.searchsorted(c, c[-1] * k / world), cuts[-1], nbr)))
    cuts.append(nbr)
    return [(cuts[k], cuts[k + 1]) for k in range(world)]


def sub_block_rows(m, a0: int, a1: int) -> synth.VbrMatrix:
    """Block rows [a0, a1) of a VBR matrix; row pointers rebased to 0."""
    rpntr = np.asarray(m.rpntr, np.int64)
    bpntrb = np.asarray(m.bpntrb, np.int64)
    bpntre = np.asarray(m.bpntre, np.int64)
    indx = np.asarray(m.indx, np.int64)
    rows = range(a0, a1)
    firsts = [bpntrb[a] for a in rows if bpntrb[a] != -1]
    lasts = [bpntre[a] for a in rows if bpntrb[a] != -1]
    if firsts:
        k0, k1 = int(min(firsts)), int(max(lasts))
    else:
        k0 = k1 = 0
    bindx = np.asarray(m.bindx, np.int64)[k0:k1]
    nb = np.where(bpntrb[a0:a1] == -1, -1, bpntrb[a0:a1] - k0)
    ne = np.where(bpntrb[a0:a1] == -1, -1, bpntre[a0:a1] - k0)
    v0, v1 = int(indx[k0]), int(indx[k1])
    val = np.asarray(m.val)[v0:v1]
    sub_indx = indx[k0:k1 + 1] - v0
    return synth.VbrMatrix(val, sub_indx, bindx, rpntr[a0:a1 + 1] - rpntr[a0], np.asarray(m.cpntr, np.int64),
                           nb.astype(np.int64), ne.astype(np.int64))


def shard_matrices(costs, world: int) -> list[list[int]]:
    """Greedy LPT: matrix indices per rank, largest cost first to the least-loaded rank."""
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: -float(costs[i])):
        r = min(range(world), key=lambda k: load[k])
        out[r].append(i)
        load[r] += float(costs[i])
    return [sorted(v) for v in out]


def matrix_cost(m, N: int = 1) -> int:
    """Algorithmic bytes of a matrix at width N (the batch balancing weight)."""
    return metrics.spmm_bytes(m, N) if N > 1 else metrics.spmv_bytes(m)
