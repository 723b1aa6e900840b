"""Multi-rank host logic on CPU (gloo, world size 2): each rank takes its
block-row shard of a VBR matrix (shard.shard_block_rows -> sub_block_rows),
builds the work-item records the library would upload for that shard
(sable_plan_layout_host, the records exactly as a plan on that rank's GPU
holds them: the per-warp compact records of the headline executor and the
standard per-CTA records), multiplies them in FP64 with the host decoder, and
the gathered row slices give the full matrix's y from the FP64 oracle.
Batch matrices are spread over ranks by cost.  The GPU path shards the same
way, one plan per rank, with no collective on the data path."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from oracle import oracle
from sable_gb300 import convert, shard, synth

from layout_decode import decode_multiply, layout


def _matrix():
    return synth.spmv_100k(seed=5, n=6000, parts=120, p=0.05)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _choice(n_blocks, seed=9):
    return np.random.default_rng(seed).random(n_blocks) < 0.5


SHAPES = ((2, 16, 32768, 0), (0, 64, 32768, 0), (0, 128, 8192, 1))   # schedule, row tile, item bytes, split layout


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = _matrix()
    x = synth.vector(m.n_cols, 3)
    a0, a1 = shard.shard_block_rows(m, world)[rank]
    sub = shard.sub_block_rows(m, a0, a1)
    # the block choice of the shard's blocks is the full matrix's choice for
    # those blocks: the blocks of block rows [a0, a1) are one contiguous run
    full = _choice(m.n_blocks)
    firsts = [int(m.bpntrb[a]) for a in range(a0, a1) if m.bpntrb[a] != -1]
    k0 = min(firsts) if firsts else 0
    dense = full[k0:k0 + sub.n_blocks]
    comp = convert.compress(sub.val, sub.rpntr, sub.cpntr, sub.indx, sub.bindx, sub.bpntrb, sub.bpntre, dense)
    ys = []
    for schedule, row_tile, chunk, split in SHAPES:
        if sub.n_rows == 0:
            ys.append(np.zeros(0))
            continue
        rec, off, byt = layout(comp, row_tile, chunk, schedule, split)
        y, cover = decode_multiply(rec, off, byt, x, sub.n_rows, compact=schedule == 2)
        assert np.all(cover == 1)
        ys.append(y)
    parts = [None] * world
    dist.all_gather_object(parts, ys)   # uneven row slices, one list per rank
    if rank == 0:
        out.put([np.concatenate([p[s] for p in parts]) for s in range(len(SHAPES))])
    dist.barrier()
    dist.destroy_process_group()


def test_block_row_shards_cover_and_balance():
    m = _matrix()
    cuts = shard.shard_block_rows(m, 4)
    assert cuts[0][0] == 0 and cuts[-1][1] == len(m.rpntr) - 1
    assert all(a1 == b0 for (_, a1), (b0, _) in zip(cuts, cuts[1:]))
    w = shard.block_row_bytes(m)
    loads = [w[a:b].sum() for a, b in cuts]
    assert max(loads) <= 1.15 * (sum(loads) / 4)


def test_shard_matrices_lpt():
    groups = shard.shard_matrices([10, 9, 8, 7, 1, 1], 2)
    assert sorted(sum(groups, [])) == list(range(6))
    loads = [sum([10, 9, 8, 7, 1, 1][i] for i in g) for g in groups]
    assert abs(loads[0] - loads[1]) <= 2


def test_two_ranks_gather_full_y():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ys = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    m = _matrix()
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, _choice(m.n_blocks))
    y_full, yabs = oracle.spmv_vbrc(comp, synth.vector(m.n_cols, 3))
    for y in ys:
        assert y.shape == y_full.shape
        assert np.all(np.abs(y - y_full) <= 1e-12 * (yabs + 1.0))
