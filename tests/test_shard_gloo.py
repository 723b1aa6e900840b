"""Multi-rank host logic on CPU (gloo, world size 2): block-row shards of a
VBR matrix computed by separate ranks and gathered give the full y; batch
matrices are spread over ranks by cost.  The GPU path shards the same way,
one plan per rank, with no collective on the data path."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from oracle import oracle
from sable_gb300 import convert, shard, synth


def _matrix():
    return synth.spmv_100k(seed=5, n=6000, parts=120, p=0.05)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = _matrix()
    x = synth.vector(m.n_cols, 3)
    a0, a1 = shard.shard_block_rows(m, world)[rank]
    sub = shard.sub_block_rows(m, a0, a1)
    dense = np.ones(sub.n_blocks, bool)
    comp = convert.compress(sub.val.astype(np.float64), sub.rpntr, sub.cpntr, sub.indx, sub.bindx, sub.bpntrb,
                            sub.bpntre, dense, value_dtype=np.float64)
    y, _ = oracle.spmv_vbrc(comp, x) if sub.n_rows else (np.zeros(0), None)
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(y))   # uneven row slices
    if rank == 0:
        out.put(np.concatenate(parts))
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
    y = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    m = _matrix()
    comp = convert.compress(m.val.astype(np.float64), m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre,
                            np.ones(m.n_blocks, bool), value_dtype=np.float64)
    y_full, _ = oracle.spmv_vbrc(comp, synth.vector(m.n_cols, 3))
    np.testing.assert_allclose(y, y_full, rtol=0, atol=1e-12)
