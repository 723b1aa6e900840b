"""Autotuner: picks the launch shape of a matrix by timing candidates on the GPU.

For one compressed matrix and width N (1 = SpMV) it tries combinations of
  row_tile      rows per tile (tile height)
  chunk_bytes   matrix bytes per work item (tile width cut)
  executor      "items" (one CTA per work item, plus the split-tile combine
                launch), "warp_items" (one warp per work item, SpMV only) or
                "ring" (the persistent kernel of a one-matrix batch, which
                keeps `stages` records in flight per CTA)
  stages        ring depth, for the ring executor
and keeps the fastest.  Every candidate is timed with CUDA events on the
current stream, L2 flushed between runs (L2Flush), median of `reps`.
The reference fixes its shape per matrix at code-generation time (one C
function per matrix, src/codegen.py:293-452); this is the GPU counterpart of
that specialisation step.  Results are cached in memory by a signature of the
matrix structure and N.  tune_batch does the same for a batch of matrices:
it times whole batches over the SpMV matrices' executor and shape, then the
SpMM matrices' item size, then the ring depth.
"""
from __future__ import annotations

import hashlib
from dataclasses import dataclass, field

import numpy as np

from .batch import Batch
from .convert import Compressed
from .plan import Plan

SPMV_CANDIDATES = [
    {"executor": "items", "row_tile": 128, "chunk_bytes": cb} for cb in (16384, 32768, 49152)
] + [
    {"executor": "warp_items", "row_tile": rt, "chunk_bytes": cb} for rt in (8, 16, 32, 128) for cb in (8192, 16384, 32768)
] + [
    {"executor": "ring", "row_tile": 128, "chunk_bytes": cb, "stages": s} for cb in (16384, 32768) for s in (2, 3)
]
SPMM_CANDIDATES = [
    {"executor": "items", "row_tile": rt, "chunk_bytes": cb} for rt in (128, 64) for cb in (16384, 32768, 49152, 65536)
] + [
    # items above the shared-memory staging size: SpMM-only plans, long K loops, no split tiles
    {"executor": "items", "row_tile": 128, "chunk_bytes": cb} for cb in (131072, 262144)
] + [{"executor": "ring", "row_tile": 128, "chunk_bytes": 32768, "stages": 2}]

_cache: dict[str, dict] = {}


def signature(comp: Compressed, N: int, spmm_tc) -> str:
    h = hashlib.sha256()
    for a in (comp.rpntr, comp.cpntr, comp.bpntrb, comp.bindx, comp.ublocks):
        h.update(np.ascontiguousarray(a, dtype=np.int64).tobytes())
    h.update(np.int64(0 if comp.indptr is None else comp.indptr[-1]).tobytes())
    h.update(f"{N}/{spmm_tc}".encode())
    return h.hexdigest()


@dataclass
class Tuned:
    """A plan (and, for the ring executor, its one-matrix batch) in the chosen shape."""
    config: dict
    plan: Plan
    batch: Batch | None = None
    N: int = 1
    table: list = field(default_factory=list)

    def run(self, x, y, stream=None):
        if self.batch is not None:
            return self.batch.run([x], [y], stream)
        return self.plan.spmv(x, y, stream) if self.N == 1 else self.plan.spmm(x, y, stream)

    def launches_per_run(self) -> int:
        """Kernels of this library per run (work items, plus the combine of
        split tiles for the per-CTA executors; the per-warp kernel combines
        them itself)."""
        splits = self.plan.stats()["scratch_floats"] > 0
        extra = splits and self.N == 1 and self.config["executor"] != "warp_items"
        return 1 + (1 if extra else 0)

    def close(self):
        if self.batch is not None:
            self.batch.close()
        self.plan.close()


def _build(comp: Compressed, cfg: dict, N: int, spmm_tc) -> Tuned:
    plan = Plan(comp, row_tile=cfg["row_tile"], chunk_bytes=cfg["chunk_bytes"], spmm_tc=spmm_tc,
                split_layout="mixed" if N == 1 else "separate",
                schedule="warp_items" if cfg["executor"] == "warp_items" else "items")
    batch = None
    if cfg["executor"] == "ring":
        batch = Batch([plan], [N], use_graph=True, stages=cfg.get("stages", 0))
    return Tuned(dict(cfg), plan, batch, N)


class L2Flush:
    """Between timed runs: write a 256 MB buffer (evicts everything of the run
    before), then read a clean 256 MB buffer, so the run starts with L2 holding
    neither its own data nor dirty lines whose write-back it would pay for."""

    def __init__(self):
        import torch
        self.w = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        self.r = torch.ones(64 << 20, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.w.fill_(1)
        self.r.sum()


_flush = None


def l2_flush():
    global _flush
    if _flush is None:
        _flush = L2Flush()
    _flush()


def time_ms(fn, reps: int = 10, warmup: int = 3) -> float:
    import torch
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(reps):
        l2_flush()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        ts.append(s.elapsed_time(e))
    return float(np.median(ts))


def tune(comp: Compressed, x, y, N: int = 1, spmm_tc="split3", candidates=None, reps: int = 10,
         use_cache: bool = True) -> Tuned:
    """Time every candidate on (x, y) and return the fastest, built."""
    key = signature(comp, N, spmm_tc)
    if use_cache and key in _cache:
        return _build(comp, _cache[key], N, spmm_tc)
    cands = candidates or (SPMV_CANDIDATES if N == 1 else SPMM_CANDIDATES)
    table, best, best_ms = [], None, float("inf")
    for cfg in cands:
        try:
            t = _build(comp, cfg, N, spmm_tc)
        except Exception as ex:  # a shape the device cannot hold (shared memory): skip it
            table.append({**cfg, "ms": None, "error": str(ex)[:80]})
            continue
        ms = time_ms(lambda: t.run(x, y), reps)
        t.plan.check()
        if t.batch is not None:
            t.batch.check()
        table.append({**cfg, "ms": round(ms, 5)})
        if ms < best_ms:
            if best is not None:
                best.close()
            best, best_ms = t, ms
        else:
            t.close()
    if best is None:
        raise RuntimeError("no autotuner candidate could be built")
    best.table = table
    _cache[key] = best.config
    return best


# Batch shapes per matrix class: the SpMV matrices' executor (per-warp kernel
# on compact records, or the batch's ring of per-CTA items) and the SpMM
# matrices' work-item size (whole block rows for the tcgen05 kernel, or
# smaller items); the ring depth only matters when ring units remain.
BATCH_SPMV_SHAPES = [
    {"executor": "warp_items", "row_tile": 16, "chunk_bytes": 32768},
    {"executor": "warp_items", "row_tile": 16, "chunk_bytes": 16384},
    {"executor": "ring", "row_tile": 128, "chunk_bytes": 32768},
]
BATCH_SPMM_SHAPES = [
    {"executor": "items", "row_tile": 128, "chunk_bytes": 262144},
    {"executor": "items", "row_tile": 128, "chunk_bytes": 131072},
    {"executor": "items", "row_tile": 128, "chunk_bytes": 32768},
]


def _batch_plan(comp: Compressed, shape: dict, N: int, spmm_tc) -> Plan:
    return Plan(comp, row_tile=shape["row_tile"], chunk_bytes=shape["chunk_bytes"],
                spmm_tc=spmm_tc if N > 1 else "off", split_layout="mixed" if N == 1 else "separate",
                schedule="warp_items" if shape["executor"] == "warp_items" else "items")


def tune_batch(comps, widths, xs, ys, spmm_tc="split3", stages=(2, 4), reps: int = 10) -> tuple[Batch, list]:
    """Pick a batch's shape by timing it whole (CUDA graph on): the SpMV
    matrices' executor and item shape, then the SpMM matrices' item size,
    then the ring depth when ring units remain (one class at a time, the
    others held at their best so far).  Returns (batch, table); the batch
    owns copies of the records, its plans are closed."""
    widths = [int(w) for w in widths]
    spmv = [i for i, w in enumerate(widths) if w == 1]
    spmm = [i for i, w in enumerate(widths) if w > 1]
    plan_cache: dict = {}

    def plans_for(idx, shape):
        key = (tuple(idx), tuple(sorted(shape.items())))
        if key not in plan_cache:
            plan_cache[key] = [_batch_plan(comps[i], shape, widths[i], spmm_tc) for i in idx]
        return plan_cache[key]

    table, best, best_ms, best_cfg = [], None, float("inf"), None

    def trial(sv, sm, st):
        nonlocal best, best_ms, best_cfg
        cfg = {"spmv": sv, "spmm": sm, "stages": st}
        plans = [None] * len(widths)
        if spmv:
            for i, p in zip(spmv, plans_for(spmv, sv)):
                plans[i] = p
        if spmm:
            for i, p in zip(spmm, plans_for(spmm, sm)):
                plans[i] = p
        try:
            b = Batch(plans, widths, use_graph=True, stages=st)
        except Exception as ex:
            table.append({**cfg, "ms": None, "error": str(ex)[:80]})
            return
        ms = time_ms(lambda: b.run(xs, ys), reps)
        b.check()
        table.append({**cfg, "ms": round(ms, 5), "n_ctas": b.info()["n_ctas"]})
        if ms < best_ms:
            if best is not None:
                best.close()
            best, best_ms, best_cfg = b, ms, cfg
        else:
            b.close()

    sv0, sm0 = BATCH_SPMV_SHAPES[0], BATCH_SPMM_SHAPES[0]
    for sv in (BATCH_SPMV_SHAPES if spmv else [sv0]):
        trial(sv, sm0, 0)
    sv_best = best_cfg["spmv"] if best_cfg else sv0
    for sm in (BATCH_SPMM_SHAPES[1:] if spmm else []):
        trial(sv_best, sm, 0)
    if best_cfg is not None and best.info()["n_units"] > 0 and (best_cfg["spmv"]["executor"] == "ring" or any(
            widths[i] < 32 for i in spmm)):
        for st in stages:
            trial(best_cfg["spmv"], best_cfg["spmm"], st)
    for ps in plan_cache.values():
        for p in ps:
            p.close()
    if best is None:
        raise RuntimeError("no batch shape could be built")
    return best, table
