"""Reference-named inspector / executor entry points (reference: src/codegen.py).

In the reference each *_codegen function writes one C (or CUDA) program for
one matrix, which is compiled and run as a separate process.  Here the same
functions build a GPU plan (libsable) instead, keep it in an in-process
registry keyed by (dir_name, filename), write a small manifest
<dir_name>/<filename>.sable.json, and return the inspector time in the
reference's unit (ms for SpMV, us for SpMM).  run_spmv / run_spmm play the
part of running the generated program: they read the dense operand from the
reference's Generated_dense_tensors files (unless one is passed), run
bench + 1 iterations, drop the first, and return the per-iteration device
times (ns) and the result.

  vbr_spmv_codegen          src/codegen.py:1438-1447
  gen_single_threaded_spmv  src/codegen.py:293-452
  gen_multi_threaded_spmv   src/codegen.py:454-643 (threads only recorded:
                            GPU parallelism replaces the OpenMP split)
  vbr_spmm_codegen          src/codegen.py:1449-1458
  gen_single_threaded_spmm  src/codegen.py:827-937
  gen_multi_threaded_spmm   src/codegen.py:939-1075
  vbr_spmv_cuda_codegen     src/codegen.py:1077-1195 (density rule
                            dense_count > density*(h*w)//100, :1158)
  vbr_spmm_cuda_codegen     src/codegen.py:1312-1436
  only_nonzeros_spmv        src/baseline.py:10-93 (the per-nonzero baseline:
  only_nonzeros_spmm        src/baseline.py:94-182  every block CSR)
"""
from __future__ import annotations

import json
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import fileio
from .convert import Compressed, block_nnz, block_table, compress
from .plan import Plan

# Launch shapes the entry points use unless plan options say otherwise: the
# fastest shapes measured on large matrices (one warp per 32 KB work item over
# 16-row tiles for SpMV; one CTA per work item of up to 256 KB, whole block
# rows, with separate dense and CSR items for SpMM: an SpMM-only plan).
# sable_gb300.autotune picks per matrix.
SPMV_SHAPE = {"schedule": "warp_items", "row_tile": 16, "chunk_bytes": 32768}
SPMM_SHAPE = {"split_layout": "separate", "row_tile": 128, "chunk_bytes": 262144}


def _with(defaults: dict, opts: dict) -> dict:
    return {**defaults, **opts}

PLANS: dict = {}


@dataclass
class PlanRecord:
    plan: Plan
    kind: str          # "spmv" or "spmm"
    n_rows: int
    n_cols: int
    bench: int = 5
    info: dict = field(default_factory=dict)


def _key(dir_name: str, filename: str):
    return (os.path.abspath(dir_name), filename)


def _register(dir_name, filename, rec: PlanRecord):
    os.makedirs(dir_name, exist_ok=True)
    old = PLANS.pop(_key(dir_name, filename), None)
    if old is not None:
        old.plan.close()
    PLANS[_key(dir_name, filename)] = rec
    man = {"kind": rec.kind, "n_rows": rec.n_rows, "n_cols": rec.n_cols, "bench": rec.bench,
           "stats": rec.plan.stats(), **rec.info}
    with open(os.path.join(dir_name, filename + ".sable.json"), "w") as f:
        json.dump(man, f, indent=1, default=int)


def load_plan(dir_name: str, filename: str) -> PlanRecord:
    try:
        return PLANS[_key(dir_name, filename)]
    except KeyError:
        raise KeyError(f"no plan for {filename} in {dir_name}: run its *_codegen first") from None


def _compressed_from_vbrc(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks, indptr, indices, csr_val):
    has_csr = indptr is not None and len(indptr) > 0
    return Compressed(
        val=np.asarray(val, dtype=np.float32), indx=np.asarray(indx, dtype=np.int64),
        bindx=np.asarray(bindx, dtype=np.int64), rpntr=np.asarray(rpntr, dtype=np.int64),
        cpntr=np.asarray(cpntr, dtype=np.int64), bpntrb=np.asarray(bpntrb, dtype=np.int64),
        bpntre=np.asarray(bpntre, dtype=np.int64), ublocks=np.asarray(ublocks, dtype=np.int64),
        indptr=np.asarray(indptr, dtype=np.int64) if has_csr else None,
        indices=np.asarray(indices, dtype=np.int64) if has_csr else None,
        csr_val=np.asarray(csr_val, dtype=np.float32) if has_csr else None)


# -- SpMV -----------------------------------------------------------------------
def gen_single_threaded_spmv(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks, indptr, indices, csr_val,
                             dir_name, filename, vbr_dir, bench: int = 5, **plan_opts) -> int:
    t1 = time.time_ns() // 1_000_000
    comp = _compressed_from_vbrc(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks, indptr, indices, csr_val)
    plan = Plan(comp, **_with(SPMV_SHAPE, plan_opts))
    _register(dir_name, filename, PlanRecord(plan, "spmv", comp.n_rows, comp.n_cols, bench,
                                             {"vbr_dir": os.path.abspath(vbr_dir), "threads": 1}))
    return time.time_ns() // 1_000_000 - t1


def gen_multi_threaded_spmv(threads, val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks, indptr, indices,
                            csr_val, dir_name: str, filename: str, vbr_dir: str, bench: int = 5, **plan_opts) -> int:
    ms = gen_single_threaded_spmv(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks, indptr, indices, csr_val,
                                  dir_name, filename, vbr_dir, bench, **plan_opts)
    PLANS[_key(dir_name, filename)].info["threads"] = int(threads)
    return ms


def vbr_spmv_codegen(filename: str, dir_name: str, vbr_dir: str, threads: int, bench: int = 5, **plan_opts) -> int:
    arrays = fileio.read_vbrc(fileio.source_path(vbr_dir, filename, ".vbrc"))
    t1 = time.time_ns() // 1_000_000
    if threads == 1:
        gen_single_threaded_spmv(*arrays, dir_name, filename, vbr_dir, bench, **plan_opts)
    else:
        gen_multi_threaded_spmv(threads, *arrays, dir_name, filename, vbr_dir, bench, **plan_opts)
    return time.time_ns() // 1_000_000 - t1


def _time_iterations(fn, iters: int) -> list[int]:
    import torch
    times = []
    for _ in range(iters):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        times.append(int(round(s.elapsed_time(e) * 1e6)))
    return times


def run_spmv(dir_name: str, filename: str, x=None):
    """Execute a registered SpMV plan like the generated program: returns
    (per-iteration ns for `bench` iterations after one dropped, y)."""
    import torch
    rec = load_plan(dir_name, filename)
    if x is None:
        x = fileio.read_dense_values(os.path.join(fileio.base_path(), "Generated_dense_tensors",
                                                  f"generated_vector_{rec.n_cols}.vector"))[: rec.n_cols]
    xd = torch.as_tensor(np.asarray(x, dtype=np.float32)).cuda()
    yd = torch.empty(rec.n_rows, dtype=torch.float32, device="cuda")
    times = _time_iterations(lambda: rec.plan.spmv(xd, yd), rec.bench + 1)[1:]
    return times, yd.cpu().numpy()


def spmv(plan: Plan, x):
    return plan.spmv(x)


# -- SpMM -----------------------------------------------------------------------
def _density_mask(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density: int, integer_rule: bool = False):
    bt = block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx)
    if density is None or density <= 0:
        return bt, np.ones(len(bt.off), dtype=bool)
    nnz = block_nnz(val, bt)
    if integer_rule:  # dense_count > (density * (h*w)) // 100   (src/codegen.py:1158, 1395)
        return bt, nnz > (int(density) * bt.size) // 100
    return bt, (nnz / bt.size) * 100 > density  # (src/codegen.py:917)


def gen_single_threaded_spmm(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density: int, dir_name: str,
                             filename: str, vbr_dir: str, spmm_tc="split3", **plan_opts) -> PlanRecord:
    bt, dense = _density_mask(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density)
    comp = compress(np.asarray(val, dtype=np.float32), rpntr, cpntr, indx, bindx, bpntrb, bpntre, dense, bt=bt)
    plan = Plan(comp, spmm_tc=spmm_tc, **_with(SPMM_SHAPE, plan_opts))
    rec = PlanRecord(plan, "spmm", comp.n_rows, comp.n_cols, 1,
                     {"vbr_dir": os.path.abspath(vbr_dir), "density": density, "threads": 1, "spmm_tc": plan.spmm_tc})
    _register(dir_name, filename, rec)
    return rec


def gen_multi_threaded_spmm(threads, val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density: int, dir_name: str,
                            filename: str, vbr_dir: str, **plan_opts) -> PlanRecord:
    rec = gen_single_threaded_spmm(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density, dir_name, filename,
                                   vbr_dir, **plan_opts)
    rec.info["threads"] = int(threads)
    return rec


def vbr_spmm_codegen(filename: str, density: int, dir_name: str, vbr_dir: str, threads: int, **plan_opts) -> int:
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(fileio.source_path(vbr_dir, filename, ".vbr"))
    t1 = time.time_ns() // 1_000
    if threads == 1:
        gen_single_threaded_spmm(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density, dir_name, filename, vbr_dir,
                                 **plan_opts)
    else:
        gen_multi_threaded_spmm(threads, val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density, dir_name, filename,
                                vbr_dir, **plan_opts)
    return time.time_ns() // 1_000 - t1


def run_spmm(dir_name: str, filename: str, X=None, N: int = 512):
    """Execute a registered SpMM plan; X defaults to the reference's
    generated_matrix_{n}x512.matrix file (row-major, width N)."""
    import torch
    rec = load_plan(dir_name, filename)
    if X is None:
        X = fileio.read_dense_values(os.path.join(fileio.base_path(), "Generated_dense_tensors",
                                                  f"generated_matrix_{rec.n_cols}x{N}.matrix")).reshape(rec.n_cols, N)
    Xd = torch.as_tensor(np.ascontiguousarray(X, dtype=np.float32)).cuda()
    Yd = torch.empty(rec.n_rows, Xd.shape[1], dtype=torch.float32, device="cuda")
    times = _time_iterations(lambda: rec.plan.spmm(Xd, Yd), rec.bench + 1)[1:]
    return times, Yd.cpu().numpy()


def spmm(plan: Plan, X):
    return plan.spmm(X)


# -- the reference's CUDA generators (unreachable there: read_vbr is not imported) --
def vbr_spmv_cuda_codegen(filename: str, dir_name: str, vbr_dir: str, density: int, **plan_opts) -> int:
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(fileio.source_path(vbr_dir, filename, ".vbr"))
    t1 = time.time_ns() // 1_000
    bt, dense = _density_mask(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density, integer_rule=True)
    comp = compress(np.asarray(val, dtype=np.float32), rpntr, cpntr, indx, bindx, bpntrb, bpntre, dense, bt=bt)
    _register(dir_name, filename, PlanRecord(Plan(comp, **_with(SPMV_SHAPE, plan_opts)), "spmv", comp.n_rows, comp.n_cols, 0,
                                             {"density": density}))
    return time.time_ns() // 1_000 - t1


def vbr_spmm_cuda_codegen(filename: str, dir_name: str, vbr_dir: str, density: int, spmm_tc="split3",
                          **plan_opts) -> int:
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(fileio.source_path(vbr_dir, filename, ".vbr"))
    t1 = time.time_ns() // 1_000
    bt, dense = _density_mask(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre, density, integer_rule=True)
    comp = compress(np.asarray(val, dtype=np.float32), rpntr, cpntr, indx, bindx, bpntrb, bpntre, dense, bt=bt)
    _register(dir_name, filename, PlanRecord(Plan(comp, spmm_tc=spmm_tc, **_with(SPMM_SHAPE, plan_opts)), "spmm",
                                             comp.n_rows,
                                             comp.n_cols, 0, {"density": density}))
    return time.time_ns() // 1_000 - t1


# -- the reference's per-nonzero baselines (src/baseline.py) --------------------
def _nonzeros_only(vbr_dir: str, filename: str):
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(fileio.source_path(vbr_dir, filename, ".vbr"))
    return compress(np.asarray(val, dtype=np.float32), rpntr, cpntr, indx, bindx, bpntrb, bpntre,
                    np.zeros(len(bindx), dtype=bool))


def only_nonzeros_spmv(filename: str, dir_name: str, vbr_dir: str, bench: int = 5, **plan_opts) -> None:
    """src/baseline.py:10-93: SpMV that touches every stored nonzero once and
    no zero (the reference emits one FP32 statement per nonzero).  Here a plan
    with every block in CSR form (the all-sparse choice) is registered as
    (dir_name, filename); run_spmv executes it."""
    comp = _nonzeros_only(vbr_dir, filename)
    _register(dir_name, filename, PlanRecord(Plan(comp, **_with(SPMV_SHAPE, plan_opts)), "spmv", comp.n_rows,
                                             comp.n_cols, bench, {"vbr_dir": os.path.abspath(vbr_dir),
                                                                  "baseline": "only_nonzeros"}))


def only_nonzeros_spmm(filename: str, dir_name: str, vbr_dir: str, bench: int = 5, **plan_opts) -> None:
    """src/baseline.py:94-182: the SpMM counterpart (FP32, every block CSR),
    registered for run_spmm."""
    comp = _nonzeros_only(vbr_dir, filename)
    _register(dir_name, filename, PlanRecord(Plan(comp, **_with(SPMM_SHAPE, plan_opts)), "spmm", comp.n_rows,
                                             comp.n_cols, bench, {"vbr_dir": os.path.abspath(vbr_dir),
                                                                  "baseline": "only_nonzeros"}))
