#!/usr/bin/env python
"""Benchmark: VBR SpMV GB/s (headline), SpMM GFLOP/s and the mixed batch,
learned+batched forms against the plain FP32 form, on one GB300.

Headline step = one SpMV y = A x over the 100000 x 100000 workload (~2e4
blocks of 10..100 rows/cols, ~5e7 stored values), x and A resident in HBM.
Forms:
  plain     the reference's block choice (its RandomForest threshold), plan
            defaults (one CTA per 32 KB work item)
  learned   the MLP cost model's block choice, launch shape picked by the
            autotuner (tile height, work-item size, executor, ring depth)
`value` = algorithmic bytes of the matrix (each block at its cheaper FP32
encoding, plus x and y; sable_gb300.metrics) / time of the learned step,
timed with CUDA events on the launching stream, L2 flushed between steps
outside the events (a 256 MB write, then a 256 MB read of a clean buffer, so
that the step neither finds its data in L2 nor pays for writing back the
flush's dirty lines).  `e2e` runs the same learned plan through
the C ABI with host buffers (sable_spmv_host: pinned x copied in, y copied
out, inside the timed region).  Also reported, each timed the same way:
  spmm_50k   50000 x 50000, N = 32 and 128: plain = reference choice, FP32
             CUDA cores; learned = MLP choice, split-BF16 tensor cores
             (three terms, six products), autotuned; error vs FP64 (scipy
             on the host) over a row sample
  batch_256  256 matrices (half SpMV, half SpMM N = 64): plain = reference
             choice, one launch per matrix, FP32; learned+batched = MLP
             choice, one persistent-kernel graph launch
`--impl reference` times the reference's CPU executor on the headline
workload: its own generated C (oracle/refc.py: gen_multi_threaded_spmv,
FP64, OpenMP over the host cores, its compiler flags; a few minutes of
compilation the first time on a host), or, where those sources were not
generated, the oracle's C port of it; its spmm_50k section times the
reference's own generated SpMM (gen_multi_threaded_spmm, density 0 as its
benchmark, FP32, pthreads) at N = 32 and 128, compiled in the same pool.
The GPU arm's cpu_baseline reports the same SpMV program when it is already
compiled on the host, else the port, for the same number of iterations; its
SpMM cpu_baselines run the reference's generated SpMM (the median of four
runs; compiled at start-up, before any GPU work, where the reference arm has
not compiled it, about a minute).  Under torchrun each rank runs its own seeded
replica (weak scaling, no collective on the data path); with --strong the
ranks instead take block-row shards of the one matrix, balanced by algorithmic
bytes (sable_gb300.shard), each writing its own rows of y (strong scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "VBR SpMV GB/s & SpMM GFLOP/s, % roofline: learned+batched vs plain, 1 GB300"
WORKLOAD = ("spmv_100k: 100000x100000 VBR, 2000x2000 partitions U[10,100], block p=0.005, "
            "density 1.0 w.p. 0.4 else U[0.05,0.5] (uniform / row-clustered), FP32 U(-1,1)")


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi"]}
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def choices(m, bt, N: int):
    """(features, reference RandomForest choice, MLP choice) of a matrix at width N."""
    from sable_gb300 import blockmodel, convert
    feats = convert.block_features(m.val, bt, N)
    rf = blockmodel.RFTableModel().choose_dense(feats)
    return feats, rf, blockmodel.MLPModel.load().choose_dense(feats)


def build_workload(rank: int):
    from sable_gb300 import convert, metrics, synth
    m = synth.spmv_100k(seed=synth.SEED_BASE + 1 + 100 * rank)
    x = synth.vector(m.n_cols, seed=31 + rank)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    nnz = convert.block_nnz(m.val, bt)
    B = metrics.spmv_matrix_bytes(bt, nnz) + 4 * (m.n_rows + m.n_cols)
    return m, x, bt, nnz, B


def time_device(fn, steps: int, warmup: int, world: int, flush):
    """Per-step CUDA-event durations (ms) on the current stream; L2 flushed
    between steps outside the events."""
    import torch
    for _ in range(warmup):
        flush()
        fn()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    evs = []
    for _ in range(steps):
        flush()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        evs.append((s, e))
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in evs]


def bench_spmm(reps: int, flush, cpu: bool = True) -> dict:
    """50000^2 SpMM at N = 32 and 128: plain FP32 vs learned split-BF16 (autotuned)."""
    import torch
    from sable_gb300 import autotune, convert, metrics, synth
    from sable_gb300.plan import Plan
    m = synth.spmm_50k()
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    nnz = int(convert.block_nnz(m.val, bt).sum())
    out = {"workload": "spmm_50k: 50000x50000, 1000x1000 partitions in [20,80], block p=0.01, 60% dense blocks, "
                       "rest density U[0.05,0.3], B 50000xN U(-1,1)", "nnz": nnz}
    A64 = None
    for N in (32, 128):
        _, rf, mlp = choices(m, bt, N)
        X = torch.as_tensor(synth.dense_operand(m.n_cols, N, 7)).cuda()
        Y = torch.empty(m.n_rows, N, device="cuda")
        comp_p = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, rf, bt=bt)
        plain = Plan(comp_p, split_layout="separate")
        ms_p = autotune.time_ms(lambda: plain.spmm(X, Y), reps)
        comp_l = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, mlp, bt=bt)
        tuned = autotune.tune(comp_l, X, Y, N=N, spmm_tc="split3")
        ms_l = autotune.time_ms(lambda: tuned.run(X, Y), reps)
        tuned.run(X, Y)
        Yl = Y.cpu().numpy().astype(np.float64)
        # error against FP64 on the host (scipy CSR of A), 4000 sampled rows
        if A64 is None:
            A64 = csr64(m, bt)
        rel = sampled_error(A64, Yl, X.cpu().numpy())
        F = metrics.spmm_flops(m, N)
        # roofline of the learned form: the larger of its algorithmic bytes at
        # the measured HBM peak and its useful flops at the measured BF16
        # tensor peak shared by the six split products
        pk = peaks()
        Bm = metrics.spmm_bytes(m, N)
        t_mem = Bm / (pk["hbm_gbs"] * 1e9)
        t_tc = F / ((pk["bf16_tflops"] or 1900.0) * 1e12 / 6)
        roof = {"bound": "hbm" if t_mem >= t_tc else "tensor", "bytes": int(Bm),
                "time_bound_us": round(max(t_mem, t_tc) * 1e6, 2),
                "frac": round(max(t_mem, t_tc) / (ms_l * 1e-3), 4),
                "achieved_gbs": round(Bm / (ms_l * 1e-3) / 1e9, 1), "peak_gbs": pk["hbm_gbs"],
                "peak_bf16_tflops": pk["bf16_tflops"], "products_per_flop": 6}
        out[f"N{N}"] = {
            "plain_fp32_gflops": round(F / (ms_p * 1e-3) / 1e9, 1), "plain_ms": round(ms_p, 4),
            "learned_tc_gflops": round(F / (ms_l * 1e-3) / 1e9, 1), "learned_ms": round(ms_l, 4),
            "learned_vs_plain": round(ms_p / ms_l, 3), "learned_config": tuned.config, "roofline": roof,
            "error_vs_fp64_scaled": {"max": float(rel.max()), "median": float(np.median(rel)), "rows": 4000,
                                     "precision": "split-BF16, three terms (hi+mid+lo), six products, FP32 accum"},
            "dense_frac_learned": round(float(mlp.mean()), 3), "dense_frac_plain": round(float(rf.mean()), 3)}
        if cpu:
            out[f"N{N}"]["cpu_baseline"] = cpu_spmm_baseline(m, X.cpu().numpy(), F, A64)
        plain.close()
        tuned.close()
    return out


def csr64(m, bt):
    """A as an FP64 scipy CSR (for the sampled-row error checks)."""
    import scipy.sparse
    rows, cols, vals = [], [], []
    for k in range(len(bt.off)):
        blk = np.asarray(m.val[bt.off[k]: bt.off[k] + bt.size[k]], np.float64).reshape(bt.w[k], bt.h[k]).T
        r, c = np.nonzero(blk)
        rows.append(r + bt.r0[k])
        cols.append(c + bt.c0[k])
        vals.append(blk[r, c])
    return scipy.sparse.csr_array((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                  shape=(m.n_rows, m.n_cols))


def sampled_error(A64, Y, Xh, rows: int = 4000) -> np.ndarray:
    """|Y - A X| / (|A||X|) in FP64 over `rows` seeded sampled rows."""
    sel = np.random.default_rng(5).choice(A64.shape[0], rows, replace=False)
    Xh = np.asarray(Xh, np.float64)
    ref = A64[sel] @ Xh
    scale = np.abs(A64[sel]) @ np.abs(Xh)
    return np.abs(np.asarray(Y, np.float64)[sel] - ref) / np.maximum(scale, 1e-300)


def compile_reference_spmm() -> None:
    """Compile the reference's generated SpMM programs that are present and
    not yet compiled on this host (both widths in one pool, about a minute),
    so that no compilation runs right before a timed CPU baseline (a run
    straight after the compilation measured up to 4x slower)."""
    from oracle import refc
    widths = [w for w in refc.SPMM_WIDTHS if refc.spmm_generated(w) and not refc.spmm_compiled(w)]
    if widths:
        refc.compile((), spmm_widths=widths)


def reference_spmm(N: int, F: float, A64, Xh, runs: int = 4):
    """The reference's own generated multi-threaded SpMM at width N
    (oracle/refc.py: gen_multi_threaded_spmm with density 0, as its own
    benchmark runs it; FP32, its CFLAGS for this host; compiled first where
    needed), or None where its sources were not generated.  The median of
    `runs` timed runs after one dropped cold run."""
    from oracle import refc
    if not refc.spmm_generated(N):
        return None
    if not refc.spmm_compiled(N):
        refc.compile((), spmm_widths=[w for w in refc.SPMM_WIDTHS if refc.spmm_generated(w)])
    r = refc.run_spmm(N, runs + 1)
    t = np.asarray(r["times_ns"][1:], np.float64) * 1e-9
    ms = float(np.median(t)) * 1e3
    rel = sampled_error(A64, r["Y"], Xh)
    return {"value": round(F / (ms * 1e-3) / 1e9, 1), "unit": "GFLOP/s", "ms": round(ms, 3),
            "cores": int(r["threads"]), "kind": "reference",
            "sample": f"full matrix, width {N}, median of {len(t)} timed runs after one dropped cold run of the reference's "
                      f"own generated multi-threaded SpMM (gen_multi_threaded_spmm, density 0 as its benchmark, "
                      f"{r['threads']} pthreads, FP32, its CFLAGS); max error vs FP64 {float(rel.max()):.1e} of "
                      f"|A||X| over 4000 sampled rows"}


def cpu_spmm_baseline(m, Xh, F, A64) -> dict:
    """The reference's own generated SpMM (reference_spmm) where its sources
    were generated, else the oracle's C port of it (gen_multi_threaded_spmm:
    FP32, i-j-k loops per dense block, block rows split over the host cores
    by LPT), its compiler flags, the full matrix."""
    ref = reference_spmm(Xh.shape[1], F, A64, Xh)
    if ref is not None:
        return ref
    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.cpu_spmm_timed(m, Xh, 0, threads, 1)
    t, used, _ = oracle.cpu_spmm_timed(m, Xh, 0, threads, 3)
    ms = float(np.mean(t)) * 1e-6
    return {"value": round(F / (ms * 1e-3) / 1e9, 1), "unit": "GFLOP/s", "ms": round(ms, 3), "cores": int(used),
            "kind": "port", "sample": f"full matrix, 3 timed SpMM iterations after one warm-up, width {Xh.shape[1]} "
                                      f"(the oracle's C port of the generated multi-threaded SpMM, FP32)"}


def bench_batch(reps: int, cpu: bool = True) -> dict:
    """256 mixed matrices: per-matrix launches (plain) vs one batched graph launch (learned)."""
    import torch
    from sable_gb300 import autotune, convert, synth
    from sable_gb300.plan import Plan
    mats, widths = synth.batch_256()
    rng = np.random.default_rng(0)
    xs, ys = [], []
    for m, w in zip(mats, widths):
        xs.append(torch.as_tensor(rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)).cuda())
        ys.append(torch.empty(m.n_rows if w == 1 else (m.n_rows, w), device="cuda"))
    from oracle import oracle
    from sable_gb300 import metrics
    plain, learned_comps = [], []
    errs_med = []
    nnz_work = 0
    bytes_work = 0   # algorithmic bytes of all 256 products (memory bound of the batch)
    for m, w in zip(mats, widths):
        bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
        f, rf, mlp = choices(m, bt, w)
        nnz_work += int(f[:, 2].sum()) * w
        bytes_work += metrics.spmv_bytes(m) if w == 1 else metrics.spmm_bytes(m, w)
        lay = "mixed" if w == 1 else "separate"
        plain.append(Plan(convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, rf, bt=bt),
                          split_layout=lay))
        learned_comps.append(convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, mlp,
                                              bt=bt))

    def run_plain():
        for p, x, y, w in zip(plain, xs, ys, widths):
            if w == 1:
                p.spmv(x, y)
            else:
                p.spmm(x, y)

    ms_p = autotune.time_ms(run_plain, reps)
    # the batch autotuner builds the learned plans per shape from the same choices
    batch, table = autotune.tune_batch(learned_comps, widths, xs, ys, spmm_tc="split3")
    ms_b = autotune.time_ms(lambda: batch.run(xs, ys), reps)
    info = batch.info()
    # every one of the batch's outputs against the FP64 oracle
    batch.run(xs, ys)
    batch.check()
    errs = []
    for m, w, x, y, p in zip(mats, widths, xs, ys, learned_comps):
        xn = x.cpu().numpy()
        yr, ya = oracle.spmv_vbrc(p, xn) if w == 1 else oracle.spmm_vbr(m, xn)
        r = oracle.report(y.cpu().numpy(), yr, ya)
        errs.append(r["max"])
        errs_med.append(r["median"])
    for p in plain:
        p.close()
    batch.close()
    cpu_b = None
    if cpu:
        # the oracle's C ports of the generated executors, one matrix after the
        # other (the reference runs one generated program per matrix), the
        # reference's block choice, all host cores per matrix
        threads, tot_ns, used = os.cpu_count() or 1, 0.0, 1
        for m, w, x in zip(mats, widths, xs):
            xn = x.cpu().numpy()
            if w == 1:
                bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
                _, rf, _ = choices(m, bt, 1)
                comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, rf, bt=bt,
                                        value_dtype=np.float64)
                t, u, _ = oracle.cpu_spmv_timed(comp, xn, threads, 3)
            else:
                t, u, _ = oracle.cpu_spmm_timed(m, xn, 0, threads, 3)
            used = max(used, int(u))   # small matrices split over fewer threads
            tot_ns += float(np.mean(t))
        cpu_ms = tot_ns * 1e-6
        cpu_b = {"value": round(2 * nnz_work / (cpu_ms * 1e6), 1), "unit": "GFLOP/s", "ms": round(cpu_ms, 3),
                 "cores": int(used), "kind": "port",
                 "sample": "all 256 matrices, sum over matrices of the mean of 3 timed iterations (the oracle's C ports "
                           "of the generated SpMV (FP64) and SpMM (FP32) executors, the reference block choice)"}
    return {"workload": "batch_256: 256 square matrices n log-U[1000,20000], partitions U[4,128], block p=0.02, "
                        "dense fraction U[0.2,0.8], sparse density U[0.02,0.4]; SpMM N=64 for half",
            "plain_ms": round(ms_p, 4), "plain_launches": len(mats) + sum(1 for w in widths if w == 1),
            "learned_batched_ms": round(ms_b, 4), "learned_vs_plain": round(ms_p / ms_b, 3),
            "work_gflop": round(2 * nnz_work / 1e9, 3), "learned_batched_gflops": round(2 * nnz_work / (ms_b * 1e6), 1),
            "roofline": {"bound": "hbm", "achieved": round(bytes_work / (ms_b * 1e-3) / 1e9, 1),
                         "peak": peaks()["hbm_gbs"], "unit": "GB/s",
                         "frac": round(bytes_work / (ms_b * 1e-3) / 1e9 / peaks()["hbm_gbs"], 4),
                         "bytes_per_run": int(bytes_work),
                         "note": "algorithmic bytes of the 256 products (each block at its cheaper FP32 encoding, "
                                 "x/X read once, y/Y written once) / batch time; the SpMM half is also bound by "
                                 "the split-BF16 tensor work (six products per dense value)"},
            "error_vs_fp64_scaled": {"max": float(np.max(errs)), "median": float(np.median(errs_med)),
                                     "matrices": len(errs), "tolerance": oracle.TOL,
                                     "measure": "per output |y - y_fp64| / (|A||x|), all 256 matrices"},
            "batch": {"n_units": info["n_units"], "n_ctas": info["n_ctas"], "stages": info["stages"],
                      "graph": True, "tuning": table},
            "cpu_baseline": cpu_b}


def run_spmm_profile(args):
    """The 50000^2 SpMM with the learned choice at one width and one launch
    shape, a few launches, nothing else (a small case for kernel profiles)."""
    import torch
    from sable_gb300 import convert, synth
    from sable_gb300.plan import Plan
    N, rt, cb = (int(v) for v in args.spmm_profile.split(","))
    m = synth.spmm_50k()
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    _, _, mlp = choices(m, bt, N)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, mlp, bt=bt)
    plan = Plan(comp, row_tile=rt, chunk_bytes=cb, spmm_tc="split3", split_layout="separate")
    X = torch.as_tensor(synth.dense_operand(m.n_cols, N, 7)).cuda()
    Y = torch.empty(m.n_rows, N, device="cuda")
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        plan.spmm(X, Y)
    s.record()
    for _ in range(args.steps):
        plan.spmm(X, Y)
    e.record()
    e.synchronize()
    plan.check()
    print(json.dumps({"spmm_profile": {"N": N, "row_tile": rt, "chunk_bytes": cb, "items": plan.stats()["n_chunks"],
                                       "ms_per_launch": s.elapsed_time(e) / args.steps}}))


def run_batch_profile(args):
    """The 256-matrix batch with the learned choice in the batch autotuner's
    usual shapes (per-warp SpMV plans, 16-row tiles, 32 KB items; SpMM plans
    with whole block rows), a few graph launches, nothing else (for kernel
    profiles and launch lists)."""
    import torch
    from sable_gb300 import autotune, convert, synth
    from sable_gb300.batch import Batch
    mats, widths = synth.batch_256()
    rng = np.random.default_rng(0)
    plans, xs, ys = [], [], []
    for m, w in zip(mats, widths):
        bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
        _, _, mlp = choices(m, bt, w)
        comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, mlp, bt=bt)
        shape = autotune.BATCH_SPMV_SHAPES[0] if w == 1 else autotune.BATCH_SPMM_SHAPES[0]
        plans.append(autotune._batch_plan(comp, shape, w, "split3"))
        xs.append(torch.as_tensor(rng.uniform(-1, 1, m.n_cols if w == 1 else (m.n_cols, w)).astype(np.float32)).cuda())
        ys.append(torch.empty(m.n_rows if w == 1 else (m.n_rows, w), device="cuda"))
    b = Batch(plans, widths, use_graph=True)
    for p in plans:
        p.close()
    for _ in range(args.warmup):
        b.run(xs, ys)
    s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record()
    for _ in range(args.steps):
        b.run(xs, ys)
    e0.record()
    e0.synchronize()
    b.check()
    print(json.dumps({"batch_profile": {"ms_per_run": s0.elapsed_time(e0) / args.steps, **b.info()}}))
    b.close()


def run_sable(args):
    import torch
    from sable_gb300 import _lib, autotune, blockmodel, convert
    from sable_gb300.plan import Plan
    if int(os.environ.get("RANK", "0")) == 0 and not args.quick and not args.no_cpu_baseline:
        compile_reference_spmm()   # before any GPU work, not beside it
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if args.strong and world > 1:
        from sable_gb300 import metrics, shard
        m_full, x, _, _, B_job = build_workload(0)
        a0, a1 = shard.shard_block_rows(m_full, world)[rank]
        m = shard.sub_block_rows(m_full, a0, a1)
        bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
        nnz = convert.block_nnz(m.val, bt)
        B = metrics.spmv_matrix_bytes(bt, nnz) + 4 * (m.n_rows + m.n_cols)
    else:
        m, x, bt, nnz, B = build_workload(rank)
        B_job = world * B
    feats, plain_choice, learned_choice = choices(m, bt, 1)
    comp_l = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, learned_choice, bt=bt)
    comp_p = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, plain_choice, bt=bt)
    plain = Plan(comp_p)
    xd = torch.as_tensor(x).cuda()
    yd = torch.empty(m.n_rows, dtype=torch.float32, device="cuda")
    if args.shape:  # a fixed per-warp shape instead of the autotuner (kernel profiles)
        rt, cb = (int(v) for v in args.shape.split(","))
        learned = autotune._build(comp_l, {"executor": "warp_items", "row_tile": rt, "chunk_bytes": cb}, 1, "split3")
    else:
        learned = autotune.tune(comp_l, xd, yd, N=1)
    flush = autotune.l2_flush

    with ClockSampler(local) as clk:
        t_learn = time_device(lambda: learned.run(xd, yd), args.steps, args.warmup, world, flush)
    t_plain = time_device(lambda: plain.spmv(xd, yd), args.steps, args.warmup, world, flush)
    # block choice alone: the reference's RandomForest choice in the learned form's launch shape
    rf_same = autotune._build(comp_p, learned.config, 1, "off")
    t_rf_same = time_device(lambda: rf_same.run(xd, yd), args.steps, args.warmup, world, flush)
    rf_same.close()
    ms_rf_same = max_over_ranks(statistics.mean(t_rf_same), world)
    ms = max_over_ranks(statistics.mean(t_learn), world)
    ms_plain = max_over_ranks(statistics.mean(t_plain), world)
    value = B_job / (ms * 1e-3) / 1e9
    value_plain = B_job / (ms_plain * 1e-3) / 1e9

    # end to end through the C ABI with host buffers (pinned), learned plan
    xh = torch.as_tensor(x).pin_memory()
    yh = torch.empty(m.n_rows, dtype=torch.float32).pin_memory()
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    e2e_plan = learned.plan
    for _ in range(args.warmup):
        _lib.check(lib.sable_spmv_host(e2e_plan.handle, xh.data_ptr(), yh.data_ptr(), stream), "spmv_host")
    barrier(world)
    e2e_t = []
    for _ in range(args.steps):
        flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(lib.sable_spmv_host(e2e_plan.handle, xh.data_ptr(), yh.data_ptr(), stream), "spmv_host")
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(statistics.mean(e2e_t), world)

    pk = peaks()
    achieved = B / (statistics.mean(t_learn) * 1e-3) / 1e9
    # DRAM bytes per launch of the work-item kernel the autotuner picked, from
    # the committed ncu summary of that kernel on this workload
    kernel = {"items": "spmv_items_kernel", "warp_items": "spmv_warp_items_kernel",
              "ring": "batch_kernel"}[learned.config["executor"]]
    traffic = None
    tf = ROOT / "profiles" / f"{kernel}_spmv_100k.md"
    if tf.exists():
        hit = re.search(r"traffic_bytes_per_launch:\s*(\d+)", tf.read_text())
        traffic = int(hit.group(1)) if hit else None
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True,
        "scaling": "strong" if args.strong and world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; no dataset)",
        "config": {"workload": WORKLOAD, "l2": "flushed between timed steps (256 MB write, then 256 MB read of a "
                                               "clean buffer so no dirty lines are written back inside the step)",
                   "choice": "learned MLP cost model (sable_gb300/models/block_cost_mlp.npz)",
                   "launch_shape": learned.config, "n_blocks": int(m.n_blocks), "stored_values": int(len(m.val)),
                   "nnz": int(nnz.sum()), "bytes_per_step": int(B), "dense_frac": round(float(learned_choice.mean()), 4),
                   "parallelism": (f"block-row shards x{world}" if args.strong and world > 1
                                   else f"replicas x{world}")},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": traffic,
                     "peak_source": pk["source"],
                     "kernel": kernel + ("" if learned.launches_per_run() == 1 else " + spmv_combine_kernel")},
        "e2e": {"value": round(B_job / e2e_s / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * m.n_cols,
                "d2h_bytes_per_step": 4 * m.n_rows},
        "gpu_launches": args.steps * learned.launches_per_run(),
        "plain": {"value": round(value_plain, 2), "unit": "GB/s", "ms_per_step": round(ms_plain, 5),
                  "choice": "reference RandomForest (models/density_threshold_spmv.pkl)",
                  "frac": round(B / (statistics.mean(t_plain) * 1e-3) / 1e9 / pk["hbm_gbs"], 4)},
        "learned_vs_plain": round(ms_plain / ms, 3),
        "block_choice_only": {"rf_choice_same_shape_ms": round(ms_rf_same, 5),
                              "learned_vs_rf_same_shape": round(ms_rf_same / ms, 3),
                              "what": "MLP vs RandomForest block choice, both in the learned form's launch shape"},
        "autotune": learned.table,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.quick:
        out["spmm_50k"] = bench_spmm(10, flush, cpu=not args.no_cpu_baseline)
        out["batch_256"] = bench_batch(10, cpu=not args.no_cpu_baseline)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(m, bt, plain_choice, x, B, args.steps)
    if rank == 0:
        print(json.dumps(out))
    learned.close()
    plain.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def reference_c(steps: int, compile_ok: bool):
    """The reference's own generated SpMV program for this workload (its
    multi-threaded form, OpenMP over the host cores; oracle/refc.py), run for
    `steps` timed iterations, or None when its sources are absent (or, with
    compile_ok False, when it is not compiled on this host yet).  Also returns
    its error against the FP64 oracle."""
    from oracle import oracle, refc
    if not refc.generated() or (not compile_ok and not refc.compiled(("mt",))):
        return None
    if compile_ok:
        # the SpMM programs compile in the same pool (the SpMV program takes longest)
        refc.compile(("mt",), spmm_widths=[w for w in refc.SPMM_WIDTHS if refc.spmm_generated(w)])
    r = refc.run(steps, kinds=("mt",))["mt"]
    m, x, comp = refc._workload()
    y, ya = oracle.spmv_vbrc(comp, x)
    rep = oracle.report(r["y"], y, ya, 1e-10)
    return r, rep


def cpu_baseline(m, bt, choice, x, B, steps: int) -> dict:
    """The reference's CPU executor on the host cores, `steps` iterations:
    its own generated C when compiled on this host (see reference_c), else
    the oracle's C port of it (FP64, its block choice, its compiler flags)."""
    ref = reference_c(steps, compile_ok=False)
    if ref is not None:
        r, rep = ref
        t = np.asarray(r["times_ns"], np.float64) * 1e-9
        return {"value": round(B / float(np.mean(t)) / 1e9, 3), "unit": "GB/s", "cores": int(r["threads"]),
                "kind": "reference",
                "sample": f"full 100000^2 matrix, {len(t)} SpMV iterations (mean) of the reference's generated "
                          f"multi-threaded C (its CFLAGS, MKL stand-in for its CSR part), FP64, its block choice; "
                          f"max error vs FP64 oracle {rep['max']:.1e} of |A||x|"}
    from oracle import oracle
    from sable_gb300 import convert
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, choice, bt=bt,
                            value_dtype=np.float64)
    threads = os.cpu_count() or 1
    oracle.cpu_spmv_timed(comp, x, threads, 2)
    t, used, _ = oracle.cpu_spmv_timed(comp, x, threads, steps)
    return {"value": round(B / (float(np.mean(t)) * 1e-9) / 1e9, 3), "unit": "GB/s", "cores": int(used),
            "kind": "port",
            "sample": f"full 100000^2 matrix, {steps} SpMV iterations (mean), FP64, reference block choice "
                      f"(the oracle's C port of the generated executor; the reference's own generated C is not "
                      f"compiled on this host)"}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    from sable_gb300 import blockmodel, convert
    m, x, bt, nnz, B = build_workload(0)
    ref = reference_c(args.steps, compile_ok=True)
    if ref is not None:
        r, rep = ref
        t = np.asarray(r["times_ns"], np.float64) * 1e-9
        ms = float(np.mean(t)) * 1e3
        kind, used = "reference", int(r["threads"])
        sample = (f"full matrix, {len(t)} timed SpMV iterations of the reference's own generated multi-threaded C "
                  f"(gen_multi_threaded_spmv, {used} OpenMP sections, its CFLAGS for this host, MKL stand-in for "
                  f"its CSR part; its first iteration dropped as it does); max error vs FP64 oracle "
                  f"{rep['max']:.1e} of |A||x|")
    else:
        plain_choice = blockmodel.RFTableModel().choose_dense(convert.block_features(m.val, bt, 1))
        comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, plain_choice, bt=bt,
                                value_dtype=np.float64)
        threads = os.cpu_count() or 1
        oracle.cpu_spmv_timed(comp, x, threads, max(1, args.warmup))
        t, used, _ = oracle.cpu_spmv_timed(comp, x, threads, args.steps)
        ms = float(np.mean(t)) * 1e-6
        kind = "port"
        sample = f"full matrix, {args.steps} timed SpMV iterations after {args.warmup} warm-up (oracle C port)"
    value = B / (ms * 1e-3) / 1e9
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; no dataset)",
        "config": {"workload": WORKLOAD, "choice": "reference RandomForest", "bytes_per_step": int(B)},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": int(used), "kind": kind,
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.quick:
        out["spmm_50k"] = reference_spmm_section()
    print(json.dumps(out))


def reference_spmm_section() -> dict:
    """The reference's own generated SpMM on the 50000^2 SpMM workload at
    N = 32 and 128 (reference_spmm), the same widths and operands as the GPU
    arm's spmm_50k section."""
    from oracle import refc
    from sable_gb300 import convert, metrics, synth
    m = synth.spmm_50k()
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    A64 = csr64(m, bt)
    out = {}
    for N in refc.SPMM_WIDTHS:
        r = reference_spmm(N, metrics.spmm_flops(m, N), A64, refc._spmm_operand(m, N))
        out[f"N{N}"] = r if r is not None else {"unavailable": "the reference's generated SpMM is not present"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="sable", choices=["sable", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--strong", action="store_true", help="under torchrun: shard the block rows of one matrix over the "
                                                          "ranks (strong scaling) instead of one replica per rank")
    ap.add_argument("--quick", action="store_true", help="headline SpMV only (no SpMM / batch sections)")
    ap.add_argument("--spmm-profile", help="N,ROW_TILE,CHUNK_BYTES: only run the 50000^2 SpMM (learned choice, "
                                           "split BF16) in this shape, for kernel profiles")
    ap.add_argument("--batch-profile", action="store_true", help="only run the 256-matrix batch in the autotuner's "
                                                                 "usual shapes (for kernel profiles)")
    ap.add_argument("--shape", help="ROW_TILE,CHUNK_BYTES: run the headline on the per-warp executor in this shape "
                                    "instead of autotuning (for kernel profiles)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.spmm_profile:
        run_spmm_profile(args)
    elif args.batch_profile:
        run_batch_profile(args)
    else:
        run_sable(args)


if __name__ == "__main__":
    main()
