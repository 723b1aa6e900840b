#!/usr/bin/env python
"""Benchmark: VBR SpMV on the 100000 x 100000 workload (GB/s, % of HBM roofline).

One step = one SpMV y = A x over the whole matrix (~2e4 blocks, ~5e7 stored
values), x and A resident in HBM.  Each timed step is bracketed by CUDA
events on the launching stream; a 256 MB buffer is written between steps to
flush L2 (129 MB), outside the events.  Forms:

  learned   per-block dense / sparse choice of the learned block model
            (byte-cost rule until its weights are trained), plan kernel
  plain     the reference's choice (its RandomForest), same kernel

`value` is the learned form; `e2e` runs the same SpMV through the C ABI
host-buffer entry (sable_spmv_host: pinned x copied in, y copied out, inside
the timed region).  `--impl reference` times the reference's CPU executor
(the oracle's C port of its generated code, FP64, all host cores) on the
same workload.  Under torchrun each rank runs its own seeded replica (weak
scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
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
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


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


def build_workload(rank: int):
    from sable_gb300 import blockmodel, convert, metrics, synth
    m = synth.spmv_100k(seed=synth.SEED_BASE + 1 + 100 * rank)
    x = synth.vector(m.n_cols, seed=31 + rank)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    nnz = convert.block_nnz(m.val, bt)
    B = metrics.spmv_matrix_bytes(bt, nnz) + 4 * (m.n_rows + m.n_cols)
    feats = convert.block_features(m.val, bt, 1)
    plain_choice = blockmodel.RFTableModel().choose_dense(feats)
    learned_model = blockmodel.default_model()
    if isinstance(learned_model, blockmodel.MLPModel):
        learned_choice = learned_model.choose_dense(feats)
        learned_name = "learned MLP cost model"
    else:
        learned_choice = 4 * bt.size <= 8 * nnz + 4 * (bt.h + 1)
        learned_name = "byte-cost rule (block model weights absent)"
    return m, x, bt, nnz, B, plain_choice, learned_choice, learned_name


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


def run_sable(args):
    import torch
    from sable_gb300 import convert
    from sable_gb300.plan import Plan
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    m, x, bt, nnz, B, plain_choice, learned_choice, learned_name = build_workload(rank)
    comp_l = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, learned_choice, bt=bt)
    comp_p = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, plain_choice, bt=bt)
    learned = Plan(comp_l)
    plain = Plan(comp_p)
    xd = torch.as_tensor(x).cuda()
    yd = torch.empty(m.n_rows, dtype=torch.float32, device="cuda")
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    flush = lambda: flush_buf.fill_(1)

    with ClockSampler(local) as clk:
        t_learn = time_device(lambda: learned.spmv(xd, yd), args.steps, args.warmup, world, flush)
    t_plain = time_device(lambda: plain.spmv(xd, yd), args.steps, args.warmup, world, flush)

    ms = max_over_ranks(statistics.mean(t_learn), world)
    ms_plain = max_over_ranks(statistics.mean(t_plain), world)
    value = world * B / (ms * 1e-3) / 1e9
    value_plain = world * B / (ms_plain * 1e-3) / 1e9

    # end to end through the C ABI with host buffers (pinned)
    xh = torch.as_tensor(x).pin_memory()
    yh = torch.empty(m.n_rows, dtype=torch.float32).pin_memory()
    from sable_gb300 import _lib
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(args.warmup):
        _lib.check(lib.sable_spmv_host(learned.handle, xh.data_ptr(), yh.data_ptr(), stream), "spmv_host")
    barrier(world)
    e2e_t = []
    for _ in range(args.steps):
        flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(lib.sable_spmv_host(learned.handle, xh.data_ptr(), yh.data_ptr(), stream), "spmv_host")
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(statistics.mean(e2e_t), world)

    pk = peaks()
    achieved = B / (statistics.mean(t_learn) * 1e-3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "spmv_100k_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("learned_bytes_per_launch")
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; no dataset)",
        "config": {"workload": WORKLOAD, "l2": "flushed between timed steps (256 MB write)",
                   "choice": learned_name, "n_blocks": int(m.n_blocks), "stored_values": int(len(m.val)),
                   "nnz": int(nnz.sum()), "bytes_per_step": int(B), "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": traffic,
                     "peak_source": pk["source"]},
        "e2e": {"value": round(world * B / e2e_s / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * m.n_cols,
                "d2h_bytes_per_step": 4 * m.n_rows},
        "gpu_launches": args.steps,
        "plain": {"value": round(value_plain, 2), "unit": "GB/s", "ms_per_step": round(ms_plain, 5),
                  "choice": "reference RandomForest (models/density_threshold_spmv.pkl)",
                  "frac": round(B / (statistics.mean(t_plain) * 1e-3) / 1e9 / pk["hbm_gbs"], 4)},
        "learned_vs_plain": round(ms_plain / ms, 3),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(m, bt, plain_choice, x, B, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(out))
    learned.close()
    plain.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def cpu_baseline(m, bt, choice, x, B, seconds: float = 15.0, threads: int | None = None) -> dict:
    """The reference's generated SpMV executor, as the oracle's C port (FP64,
    its own block choice), on the host cores."""
    from oracle import oracle
    from sable_gb300 import convert
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, choice, bt=bt,
                            value_dtype=np.float64)
    threads = threads or os.cpu_count() or 1
    t, used, _ = oracle.cpu_spmv_timed(comp, x, threads, 2)  # warm-up, sizes the sample
    per = max(float(np.median(t)) * 1e-9, 1e-4)
    iters = int(max(3, min(200, seconds / per)))
    t, used, _ = oracle.cpu_spmv_timed(comp, x, threads, iters)
    med = float(np.median(t)) * 1e-9
    return {"value": round(B / med / 1e9, 3), "unit": "GB/s", "cores": int(threads), "kind": "port",
            "sample": f"full 100000^2 matrix, {iters} SpMV iterations (median), FP64, reference block choice"}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    from sable_gb300 import convert
    m, x, bt, nnz, B, plain_choice, _, _ = build_workload(0)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, plain_choice, bt=bt,
                            value_dtype=np.float64)
    threads = os.cpu_count() or 1
    oracle.cpu_spmv_timed(comp, x, threads, max(1, args.warmup))
    t, used, _ = oracle.cpu_spmv_timed(comp, x, threads, args.steps)
    ms = float(np.mean(t)) * 1e-6
    value = B / (ms * 1e-3) / 1e9
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; no dataset)",
        "config": {"workload": WORKLOAD, "choice": "reference RandomForest", "bytes_per_step": int(B)},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": int(threads), "kind": "port",
                         "sample": f"full matrix, {args.steps} timed SpMV iterations after {args.warmup} warm-up"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="sable", choices=["sable", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_sable(args)


if __name__ == "__main__":
    main()
