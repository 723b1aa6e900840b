"""Train the block cost model (MLP 6 -> 64 -> 64 -> 2) on GB300 timings.

    python -m sable_gb300.models.train_block_mlp --count 200000 \\
        --out sable_gb300/models/block_cost_mlp.npz [--save-data t.npz | --data t.npz]

1. Times every block of the synthetic block set (synth.blocks_200k: h, w
   log-uniform in [2, 256], density U[0.01, 1], uniform / banded /
   row-clustered, N in {1, 8, 32, 128}) as a dense and as a sparse work item
   on the GPU (blocktiming.timing_set) — the counterpart of the reference's
   CPU timing study (studies/threshold.py:32-86).
2. Targets: log2(1 + cycles) of both forms.  80 % of the blocks train the
   network with libsable's own kernels (Adam, sable_mlp_train_step); 20 %
   are held out.
3. kappa_spmv: the median cycles per stored byte of the large (>= 50 KB)
   dense SpMV blocks of the training part, the cost of a byte when DRAM is
   saturated.  SpMV decisions add it per stored byte to the predicted cycles
   (blockmodel.decision_costs).
4. Reports on the held-out blocks the regret of each choice rule against the
   measured-best form — the MLP (pure cycle prediction, and its decision rule
   with the byte term, measured by cycles + kappa_spmv x bytes), the
   reference RandomForest (the fallback), the byte rule, fixed density
   thresholds — overall and per N, and writes the weights, normalisation,
   kappa_spmv and these figures to --out.
Needs a CUDA device; prints one JSON summary line last.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def main(argv=None) -> int:
    from sable_gb300 import blockmodel, blocktiming, synth

    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=200000)
    ap.add_argument("--seed", type=int, default=synth.SEED_BASE + 4)
    ap.add_argument("--batch-blocks", type=int, default=10000)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=str(blockmodel.MLP_FILE))
    ap.add_argument("--data", help="load timings from this .npz instead of timing")
    ap.add_argument("--save-data", help="write the timings to this .npz")
    a = ap.parse_args(argv)
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731

    t0 = time.time()
    if a.data:
        with np.load(a.data) as z:
            feats, cd, cs = z["feats"], z["cyc_dense"], z["cyc_sparse"]
    else:
        feats, cd, cs = blocktiming.timing_set(a.seed, a.count, a.batch_blocks, log=log, reps=a.reps)
        if a.save_data:
            np.savez_compressed(a.save_data, feats=feats, cyc_dense=cd, cyc_sparse=cs)
    t_timing = time.time() - t0
    n = len(feats)
    targets = np.log2(1.0 + np.stack([cd, cs], 1)).astype(np.float32)
    perm = np.random.default_rng(a.seed).permutation(n)
    ntr = int(0.8 * n)
    tr, te = perm[:ntr], perm[ntr:]
    g = blockmodel.transform_features(feats[tr])
    mean, std = g.mean(0).astype(np.float32), (g.std(0) + 1e-3).astype(np.float32)

    t1 = time.time()
    trainer = blockmodel.MLPTrainer(blockmodel.init_params(a.seed), mean, std)
    hist = trainer.fit(feats[tr], targets[tr], epochs=a.epochs, batch=2048, lr=a.lr, lr_final=a.lr / 10, seed=a.seed,
                       log=log)
    t_train = time.time() - t1
    model = blockmodel.MLPModel(trainer.params(), mean, std)
    ftr = feats[tr]
    big = (ftr[:, 5] == 1) & (4 * ftr[:, 0] * ftr[:, 1] >= 50000)
    kappa = float(np.median(cd[tr][big] / (4 * ftr[big, 0] * ftr[big, 1]))) if big.any() else 0.0

    ft, dt, st = feats[te], cd[te], cs[te]
    pred = model.predict(ft)
    # SpMV blocks measured by cycles + kappa x stored bytes: the decision cost
    sv = ft[:, 5] == 1
    meas = blockmodel.decision_costs(np.log2(1.0 + np.stack([dt, st], 1)), ft, kappa)
    dec = blockmodel.decision_costs(pred, ft, kappa)
    rules = {
        "mlp": pred[:, 0] < pred[:, 1],
        "mlp_decision": dec[:, 0] < dec[:, 1],
        "rf_reference": blockmodel.RFTableModel().choose_dense(ft),
        "byte_rule": blockmodel.byte_rule(ft),
        "all_dense": np.ones(len(te), bool),
        "all_sparse": np.zeros(len(te), bool),
    }
    for thr in (20, 50, 80):
        rules[f"density_gt_{thr}"] = blockmodel.ThresholdModel(thr).choose_dense(ft)
    summary = {"blocks": int(n), "train": int(ntr), "held_out": int(len(te)), "timing_s": round(t_timing, 1),
               "train_s": round(t_train, 1), "final_loss": hist[-1],
               "rmse_log2": float(np.sqrt(((pred - targets[te]) ** 2).mean())),
               "regret": {k: blockmodel.regret(v, dt, st) for k, v in rules.items()},
               "regret_by_N": {}}
    for N in (1, 8, 32, 128):
        sel = ft[:, 5] == N
        summary["regret_by_N"][str(N)] = {k: blockmodel.regret(v[sel], dt[sel], st[sel]) for k, v in rules.items()}
    summary["kappa_spmv"] = kappa
    summary["regret_spmv_decision_cost"] = {k: blockmodel.regret(v[sv], meas[sv, 0], meas[sv, 1])
                                            for k, v in rules.items()}
    model.meta = {"trained_on": "synthetic blocks_200k timings (SM cycles, GB300)", "blocks": n,
                  "regret_mlp": summary["regret"]["mlp"], "regret_rf": summary["regret"]["rf_reference"],
                  "regret_byte_rule": summary["regret"]["byte_rule"], "epochs": a.epochs, "kappa_spmv": kappa,
                  "regret_mlp_spmv_decision": summary["regret_spmv_decision_cost"]["mlp_decision"],
                  "regret_rf_spmv_decision": summary["regret_spmv_decision_cost"]["rf_reference"]}
    model.save(a.out)
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    sys.exit(main())
