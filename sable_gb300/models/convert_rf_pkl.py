"""Extract the reference RandomForest block model into a flat tree table.

Usage: python -m sable_gb300.models.convert_rf_pkl <density_threshold_spmv.pkl>

The reference pickle (models/density_threshold_spmv.pkl of reikdas/SABLE,
scikit-learn RandomForestClassifier over [rows, cols, density%], class 1 =
keep the block dense) is loaded with a whitelisting unpickler and written as
density_threshold_spmv_rf.npz beside this script, which RFTableModel reads
without scikit-learn.  The script checks the table against the pickle's own
predict() on a grid of inputs before writing it.
"""
import sys
import warnings

import numpy as np

from sable_gb300 import blockmodel


def main(pkl: str) -> None:
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        model = blockmodel.load_reference_pkl(pkl)
    table = blockmodel.rf_to_table(model)
    np.savez_compressed(blockmodel.RF_TABLE, **table)
    rf = blockmodel.RFTableModel(blockmodel.RF_TABLE)
    rng = np.random.default_rng(0)
    X = np.stack([np.exp(rng.uniform(0, np.log(6000), 20000)).round(),
                  np.exp(rng.uniform(0, np.log(6000), 20000)).round(),
                  rng.uniform(0, 100, 20000)], axis=1)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = model.predict(X)
    mine = rf.predict(X)
    bad = int((ref != mine).sum())
    print(f"wrote {blockmodel.RF_TABLE} ({table['left'].size} nodes, {len(table['roots'])} trees); mismatches {bad}/20000")
    if bad:
        raise SystemExit("table disagrees with the pickle")


if __name__ == "__main__":
    main(sys.argv[1])
