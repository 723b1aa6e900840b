"""Device timings of dense / sparse block forms (the block model's data)."""
import numpy as np
import pytest

from sable_gb300 import blocktiming, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [1, 32])
def test_time_blocks_covers_every_block(cuda, N):
    blocks = [s.block for s, _ in zip(synth.blocks_200k(count=300), range(300))]
    cd, cs = blocktiming.time_blocks(blocks, N, reps=3)
    assert cd.shape == cs.shape == (300,)
    assert np.all(cd > 0) and np.all(cs > 0)
    # a 256 x 256 dense block costs more than a 2 x 2 one in both forms
    big = max(range(300), key=lambda k: blocks[k].size)
    small = min(range(300), key=lambda k: blocks[k].size)
    assert cd[big] > cd[small] and cs[big] > cs[small]


def test_trained_model_gains_over_reference_threshold(cuda):
    """On freshly timed blocks the model never saw (another seed), the
    committed MLP's choice is within 5 % of the measured-best per-block
    choice and well ahead of the reference RandomForest threshold."""
    from sable_gb300 import blockmodel
    model = blockmodel.MLPModel.load()
    rf = blockmodel.RFTableModel()
    feats, cd, cs = blocktiming.timing_set(seed=77, count=6000, batch=2000, reps=3)
    p = model.predict(feats)
    r_mlp = blockmodel.regret(p[:, 0] < p[:, 1], cd, cs)
    r_rf = blockmodel.regret(rf.choose_dense(feats), cd, cs)
    assert r_mlp <= 0.05, (r_mlp, r_rf)
    assert r_rf > 3 * r_mlp, (r_mlp, r_rf)
    # the plans' decision rule (cycles + kappa_spmv x stored bytes for SpMV):
    # within 5 % by cycles, and by its own cost on the SpMV blocks
    dec = model.choose_dense(feats)
    assert blockmodel.regret(dec, cd, cs) <= 0.05
    sv = feats[:, 5] == 1
    meas = blockmodel.decision_costs(np.log2(1.0 + np.stack([cd, cs], 1)), feats, model.kappa_spmv)
    r_dec = blockmodel.regret(dec[sv], meas[sv, 0], meas[sv, 1])
    r_rf_dec = blockmodel.regret(rf.choose_dense(feats)[sv], meas[sv, 0], meas[sv, 1])
    assert r_dec <= 0.05 and r_rf_dec > 3 * r_dec, (r_dec, r_rf_dec)
