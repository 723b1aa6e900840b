"""Host side of the block cost model: the block-diagonal timing layout, the
feature rows, the choice rules and the regret measure."""
import numpy as np

from sable_gb300 import blockmodel, blocktiming, convert, synth
from oracle import mlp_oracle


def sample_blocks(n, seed=synth.SEED_BASE + 4):
    return [s.block for s, _ in zip(synth.blocks_200k(seed, count=n), range(n))]


def test_diag_layout_round_trip():
    blocks = sample_blocks(60)
    m = blocktiming.diag_vbr(blocks)
    assert m.n_blocks == 60 and m.n_rows == sum(b.shape[0] for b in blocks)
    back = blocktiming.matrix_blocks(m)
    assert all(np.array_equal(a, b) for a, b in zip(blocks, back))


def test_companion_layout():
    """Sample block k and its dense companion share block row k."""
    blocks = sample_blocks(40)
    m = blocktiming.diag_vbr(blocks, companion_cols=64)
    convert.validate(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx)
    assert m.n_blocks == 80 and m.n_cols == sum(b.shape[1] for b in blocks) + 64 * 40
    back = blocktiming.matrix_blocks(m)
    assert all(np.array_equal(a, back[2 * k]) for k, a in enumerate(blocks))
    assert all(back[2 * k + 1].shape == (a.shape[0], 64) and np.all(back[2 * k + 1] != 0) for k, a in enumerate(blocks))


def test_block_stats_match_feature_rows():
    blocks = sample_blocks(80)
    m = blocktiming.diag_vbr(blocks)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    np.testing.assert_allclose(blocktiming.block_stats(blocks, 32), convert.block_features(m.val, bt, 32), rtol=1e-6)


def test_product_transform_and_init_match_oracle():
    f = np.abs(np.random.default_rng(1).normal(5, 3, (20, 6))).astype(np.float32)
    np.testing.assert_allclose(blockmodel.transform_features(f), mlp_oracle.transform(f, np.zeros(6), np.ones(6)))
    assert blockmodel.init_params(3).size == mlp_oracle.NPARAMS


def test_regret_and_rules():
    td = np.array([1.0, 5.0, 2.0])
    ts = np.array([2.0, 1.0, 2.0])
    assert blockmodel.regret(np.array([True, False, True]), td, ts) == 0.0
    assert abs(blockmodel.regret(np.array([False, True, False]), td, ts) - (2 + 5 + 2) / 4 + 1) < 1e-12
    f = np.array([[10, 10, 100, 1.0, 0, 1], [10, 10, 5, 0.05, 0, 1]], np.float32)
    np.testing.assert_array_equal(blockmodel.byte_rule(f), [True, False])


def test_decision_costs():
    """Stored bytes per form (compact 6-byte CSR entries for SpMV, standard
    8-byte entries + row pointers for SpMM) and the byte term of the SpMV
    decision cost."""
    f = np.array([[10, 20, 50, 0.25, 0, 1], [10, 20, 50, 0.25, 0, 32]], np.float32)
    np.testing.assert_array_equal(blockmodel.stored_bytes(f), [[800, 300], [800, 444]])
    lc = np.log2(1.0 + np.array([[100.0, 200.0], [100.0, 200.0]]))
    c = blockmodel.decision_costs(lc, f, 2.0)
    np.testing.assert_allclose(c, [[100 + 1600, 200 + 600], [100, 200]])  # no byte term for SpMM


def test_committed_model_file():
    z = np.load(blockmodel.MLP_FILE)
    assert z["params"].shape == (mlp_oracle.NPARAMS,) and np.all(np.isfinite(z["params"]))
    assert np.all(z["std"] > 0)
    assert float(z["regret_mlp"]) <= 0.05 < float(z["regret_rf"])
    # the SpMV decision rule's byte term: measured, plausible, and its regret
    assert 0.5 < float(z["kappa_spmv"]) < 8.0
    assert float(z["regret_mlp_spmv_decision"]) <= 0.05 < float(z["regret_rf_spmv_decision"])
