"""The work-item records a plan uploads, decoded on the host and multiplied in
FP64 (sable_plan_layout_host: the records exactly as built, no GPU), against
the FP64 oracle: the standard records (ItemHeader: x column per panel
column, CSR entries with columns) and the compact records of the per-warp
executor (CompactHeader: x window as column runs, CSR entries as value +
window position / row word), every tile and split tile, with the format
invariants the kernels rely on checked along the way."""
import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import convert, synth

from layout_decode import decode_multiply, layout, random_vbr

CASES = {
    "edges": (7, [1, 300, 5, 1, 64, 129, 7, 2, 40], [1, 3, 200, 1, 9, 33, 128, 2, 4, 77], 0.6),
    "wide_rows": (8, [8, 30, 70], [40] * 60, 0.8),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("schedule", [0, 2])
@pytest.mark.parametrize("row_tile", [8, 17, 64, 128])
@pytest.mark.parametrize("chunk_bytes", [4096, 32768])
@pytest.mark.parametrize("split_layout", [0, 1])
def test_records_multiply_like_the_oracle(case, schedule, row_tile, chunk_bytes, split_layout):
    seed, rs, cs, p = CASES[case]
    m = random_vbr(seed, rs, cs, p)
    rng = np.random.default_rng(seed + 1)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, rng.random(m.n_blocks) < 0.5)
    x = synth.vector(m.n_cols, seed + 2).astype(np.float64)
    rec, off, byt = layout(comp, row_tile, chunk_bytes, schedule, split_layout)
    y, cover = decode_multiply(rec, off, byt, x, m.n_rows, compact=schedule == 2)
    y_ref, yabs = oracle.spmv_vbrc(comp, x)
    assert np.all(cover == 1)           # every row by exactly one tile
    assert np.all(np.abs(y - y_ref) <= 1e-12 * (yabs + 1.0))


def test_example_fixture_compact(golden):
    """The reference's 11x11 example: the compact records of every shape give
    its canonical y = A 1."""
    ex = synth.VbrMatrix(*[np.asarray(a) for a in golden.arrays("example_arrays")])
    comp = convert.compress(np.asarray(ex.val, np.float32), ex.rpntr, ex.cpntr, ex.indx, ex.bindx, ex.bpntrb,
                            ex.bpntre, np.ones(ex.n_blocks, bool))
    for rt in (1, 2, 8, 128):
        rec, off, byt = layout(comp, rt, 4096, 2, 0)
        y, cover = decode_multiply(rec, off, byt, np.ones(11), 11, compact=True)
        np.testing.assert_allclose(y, golden.arr("example_canon", "spmv"), rtol=1e-6)
