"""The work-item records a plan uploads, decoded on the host and multiplied in
FP64 (sable_plan_layout_host: the records exactly as built, no GPU), against
the FP64 oracle: the standard records (ItemHeader: x column per panel
column, CSR entries with columns) and the compact records of the per-warp
executor (CompactHeader: x window as column runs, CSR entries as value +
window position / row word), every tile and split tile, with the format
invariants the kernels rely on checked along the way."""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import _lib, convert, synth

HDR = np.dtype([("row0", "<i4"), ("h", "<i4"), ("nq", "<i4"), ("ns", "<i4"), ("xcol_off", "<i4"),
                ("panel_off", "<i4"), ("rp_off", "<i4"), ("csr_off", "<i4"), ("tile", "<i4"), ("kidx", "<i4"),
                ("nitem", "<i4"), ("g", "<i4"), ("part_base", "<i8"), ("bytes", "<i4"), ("mat", "<i4")])
CHDR = np.dtype([("row0", "<i4"), ("h", "<i4"), ("nq", "<i4"), ("ns", "<i4"), ("runs_off", "<i4"),
                 ("panel_off", "<i4"), ("rp_off", "<i4"), ("val_off", "<i4"), ("tile", "<i4"), ("kidx", "<i4"),
                 ("nitem", "<i4"), ("meta_off", "<i4"), ("part_base", "<i8"), ("bytes", "<i4"), ("nrun", "<i2"),
                 ("nw", "<i2")])
assert HDR.itemsize == 64 and CHDR.itemsize == 64
CW_MAX, CW_MAX_ROWS = 1024, 64


def layout(comp, row_tile, chunk_bytes, schedule, split_layout):
    desc, keep = _lib.make_desc(comp)
    opts = _lib.PlanOpts(row_tile, chunk_bytes, 0, -1, schedule, split_layout)
    lib = _lib.load()
    nb, ni = ctypes.c_int64(), ctypes.c_int64()
    args = (ctypes.byref(desc), ctypes.byref(opts))
    _lib.check(lib.sable_plan_layout_host(*args, None, 0, ctypes.byref(nb), None, None, 0, ctypes.byref(ni)), "layout")
    rec = np.zeros(nb.value, np.uint8)
    off = np.zeros(ni.value, np.int64)
    byt = np.zeros(ni.value, np.int32)
    _lib.check(lib.sable_plan_layout_host(*args, rec.ctypes.data, rec.size, ctypes.byref(nb), off.ctypes.data,
                                          byt.ctypes.data, ni.value, ctypes.byref(ni)), "layout")
    return rec, off, byt


def decode_multiply(rec, off, byt, x, n_rows, compact):
    """y = A x from the records alone (FP64), plus the rows each tile covers."""
    x = np.asarray(x, np.float64)
    y = np.zeros(n_rows)
    cover = np.zeros(n_rows, np.int64)
    split_items = {}
    for o, b in zip(off, byt):
        R = rec[o:o + b]
        assert o % 16 == 0 and b % 16 == 0
        hd = np.frombuffer(R[:64].tobytes(), CHDR if compact else HDR)[0]
        assert hd["bytes"] == b
        h, nq, ns, row0 = int(hd["h"]), int(hd["nq"]), int(hd["ns"]), int(hd["row0"])
        panel = np.frombuffer(R[hd["panel_off"]:hd["panel_off"] + 16 * nq * h].tobytes(), "<f4").reshape(nq, h, 4)
        if compact:
            assert 1 <= h <= CW_MAX_ROWS
            runs = np.frombuffer(R[hd["runs_off"]:hd["runs_off"] + 8 * int(hd["nrun"])].tobytes(), "<i4").reshape(-1, 2)
            assert np.all(runs[:, 1] >= 1)
            xw = np.concatenate([np.zeros(ln) if c0 < 0 else x[c0:c0 + ln] for c0, ln in runs]) if len(runs) \
                else np.zeros(0)
            assert len(xw) == hd["nw"] <= CW_MAX and 4 * nq <= len(xw)
            part = np.einsum("qic,qc->i", panel.astype(np.float64), xw[:4 * nq].reshape(nq, 4)) if nq else np.zeros(h)
            if ns:
                val = np.frombuffer(R[hd["val_off"]:hd["val_off"] + 4 * ns].tobytes(), "<f4").astype(np.float64)
                meta = np.frombuffer(R[hd["meta_off"]:hd["meta_off"] + 2 * ns].tobytes(), "<u2").astype(np.int64)
                pos, row = meta & 1023, meta >> 10
                assert np.all((pos >= 4 * nq) & (pos < len(xw))) and np.all(row < h) and np.all(np.diff(row) >= 0)
                part = part + np.bincount(row, weights=val * xw[pos], minlength=h)
        else:
            xcol = np.frombuffer(R[hd["xcol_off"]:hd["xcol_off"] + 16 * nq].tobytes(), "<i4")
            part = np.einsum("qic,qc->i", panel.astype(np.float64), x[xcol].reshape(nq, 4)) if nq else np.zeros(h)
            if ns:
                rp = np.frombuffer(R[hd["rp_off"]:hd["rp_off"] + 4 * (h + 1)].tobytes(), "<i4")
                E = np.frombuffer(R[hd["csr_off"]:hd["csr_off"] + 8 * ns].tobytes(), "<u4").reshape(ns, 2)
                assert rp[0] == 0 and rp[-1] == ns and np.all(np.diff(rp) >= 0)
                val = E[:, 0].copy().view("<f4").astype(np.float64)
                part = part + np.bincount(np.repeat(np.arange(h), np.diff(rp)), weights=val * x[E[:, 1]], minlength=h)
        y[row0:row0 + h] += part
        if hd["nitem"] > 1:
            split_items.setdefault(int(hd["tile"]), []).append((row0, h, int(hd["kidx"]), int(hd["nitem"])))
        else:
            cover[row0:row0 + h] += 1
    for t, its in split_items.items():   # a split tile: all its items, same rows, kidx 0..nitem-1
        row0, h, _, nitem = its[0]
        assert sorted(k for _, _, k, _ in its) == list(range(nitem))
        assert all(r == row0 and hh == h for r, hh, _, _ in its)
        cover[row0:row0 + h] += 1
    return y, cover


def random_vbr(seed, rsizes, csizes, p):
    rng = np.random.default_rng(seed)
    present = rng.random((len(rsizes), len(csizes))) < p

    def fill(r, h, w, a, b):
        v = r.uniform(-1, 1, (h, w)).astype(np.float32)
        return v if r.random() < 0.5 else v * synth.block_pattern(r, h, w, r.uniform(0.02, 0.5), "uniform")

    return synth.assemble(rng, np.asarray(rsizes), np.asarray(csizes), present, fill)


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
