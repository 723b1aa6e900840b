"""Host decoder of the work-item records a plan uploads (shared by the CPU
tests): sable_plan_layout_host returns the records exactly as built, no GPU;
decode_multiply walks them in FP64 and checks the format invariants the
kernels rely on (16-byte alignment, window runs, 16-bit position / row words,
row pointers, split tiles)."""
import ctypes

import numpy as np

from sable_gb300 import _lib, synth

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
