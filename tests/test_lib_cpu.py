"""libsable host-side checks that need no GPU: the library loads, exports
every symbol include/sable.h declares, validates VBR arrays before any CUDA
call, and computes block features like the numpy path."""
import ctypes
import pathlib
import re

import numpy as np
import pytest

from sable_gb300 import _lib, convert, synth

HEADER = pathlib.Path(__file__).resolve().parents[1] / "include" / "sable.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sable_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_strerror_and_version():
    lib = _lib.load()
    assert lib.sable_strerror(_lib.SABLE_ERR_INVALID) == b"invalid VBR arrays"
    assert b"sm_103a" in lib.sable_version()


def _desc_for(m, **override):
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre,
                            np.ones(m.n_blocks, dtype=bool))
    for k, v in override.items():
        setattr(comp, k, v)
    return _lib.make_desc(comp)


@pytest.mark.parametrize("mutate,code", [
    ("bindx_desc", _lib.SABLE_ERR_INVALID),
    ("rpntr_flat", _lib.SABLE_ERR_INVALID),
    ("indx_short", _lib.SABLE_ERR_INVALID),
    ("bpntr_gap", _lib.SABLE_ERR_INVALID),
])
def test_invalid_vbr_rejected_before_cuda(mutate, code):
    m = synth.spmv_1000()
    bindx, rpntr, indx, bpntrb = m.bindx.copy(), m.rpntr.copy(), m.indx.copy(), m.bpntrb.copy()
    rows = np.nonzero(m.bpntre - m.bpntrb > 1)[0]
    a = int(rows[0])
    if mutate == "bindx_desc":
        b0 = int(m.bpntrb[a])
        bindx[b0], bindx[b0 + 1] = bindx[b0 + 1], bindx[b0]
    elif mutate == "rpntr_flat":
        rpntr[2] = rpntr[1]
    elif mutate == "indx_short":
        indx[1] -= 1
    elif mutate == "bpntr_gap":
        bpntrb[a] += 1
    desc, keep = _desc_for(m, bindx=bindx, rpntr=rpntr, indx=indx, bpntrb=bpntrb)
    h = ctypes.c_void_p()
    lib = _lib.load()
    rc = lib.sable_plan_create(ctypes.byref(desc), None, ctypes.byref(h))
    assert rc == code, (rc, lib.sable_last_error())
    assert not h.value


def test_block_features_match_numpy():
    m = synth.spmm_50k(seed=1010, n=400, parts=10, p=0.3)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre,
                            np.ones(m.n_blocks, dtype=bool))
    desc, keep = _lib.make_desc(comp)
    out = np.zeros((m.n_blocks, 6), dtype=np.float32)
    _lib.check(_lib.load().sable_block_features(ctypes.byref(desc), 32, out.ctypes.data), "features")
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    ref = convert.block_features(m.val, bt, 32)
    np.testing.assert_allclose(out, ref, rtol=1e-6)


def dry_run(comp, row_tile=0, chunk_bytes=0, split_layout=0, schedule=0):
    desc, keep = _lib.make_desc(comp)
    st = _lib.PlanStats()
    opts = _lib.PlanOpts(row_tile, chunk_bytes, 0, -1, schedule, split_layout)
    _lib.check(_lib.load().sable_plan_dry_run(ctypes.byref(desc), ctypes.byref(opts), ctypes.byref(st)), "dry_run")
    return {k: getattr(st, k) for k, _ in st._fields_}


@pytest.mark.parametrize("row_tile", [128, 64, 17, 1])
@pytest.mark.parametrize("chunk_bytes", [0, 4096, 6000, 32768])
@pytest.mark.parametrize("split_layout", [0, 1])
@pytest.mark.parametrize("schedule", [0, 2])
def test_layout_builder_edge_shapes(row_tile, chunk_bytes, split_layout, schedule):
    """Tall rows, width/height-1 partitions, empty rows, tiny work items:
    the builder's own bounds check (check_layout; for the per-warp executor's
    compact records check_compact_layout) passes and every stored value lands
    in the panel or the CSR segments exactly once."""
    rng = np.random.default_rng(1)
    rs, cs = np.array([1, 300, 5, 1, 64, 129, 7, 2, 40]), np.array([1, 3, 200, 1, 9, 33, 128, 2, 4, 77])
    present = rng.random((len(rs), len(cs))) < 0.6
    present[2, :] = False
    m = synth.assemble(rng, rs, cs, present, lambda r, h, w, a, b: r.uniform(-1, 1, (h, w)) *
                       (r.random((h, w)) < 0.4))
    dense = rng.random(m.n_blocks) < 0.5
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    st = dry_run(comp, row_tile, chunk_bytes, split_layout, schedule)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    assert st["dense_values"] == int(bt.size[dense].sum())
    assert st["sparse_nnz"] == (0 if comp.indptr is None else int(comp.indptr[-1]))
    assert st["dense_padded"] >= st["dense_values"]


@pytest.mark.parametrize("dense_frac", [0.0, 1.0, 0.5])
@pytest.mark.parametrize("split_layout", [0, 1])
def test_compact_window_overflow_splits(dense_frac, split_layout):
    """Compact records: a block row whose panel columns or CSR columns exceed
    the 1024-position x window is cut into more items until every window
    fits; the builder's checker (check_compact_layout) passes and nothing is
    lost."""
    rng = np.random.default_rng(5)
    rs, cs = np.array([8, 30]), np.full(60, 40)   # 2400 columns per block row
    present = np.ones((2, 60), bool)
    m = synth.assemble(rng, rs, cs, present, lambda r, h, w, a, b: r.uniform(-1, 1, (h, w)) *
                       (r.random((h, w)) < 0.3))
    dense = rng.random(m.n_blocks) < dense_frac
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    st = dry_run(comp, 8, 32768, split_layout, schedule=2)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    assert st["dense_values"] == int(bt.size[dense].sum())
    assert st["sparse_nnz"] == (0 if comp.indptr is None else int(comp.indptr[-1]))
    assert st["n_chunks"] > st["n_tiles"]   # windows forced splits


def test_large_items_schedule_0_only():
    """chunk_bytes above the staging size: accepted for one CTA per item (an
    SpMM-only plan), refused for the warp executors."""
    m = synth.spmm_50k(n=4000, parts=80)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, np.ones(m.n_blocks, bool))
    st = dry_run(comp, 128, 262144)
    assert st["n_chunks"] <= st["n_tiles"] + 2
    for sched in (1, 2):
        with pytest.raises(_lib.SableError):
            dry_run(comp, 128, 262144, schedule=sched)


def test_layout_builder_100k():
    """The 100000^2 workload builds, with < 2 % panel padding."""
    m = synth.spmv_100k()
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    nnz = convert.block_nnz(m.val, bt)
    dense = 4 * bt.size <= 8 * nnz + 4 * (bt.h + 1)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense, bt=bt)
    st = dry_run(comp)
    assert st["dense_values"] == int(bt.size[dense].sum())
    assert st["dense_padded"] < 1.02 * st["dense_values"]
    assert 15000 < m.n_blocks < 25000
    # compact records (per-warp executor, 8-row tiles): x columns as runs and
    # 6-byte CSR entries make the records smaller than the standard ones
    std8 = dry_run(comp, 8, 32768)
    cmp8 = dry_run(comp, 8, 32768, schedule=2)
    assert cmp8["dense_values"] == st["dense_values"] and cmp8["sparse_nnz"] == st["sparse_nnz"]
    assert cmp8["device_bytes"] < 0.95 * std8["device_bytes"]
