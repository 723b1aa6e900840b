"""ORACLE — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module, as the checker or the timed CPU reference; the product
(sable_gb300) never imports it.

Host FP64 oracle of the reference's generated executor (see vbr_oracle.c
for the file:line each routine follows) and the per-row parity measure:

    |y_gpu - y_ref|_i <= tol * (|A| |x|)_i ,  tol = 1e-5

report(): max and median of |y_gpu - y_ref|_i / (|A||x|)_i over rows.
"""
from __future__ import annotations

import ctypes
from ctypes import c_int, c_int32, c_int64, c_void_p

import numpy as np

from . import build as _build

TOL = 1e-5
# Split-BF16 with two terms per operand (three products): each product is
# off by at most |a_lo b_lo| + |a r_b| + |r_a b| <= 3 * 2^-16 |a b|, r being
# what hi + lo leave out of an FP32 value (round-to-nearest BF16 twice).
TOL_SPLIT2 = 3.0 * 2.0 ** -16
_libs = {}


def _load(which: str) -> ctypes.CDLL:
    if which not in _libs:
        _build.build()
        lib = ctypes.CDLL(str(_build.CHECKER if which == "checker" else _build.CPUREF))
        i32, i64, p = c_int32, c_int64, c_void_p
        lib.oracle_spmv_vbrc.restype = c_int
        lib.oracle_spmv_vbrc.argtypes = [i32, i32, i32, i32, p, p, p, p, p, p, i64, p, p, i64, p, p, p, p, p, p]
        lib.oracle_spmm_vbr.restype = c_int
        lib.oracle_spmm_vbr.argtypes = [i32, i32, i32, i32, p, p, p, p, p, p, i64, p, i32, i32, p, p, p]
        lib.cpu_spmv_timed.restype = c_int
        lib.cpu_spmv_timed.argtypes = [i32, i32, i32, p, p, p, p, p, p, i64, p, p, i64, p, p, p, p, p, c_int, c_int, p]
        lib.cpu_spmm_timed.restype = c_int
        lib.cpu_spmm_timed.argtypes = [i32, i32, i32, p, p, p, p, p, p, i64, p, i32, i32, p, p, c_int, c_int, p]
        _libs[which] = lib
    return _libs[which]


def _a(x, dt):
    return np.ascontiguousarray(np.asarray(x), dtype=dt)


def _p(a):
    return None if a is None or a.size == 0 else a.ctypes.data


class _Vbrc:
    """Arrays of a compressed matrix in the oracle's C types."""

    def __init__(self, comp, value_dtype=np.float64):
        self.rpntr = _a(comp.rpntr, np.int32)
        self.cpntr = _a(comp.cpntr, np.int32)
        self.bpntrb = _a(comp.bpntrb, np.int32)
        self.bpntre = _a(comp.bpntre, np.int32)
        self.bindx = _a(comp.bindx, np.int32)
        self.indx = _a(comp.indx, np.int64)
        self.val = _a(comp.val, value_dtype)
        self.ublocks = _a(comp.ublocks, np.int32)
        has = comp.indptr is not None and len(comp.indptr) > 0
        self.indptr = _a(comp.indptr, np.int64) if has else None
        self.indices = _a(comp.indices, np.int32) if has else None
        self.csr_val = _a(comp.csr_val, np.float64) if has else None
        self.n_rows = int(self.rpntr[-1])
        self.n_cols = int(self.cpntr[-1])
        self.nbr = len(self.rpntr) - 1
        self.nbc = len(self.cpntr) - 1


def spmv_vbrc(comp, x):
    """FP64 y and |A||x| of a compressed matrix (oracle_spmv_vbrc)."""
    v = _Vbrc(comp)
    x = _a(x, np.float64)
    y = np.zeros(v.n_rows)
    ya = np.zeros(v.n_rows)
    rc = _load("checker").oracle_spmv_vbrc(v.n_rows, v.n_cols, v.nbr, v.nbc, _p(v.rpntr), _p(v.cpntr), _p(v.bpntrb),
                                           _p(v.bpntre), _p(v.bindx), _p(v.indx), len(v.indx) - 1, _p(v.val),
                                           _p(v.ublocks), len(v.ublocks), _p(v.indptr), _p(v.indices),
                                           _p(v.csr_val), _p(x), _p(y), _p(ya))
    if rc:
        raise ValueError("oracle_spmv_vbrc: inconsistent arrays")
    return y, ya


def spmm_vbr(m, X, density: int = 0):
    """FP64 Y and |A||X| of an uncompressed matrix (oracle_spmm_vbr)."""
    rp, cp = _a(m.rpntr, np.int32), _a(m.cpntr, np.int32)
    bb, be, bi = _a(m.bpntrb, np.int32), _a(m.bpntre, np.int32), _a(m.bindx, np.int32)
    ix, val = _a(m.indx, np.int64), _a(m.val, np.float64)
    X = _a(X, np.float64)
    N = X.shape[1]
    n_rows = int(rp[-1])
    Y = np.zeros((n_rows, N))
    Ya = np.zeros((n_rows, N))
    rc = _load("checker").oracle_spmm_vbr(n_rows, int(cp[-1]), len(rp) - 1, len(cp) - 1, _p(rp), _p(cp), _p(bb),
                                          _p(be), _p(bi), _p(ix), len(bi), _p(val), int(density), N, _p(X), _p(Y),
                                          _p(Ya))
    if rc:
        raise ValueError("oracle_spmm_vbr: inconsistent arrays")
    return Y, Ya


def report(y_gpu, y_ref, yabs, tol: float = TOL) -> dict:
    """Per-row error relative to |A||x| (max, median) and the pass flag at tol."""
    y_gpu = np.asarray(y_gpu, dtype=np.float64).ravel()
    y_ref = np.asarray(y_ref, dtype=np.float64).ravel()
    scale = np.asarray(yabs, dtype=np.float64).ravel()
    err = np.abs(y_gpu - y_ref)
    ratio = np.where(scale > 0, err / np.where(scale > 0, scale, 1.0), np.where(err > 0, np.inf, 0.0))
    mx = float(ratio.max()) if ratio.size else 0.0
    return {"max": mx, "median": float(np.median(ratio)) if ratio.size else 0.0, "pass": bool(mx <= tol),
            "rows": int(ratio.size)}


def cpu_spmv_timed(comp, x, threads: int, iters: int):
    """Timed CPU port of the generated SpMV executor (FP64 as the reference).
    Returns (per-iteration ns, threads used, y)."""
    v = _Vbrc(comp)
    x = _a(x, np.float64)
    y = np.zeros(v.n_rows)
    times = np.zeros(iters, dtype=np.int64)
    used = _load("cpuref").cpu_spmv_timed(v.n_rows, v.nbr, v.nbc, _p(v.rpntr), _p(v.cpntr), _p(v.bpntrb),
                                          _p(v.bpntre), _p(v.bindx), _p(v.indx), len(v.indx) - 1, _p(v.val),
                                          _p(v.ublocks), len(v.ublocks), _p(v.indptr), _p(v.indices), _p(v.csr_val),
                                          _p(x), _p(y), int(threads), int(iters), _p(times))
    return times, used, y


def cpu_spmm_timed(m, X, density: int, threads: int, iters: int):
    """Timed CPU port of the generated SpMM executor (FP32 as the reference)."""
    rp, cp = _a(m.rpntr, np.int32), _a(m.cpntr, np.int32)
    bb, be, bi = _a(m.bpntrb, np.int32), _a(m.bpntre, np.int32), _a(m.bindx, np.int32)
    ix, val = _a(m.indx, np.int64), _a(m.val, np.float32)
    X = _a(X, np.float32)
    N = X.shape[1]
    Y = np.zeros((int(rp[-1]), N), dtype=np.float32)
    times = np.zeros(iters, dtype=np.int64)
    used = _load("cpuref").cpu_spmm_timed(int(rp[-1]), len(rp) - 1, len(cp) - 1, _p(rp), _p(cp), _p(bb), _p(be),
                                          _p(bi), _p(ix), len(bi), _p(val), int(density), N, _p(X), _p(Y),
                                          int(threads), int(iters), _p(times))
    return times, used, Y
