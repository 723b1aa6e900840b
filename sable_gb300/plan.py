"""Python handle of a libsable plan (one matrix laid out on the GPU).

A plan is what the reference's inspector produces (one generated C program
per matrix, src/codegen.py:293-452): here it is a device layout built by
sable_plan_create and executed by sable_spmv / sable_spmm on a CUDA stream.
PyTorch supplies device memory and streams only.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .convert import Compressed, compress, block_table, choose_dense


def _stream_handle(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


class Plan:
    """GPU plan of one compressed VBR matrix.

    schedule "items" (one CTA per work item) serves SpMV, SpMM and batches;
    with chunk_bytes above 78643 (up to 1 MB, whole block rows per item) it
    is an SpMM-only plan.  "warp_items" (one warp per compact work item, the
    fastest SpMV on large matrices) is an SpMV-only plan.  The other product
    on such a plan raises SableError (SABLE_ERR_UNSUPPORTED)."""

    SCHEDULES = {"items": 0, "persistent": 1, "warp_items": 2}
    SPLIT_LAYOUTS = {"mixed": 0, "separate": 1}
    # dense-block SpMM precision for N >= 32: FP32 CUDA cores, or split BF16 on
    # the tensor cores with 2 terms (3 products) or 3 terms (6 products)
    TC_MODES = {False: 0, True: 1, 0: 0, 1: 1, 2: 2, "off": 0, "split2": 1, "split3": 2}

    # split-BF16 SpMM kernel: tcgen05 MMAs with TMEM accumulators, or the
    # warp-level mma.sync path
    TC_KERNELS = {"umma": 0, "mma_sync": 1}

    def __init__(self, comp: Compressed, row_tile: int = 0, chunk_bytes: int = 0, spmm_tc=False,
                 device: int | None = None, schedule: str = "items", split_layout: str = "mixed",
                 tc_kernel: str = "umma"):
        lib = _lib.load()
        desc, keep = _lib.make_desc(comp)
        if spmm_tc not in self.TC_MODES:
            raise ValueError(f"spmm_tc {spmm_tc!r}: one of {sorted(map(str, self.TC_MODES))}")
        if tc_kernel not in self.TC_KERNELS:
            raise ValueError(f"tc_kernel {tc_kernel!r}: one of {sorted(self.TC_KERNELS)}")
        opts = _lib.PlanOpts(int(row_tile), int(chunk_bytes), self.TC_MODES[spmm_tc], -1 if device is None else int(device),
                             self.SCHEDULES[schedule], self.SPLIT_LAYOUTS[split_layout], self.TC_KERNELS[tc_kernel])
        h = ctypes.c_void_p()
        _lib.check(lib.sable_plan_create(ctypes.byref(desc), ctypes.byref(opts), ctypes.byref(h)), "sable_plan_create")
        del keep
        self._h = h
        self.n_rows = comp.n_rows
        self.n_cols = comp.n_cols
        self.spmm_tc = self.TC_MODES[spmm_tc]
        self.row_tile = row_tile
        self.chunk_bytes = chunk_bytes
        self.schedule = schedule
        self.split_layout = split_layout
        self.tc_kernel = tc_kernel

    @property
    def handle(self) -> int:
        if not self._h:
            raise RuntimeError("plan is closed")
        return self._h.value

    def stats(self) -> dict:
        s = _lib.PlanStats()
        _lib.check(_lib.load().sable_plan_get_stats(self.handle, ctypes.byref(s)), "sable_plan_get_stats")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def check(self, stream=None) -> None:
        """Raise if a bounded device wait ran out in an earlier launch."""
        _lib.check(_lib.load().sable_plan_check(self.handle, _stream_handle(stream)), "sable_plan_check")

    def chunk_tiles(self) -> np.ndarray:
        n = self.stats()["n_chunks"]
        out = np.zeros(n, dtype=np.int64)
        _lib.check(_lib.load().sable_plan_chunk_tiles(self.handle, out.ctypes.data), "sable_plan_chunk_tiles")
        return out

    # -- SpMV ----------------------------------------------------------------
    def spmv(self, x, y=None, stream=None):
        """y = A x for CUDA float32 tensors (y allocated when None)."""
        import torch
        _check_dev(x, self.n_cols, "x")
        if y is None:
            y = torch.empty(self.n_rows, dtype=torch.float32, device=x.device)
        _check_dev(y, self.n_rows, "y")
        _lib.check(_lib.load().sable_spmv(self.handle, x.data_ptr(), y.data_ptr(), _stream_handle(stream)), "sable_spmv")
        return y

    def spmv_timed(self, x, y, cycles, stream=None):
        _lib.check(_lib.load().sable_spmv_timed(self.handle, x.data_ptr(), y.data_ptr(), cycles.data_ptr(),
                                                _stream_handle(stream)), "sable_spmv_timed")

    def spmv_host(self, x: np.ndarray, y: np.ndarray | None = None, stream=None) -> np.ndarray:
        """y = A x from host buffers (copies in and out, synchronises)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.shape != (self.n_cols,):
            raise ValueError(f"x must have {self.n_cols} entries")
        if y is None:
            y = np.empty(self.n_rows, dtype=np.float32)
        _lib.check(_lib.load().sable_spmv_host(self.handle, x.ctypes.data, y.ctypes.data, _stream_handle(stream)),
                   "sable_spmv_host")
        return y

    # -- SpMM ----------------------------------------------------------------
    def spmm(self, X, Y=None, stream=None):
        """Y = A X for row-major CUDA float32 tensors X [n_cols, N]."""
        import torch
        if X.dim() != 2 or X.shape[0] != self.n_cols:
            raise ValueError(f"X must be [{self.n_cols}, N]")
        N = X.shape[1]
        if Y is None:
            Y = torch.empty(self.n_rows, N, dtype=torch.float32, device=X.device)
        if X.dtype != torch.float32 or Y.dtype != torch.float32 or not X.is_cuda or not Y.is_cuda:
            raise TypeError("X and Y must be float32 CUDA tensors")
        if X.stride(1) != 1 or Y.stride(1) != 1:
            raise ValueError("X and Y must be row-major")
        _lib.check(_lib.load().sable_spmm(self.handle, X.data_ptr(), X.stride(0), Y.data_ptr(), Y.stride(0), N,
                                          _stream_handle(stream)), "sable_spmm")
        return Y

    def spmm_timed(self, X, Y, cycles, stream=None):
        _lib.check(_lib.load().sable_spmm_timed(self.handle, X.data_ptr(), Y.data_ptr(), X.shape[1], cycles.data_ptr(),
                                                _stream_handle(stream)), "sable_spmm_timed")

    def spmm_host(self, X: np.ndarray, stream=None) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        N = X.shape[1]
        Y = np.empty((self.n_rows, N), dtype=np.float32)
        _lib.check(_lib.load().sable_spmm_host(self.handle, X.ctypes.data, Y.ctypes.data, N, _stream_handle(stream)),
                   "sable_spmm_host")
        return Y

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.load().sable_plan_destroy(self._h.value)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _check_dev(t, n, name):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32:
        raise TypeError(f"{name} must be a float32 CUDA tensor")
    if t.numel() != n or not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous with {n} entries")


def plan_from_vbr(m, dense_mask=None, density=None, model=None, N: int = 1, **opts) -> Plan:
    """Plan of an uncompressed VBR matrix (arrays val, indx, bindx, rpntr,
    cpntr, bpntrb, bpntre) with the per-block choice given by dense_mask, a
    density threshold, or a block model (see convert.choose_dense)."""
    bt = block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    if dense_mask is None:
        if density is None and model is None:
            dense_mask = np.ones(len(bt.off), dtype=bool)
        else:
            dense_mask = choose_dense(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre,
                                      density=density, model=model, N=N, bt=bt)
    comp = compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense_mask, bt=bt)
    return Plan(comp, **opts)
