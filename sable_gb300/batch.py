"""Many VBR matrices in one persistent kernel launch (libsable's batch).

    b = Batch([plan_a, plan_b, ...], widths=[1, 64, ...], use_graph=True)
    b.run([x_a, X_b, ...], [y_a, Y_b, ...])      # CUDA tensors, row-major

width 1 runs SpMV on that matrix, width N > 1 (a multiple of 4) SpMM of
width N.  The batch copies the plans' device records at creation, so the
plans may be closed afterwards.  One CUDA graph launch per run (or, without
the graph, the same launches in a row), whatever the number of matrices:
the tcgen05 kernel over the split-BF16 SpMM matrices (one launch per N-slice
width), the per-warp kernel over the SpMV matrices of per-warp plans, the
persistent kernel over the work queue of the rest, and the combine of split
tiles, each only when it has work.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .plan import Plan, _stream_handle


class Batch:
    def __init__(self, plans: list[Plan], widths, ctas_per_sm: int = 0, use_graph: bool = True, stages: int = 0):
        widths = np.ascontiguousarray(widths, dtype=np.int32)
        if len(widths) != len(plans) or not len(plans):
            raise ValueError("one width per plan, at least one plan")
        self.widths = widths
        self.n_rows = [p.n_rows for p in plans]
        self.n_cols = [p.n_cols for p in plans]
        handles = (ctypes.c_void_p * len(plans))(*[p.handle for p in plans])
        opts = _lib.BatchOpts(int(ctas_per_sm), int(bool(use_graph)), int(stages))
        h = ctypes.c_void_p()
        _lib.check(_lib.load().sable_batch_create(handles, len(plans), widths.ctypes.data, ctypes.byref(opts),
                                                  ctypes.byref(h)), "sable_batch_create")
        self._h = h

    @property
    def handle(self) -> int:
        if not self._h:
            raise RuntimeError("batch is closed")
        return self._h.value

    def info(self) -> dict:
        i = _lib.BatchInfo()
        _lib.check(_lib.load().sable_batch_get_info(self.handle, ctypes.byref(i)), "sable_batch_get_info")
        return {k: getattr(i, k) for k, _ in i._fields_}

    def outputs(self, device="cuda"):
        """Result tensors of the right shapes (y [n_rows] or Y [n_rows, N])."""
        import torch
        return [torch.empty(r, dtype=torch.float32, device=device) if w == 1 else
                torch.empty(r, int(w), dtype=torch.float32, device=device) for r, w in zip(self.n_rows, self.widths)]

    def run(self, xs, ys, stream=None):
        import torch
        n = len(self.widths)
        if len(xs) != n or len(ys) != n:
            raise ValueError(f"need {n} operands and {n} results")
        for i, (x, y, w) in enumerate(zip(xs, ys, self.widths)):
            for t, rows, name in ((x, self.n_cols[i], "x"), (y, self.n_rows[i], "y")):
                if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
                    raise TypeError(f"{name}[{i}] must be a contiguous float32 CUDA tensor")
                if t.numel() != rows * int(w):
                    raise ValueError(f"{name}[{i}] must hold {rows} x {int(w)} values")
        xp = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
        yp = (ctypes.c_void_p * n)(*[y.data_ptr() for y in ys])
        _lib.check(_lib.load().sable_batch_run(self.handle, xp, yp, _stream_handle(stream)), "sable_batch_run")
        return ys

    def check(self, stream=None) -> None:
        _lib.check(_lib.load().sable_batch_check(self.handle, _stream_handle(stream)), "sable_batch_check")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.load().sable_batch_destroy(self._h.value)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
