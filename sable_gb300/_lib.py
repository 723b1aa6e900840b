"""ctypes binding of libsable.so (the C ABI declared in include/sable.h).

The library is the only compute path of this package: if it cannot be built
or loaded, every operation raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import c_double, POINTER, c_char_p, c_float, c_int, c_int32, c_int64, c_void_p

import numpy as np

SABLE_OK = 0
SABLE_ERR_INVALID = -1
SABLE_ERR_CUDA = -2
SABLE_ERR_NOMEM = -3
SABLE_ERR_UNSUPPORTED = -4
SABLE_ERR_TIMEOUT = -5
SABLE_ERR_ARG = -6
MLP_NPARAMS = 4738


class SableError(RuntimeError):
    """A libsable call returned a negative status."""

    def __init__(self, code: int, where: str, detail: str):
        self.code = code
        super().__init__(f"{where}: {detail} (status {code})")


class VbrcDesc(ctypes.Structure):
    _fields_ = [
        ("n_rows", c_int32), ("n_cols", c_int32), ("n_block_rows", c_int32), ("n_block_cols", c_int32),
        ("rpntr", c_void_p), ("cpntr", c_void_p), ("bpntrb", c_void_p), ("bpntre", c_void_p), ("bindx", c_void_p),
        ("n_blocks", c_int64),
        ("val", c_void_p), ("indx", c_void_p), ("n_dense", c_int64),
        ("ublocks", c_void_p), ("n_ublocks", c_int64),
        ("indptr", c_void_p), ("indices", c_void_p), ("csr_val", c_void_p),
    ]


class PlanOpts(ctypes.Structure):
    _fields_ = [("row_tile", c_int32), ("chunk_bytes", c_int32), ("spmm_tc", c_int32), ("device", c_int32),
                ("schedule", c_int32), ("split_layout", c_int32), ("tc_kernel", c_int32)]


class CsrDesc(ctypes.Structure):
    _fields_ = [("n_rows", c_int32), ("n_cols", c_int32), ("indptr", c_void_p), ("indices", c_void_p),
                ("data", c_void_p), ("value_bytes", c_int32), ("nnz", c_int64)]


class PlanStats(ctypes.Structure):
    _fields_ = [
        ("n_tiles", c_int64), ("n_chunks", c_int64), ("dense_values", c_int64), ("dense_padded", c_int64),
        ("sparse_nnz", c_int64), ("device_bytes", c_int64), ("scratch_floats", c_int64),
    ]


class BatchOpts(ctypes.Structure):
    _fields_ = [("ctas_per_sm", c_int32), ("use_graph", c_int32), ("stages", c_int32)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("n_mats", c_int32), ("n_ctas", c_int32), ("n_units", c_int64), ("device_bytes", c_int64),
                ("smem_bytes", c_int32), ("stage_bytes", c_int32), ("stages", c_int32)]


# name -> (restype, argtypes); every symbol of include/sable.h.
SIGNATURES = {
    "sable_plan_create": (c_int, [POINTER(VbrcDesc), POINTER(PlanOpts), POINTER(c_void_p)]),
    "sable_plan_destroy": (c_int, [c_void_p]),
    "sable_plan_get_stats": (c_int, [c_void_p, POINTER(PlanStats)]),
    "sable_plan_dry_run": (c_int, [POINTER(VbrcDesc), POINTER(PlanOpts), POINTER(PlanStats)]),
    "sable_plan_layout_host": (c_int, [POINTER(VbrcDesc), POINTER(PlanOpts), c_void_p, c_int64, POINTER(c_int64),
                                       c_void_p, c_void_p, c_int64, POINTER(c_int64)]),
    "sable_plan_check": (c_int, [c_void_p, c_void_p]),
    "sable_spmv": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "sable_spmv_host": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "sable_spmm": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_void_p]),
    "sable_spmm_host": (c_int, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p]),
    "sable_spmm_noalloc": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_void_p]),
    "sable_spmv_timed": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sable_spmm_timed": (c_int, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p]),
    "sable_plan_chunk_tiles": (c_int, [c_void_p, c_void_p]),
    "sable_batch_create": (c_int, [c_void_p, c_int32, c_void_p, POINTER(BatchOpts), POINTER(c_void_p)]),
    "sable_batch_run": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "sable_batch_check": (c_int, [c_void_p, c_void_p]),
    "sable_batch_get_info": (c_int, [c_void_p, POINTER(BatchInfo)]),
    "sable_batch_destroy": (c_int, [c_void_p]),
    "sable_block_features": (c_int, [POINTER(VbrcDesc), c_int32, c_void_p]),
    "sable_vbr_from_csr": (c_int, [POINTER(CsrDesc), c_int32, c_void_p, c_int32, c_void_p, c_int32,
                                   POINTER(c_void_p)]),
    "sable_vbr_build_sizes": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64)]),
    "sable_vbr_build_copy": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sable_vbr_build_destroy": (c_int, [c_void_p]),
    "sable_similarity_cuts": (c_int, [POINTER(CsrDesc), POINTER(CsrDesc), c_double, c_int32, c_int32, c_void_p,
                                      POINTER(c_int32), c_void_p, POINTER(c_int32)]),
    "sable_mlp_create": (c_int, [POINTER(c_void_p)]),
    "sable_mlp_destroy": (c_int, [c_void_p]),
    "sable_mlp_set_params": (c_int, [c_void_p, c_void_p]),
    "sable_mlp_get_params": (c_int, [c_void_p, c_void_p]),
    "sable_mlp_set_norm": (c_int, [c_void_p, c_void_p, c_void_p]),
    "sable_mlp_infer": (c_int, [c_void_p, c_void_p, c_int32, c_void_p, c_void_p]),
    "sable_mlp_loss_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p]),
    "sable_mlp_train_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_float, c_void_p, c_void_p]),
    "sable_selftest_wait": (c_int, [ctypes.c_int64, c_int32, c_void_p, c_void_p]),
    "sable_strerror": (c_char_p, [c_int]),
    "sable_last_error": (c_char_p, []),
    "sable_version": (c_char_p, []),
}

_lib = None
_lock = threading.Lock()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libsable.so from the in-tree build directory (building it first if needed)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build

        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not path.exists():
            raise RuntimeError(f"libsable.so is not built ({path}); run `python -m sable_gb300.build`")
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int, where: str) -> None:
    if rc != SABLE_OK:
        lib = load()
        detail = lib.sable_last_error().decode() or lib.sable_strerror(rc).decode()
        raise SableError(rc, where, detail)


def ptr(a: np.ndarray | None) -> int | None:
    """Host address of a C-contiguous numpy array (None for None / empty)."""
    if a is None or a.size == 0:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data


def make_desc(m) -> tuple[VbrcDesc, list]:
    """Build a VbrcDesc from a compressed-VBR object (see convert.Compressed);
    returns the descriptor and the list of arrays that must outlive the call."""
    keep = []

    def arr(x, dt):
        if x is None:
            return None
        a = np.ascontiguousarray(np.asarray(x), dtype=dt)
        keep.append(a)
        return a

    rpntr = arr(m.rpntr, np.int32)
    cpntr = arr(m.cpntr, np.int32)
    bpntrb = arr(m.bpntrb, np.int32)
    bpntre = arr(m.bpntre, np.int32)
    bindx = arr(m.bindx, np.int32)
    val = arr(m.val, np.float32)
    indx = arr(m.indx, np.int64)
    ublocks = arr(m.ublocks, np.int32)
    has_csr = m.indptr is not None and len(m.indptr) > 0
    indptr = arr(m.indptr, np.int64) if has_csr else None
    indices = arr(m.indices, np.int32) if has_csr else None
    csr_val = arr(m.csr_val, np.float32) if has_csr else None
    d = VbrcDesc()
    d.n_rows = int(rpntr[-1])
    d.n_cols = int(cpntr[-1])
    d.n_block_rows = len(rpntr) - 1
    d.n_block_cols = len(cpntr) - 1
    d.rpntr, d.cpntr, d.bpntrb, d.bpntre, d.bindx = ptr(rpntr), ptr(cpntr), ptr(bpntrb), ptr(bpntre), ptr(bindx)
    d.n_blocks = len(bindx)
    d.val, d.indx = ptr(val), ptr(indx)
    d.n_dense = len(indx) - 1
    d.ublocks, d.n_ublocks = ptr(ublocks), len(ublocks)
    d.indptr, d.indices, d.csr_val = ptr(indptr), ptr(indices), ptr(csr_val)
    return d, keep
