"""VBR construction and the dense / sparse block split
(reference: utils/convert_real_to_vbr.py).

convert_vbr_to_compressed  utils/convert_real_to_vbr.py:18-96
    For every stored block, density% = nnz / (h*w) * 100 (:39-50).  With a
    `density` threshold the block goes to the CSR part when density% <=
    density (:51-54); otherwise the block model decides (:55-60; the
    reference loads a pickled RandomForest, here any object of
    blockmodel.py).  Dense blocks are re-packed into val2 / indx2; the
    nonzeros of the other blocks form one global CSR with a zero sentinel at
    (m-1, n-1) when that row or column is absent (:70-79), built with the
    same scipy coo -> csr conversion; `ublocks` lists their ordinals.
convert_sparse_to_vbr      utils/convert_real_to_vbr.py:98-199
    Every nonzero (rpntr x cpntr) block is materialised dense, column-major.

The reference walks every element in Python; here each step is a numpy
array operation over all stored values, with the same results.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np
import scipy.sparse

from . import fileio


@dataclass
class Compressed:
    """A matrix in the reference's .vbrc form (see include/sable.h)."""
    val: np.ndarray        # dense blocks only (float32 on the device)
    indx: np.ndarray       # n_dense + 1
    bindx: np.ndarray
    rpntr: np.ndarray
    cpntr: np.ndarray
    bpntrb: np.ndarray
    bpntre: np.ndarray
    ublocks: np.ndarray
    indptr: np.ndarray | None
    indices: np.ndarray | None
    csr_val: np.ndarray | None

    @property
    def n_rows(self) -> int:
        return int(self.rpntr[-1])

    @property
    def n_cols(self) -> int:
        return int(self.cpntr[-1])


@dataclass
class BlockTable:
    """One entry per stored block, in generator order (block row, then
    ascending block column; src/codegen.py:421-435)."""
    row: np.ndarray   # block row a
    col: np.ndarray   # block column b
    h: np.ndarray
    w: np.ndarray
    r0: np.ndarray    # first matrix row
    c0: np.ndarray    # first matrix column
    off: np.ndarray   # offset in val
    size: np.ndarray  # h * w


def validate(rpntr, cpntr, bpntrb, bpntre, bindx) -> None:
    """The structural rules the generator relies on (it numbers blocks by
    block row, then ascending column, and reads values in that order)."""
    rpntr, cpntr = np.asarray(rpntr), np.asarray(cpntr)
    bpntrb, bpntre, bindx = np.asarray(bpntrb), np.asarray(bpntre), np.asarray(bindx)
    if rpntr[0] != 0 or cpntr[0] != 0:
        raise ValueError("rpntr[0] and cpntr[0] must be 0")
    if np.any(np.diff(rpntr) <= 0) or np.any(np.diff(cpntr) <= 0):
        raise ValueError("rpntr / cpntr must be strictly increasing")
    if len(bpntrb) != len(rpntr) - 1 or len(bpntre) != len(rpntr) - 1:
        raise ValueError("bpntrb / bpntre need one entry per block row")
    nxt = 0
    nbc = len(cpntr) - 1
    for a in range(len(bpntrb)):
        b0, b1 = int(bpntrb[a]), int(bpntre[a])
        if b0 == -1:
            continue
        if b0 != nxt or b1 < b0 or b1 > len(bindx):
            raise ValueError(f"block row {a}: range [{b0},{b1}) does not continue at {nxt}")
        seg = bindx[b0:b1]
        if len(seg) and (seg.min() < 0 or seg.max() >= nbc or np.any(np.diff(seg) <= 0)):
            raise ValueError(f"block row {a}: bindx must be ascending block columns")
        nxt = b1
    if nxt != len(bindx):
        raise ValueError("block rows do not cover bindx")


def block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx) -> BlockTable:
    rpntr = np.asarray(rpntr, dtype=np.int64)
    cpntr = np.asarray(cpntr, dtype=np.int64)
    bpntrb = np.asarray(bpntrb, dtype=np.int64)
    bpntre = np.asarray(bpntre, dtype=np.int64)
    bindx = np.asarray(bindx, dtype=np.int64)
    validate(rpntr, cpntr, bpntrb, bpntre, bindx)
    counts = np.where(bpntrb == -1, 0, bpntre - bpntrb)
    row = np.repeat(np.arange(len(bpntrb), dtype=np.int64), counts)
    col = bindx
    h = rpntr[row + 1] - rpntr[row]
    w = cpntr[col + 1] - cpntr[col]
    size = h * w
    off = np.asarray(indx, dtype=np.int64)[: len(bindx)]
    return BlockTable(row, col, h, w, rpntr[row], cpntr[col], off, size)


def block_nnz(val, bt: BlockTable) -> np.ndarray:
    """Nonzeros per block (the reference counts val != 0.0, :39-45)."""
    val = np.asarray(val)
    if len(bt.off) == 0:
        return np.zeros(0, dtype=np.int64)
    nz = (val != 0).astype(np.int64)
    cs = np.concatenate([[0], np.cumsum(nz)])
    return cs[bt.off + bt.size] - cs[bt.off]


def block_density_pct(nnz: np.ndarray, bt: BlockTable) -> np.ndarray:
    """(dense_count / (dense_count + sparse_count)) * 100, as at :50."""
    return (nnz / bt.size) * 100


def block_features(val, bt: BlockTable, N: int = 1) -> np.ndarray:
    """Block-model features (rows, cols, nnz, density, variance of nnz per
    row, N), float32 [n_blocks, 6]; vectorised over all stored values."""
    val = np.asarray(val)
    nb = len(bt.off)
    feats = np.zeros((nb, 6), dtype=np.float32)
    if nb == 0:
        return feats
    nnz = block_nnz(val, bt)
    # per-row nnz: element e of block k is at local row (e - off) % h
    total = int(bt.size.sum())
    blk = np.repeat(np.arange(nb), bt.size)
    local = np.arange(total, dtype=np.int64) - np.repeat(np.cumsum(bt.size) - bt.size, bt.size)
    elem = np.repeat(bt.off, bt.size) + local
    lrow = local % np.repeat(bt.h, bt.size)
    rowbase = np.repeat(np.cumsum(bt.h) - bt.h, bt.size)
    rownnz = np.bincount(rowbase + lrow, weights=(val[elem] != 0).astype(np.float64), minlength=int(bt.h.sum()))
    rb = np.repeat(np.arange(nb), bt.h)
    mean = nnz / bt.h
    var = np.bincount(rb, weights=(rownnz - mean[rb]) ** 2, minlength=nb) / bt.h
    del blk
    feats[:, 0] = bt.h
    feats[:, 1] = bt.w
    feats[:, 2] = nnz
    feats[:, 3] = nnz / bt.size
    feats[:, 4] = var
    feats[:, 5] = N
    return feats


def compress(val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, dense_mask, bt: BlockTable | None = None,
             value_dtype=np.float32) -> Compressed:
    """Split the stored blocks into dense blocks (dense_mask True) and one
    global CSR of the others, as convert_vbr_to_compressed does (:61-83)."""
    val = np.asarray(val)
    if bt is None:
        bt = block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx)
    dense_mask = np.asarray(dense_mask, dtype=bool)
    nb = len(bt.off)
    if len(dense_mask) != nb:
        raise ValueError("dense_mask needs one entry per stored block")
    m, n = int(np.asarray(rpntr)[-1]), int(np.asarray(cpntr)[-1])
    sizes = bt.size
    if nb:
        # values of the dense blocks, in order
        starts = bt.off[dense_mask]
        lens = sizes[dense_mask]
        if len(starts):
            idx = np.repeat(starts - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens) + np.arange(int(lens.sum()))
            val2 = val[idx]
        else:
            val2 = np.zeros(0, dtype=val.dtype)
    else:
        val2 = np.zeros(0, dtype=val.dtype)
    indx2 = np.concatenate([[0], np.cumsum(sizes[dense_mask])]).astype(np.int64)
    ublocks = np.nonzero(~dense_mask)[0].astype(np.int64)
    sp = ~dense_mask
    indptr = indices = csr_val = None
    if sp.any():
        lens = sizes[sp]
        offs = bt.off[sp]
        base = np.repeat(offs - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens)
        local = np.arange(int(lens.sum()), dtype=np.int64) - np.repeat(np.concatenate([[0], np.cumsum(lens)[:-1]]), lens)
        elem = base + np.arange(int(lens.sum()), dtype=np.int64)
        hh = np.repeat(bt.h[sp], lens)
        v = val[elem]
        keep = v != 0.0
        coo_i = (np.repeat(bt.r0[sp], lens) + local % hh)[keep]
        coo_j = (np.repeat(bt.c0[sp], lens) + local // hh)[keep]
        coo_v = v[keep].astype(np.float64)
        if len(coo_i) > 0:
            if not np.any(coo_i == m - 1) or not np.any(coo_j == n - 1):
                coo_i = np.append(coo_i, m - 1)
                coo_j = np.append(coo_j, n - 1)
                coo_v = np.append(coo_v, 0.0)
            csr = scipy.sparse.coo_array((coo_v, (coo_i, coo_j))).tocsr()
            indptr, indices, csr_val = csr.indptr, csr.indices, csr.data
            assert len(indptr) == m + 1
    return Compressed(val=np.asarray(val2, dtype=value_dtype), indx=indx2, bindx=np.asarray(bindx, dtype=np.int64),
                      rpntr=np.asarray(rpntr, dtype=np.int64), cpntr=np.asarray(cpntr, dtype=np.int64),
                      bpntrb=np.asarray(bpntrb, dtype=np.int64), bpntre=np.asarray(bpntre, dtype=np.int64),
                      ublocks=ublocks, indptr=indptr, indices=indices, csr_val=csr_val)


def choose_dense(val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, density=None, model=None, N: int = 1,
                 bt: BlockTable | None = None) -> np.ndarray:
    """Per-block decision: True = keep dense.  With `density`, dense iff
    density% > density (utils/convert_real_to_vbr.py:51-54); otherwise the
    block model decides (:55-60)."""
    if bt is None:
        bt = block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx)
    if density is not None:
        nnz = block_nnz(val, bt)
        return block_density_pct(nnz, bt) > density
    from . import blockmodel
    if model is None:
        model = blockmodel.default_model()
    return np.asarray(model.choose_dense(block_features(val, bt, N)), dtype=bool)


def convert_vbr_to_compressed(val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, fname, dst_dir, density=None,
                              model=None, N: int = 1, write: bool = True, binary: bool = False):
    """utils/convert_real_to_vbr.py:18-96; returns (val2, indx2, bindx,
    bpntrb, bpntre, ublocks, indptr, indices, csr_val) and writes
    <dst_dir>/<fname>.vbrc (unless write=False; binary=True writes the
    binary form <fname>.vbrcb instead)."""
    val = np.asarray(val, dtype=np.float64)
    bt = block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx)
    dense = choose_dense(val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, density=density, model=model, N=N, bt=bt)
    c = compress(val, rpntr, cpntr, indx, bindx, bpntrb, bpntre, dense, bt=bt, value_dtype=np.float64)
    indptr = c.indptr if c.indptr is not None else np.zeros(0, dtype=np.int64)
    indices = c.indices if c.indices is not None else np.zeros(0, dtype=np.int64)
    csr_val = c.csr_val if c.csr_val is not None else np.zeros(0)
    if write:
        writer = fileio.write_vbrc_binary if binary else fileio.write_vbrc
        writer(os.path.join(dst_dir, f"{fname}.vbrc" + ("b" if binary else "")), c.val, csr_val, indptr, indices,
               c.indx, bindx, rpntr, cpntr, bpntrb, bpntre, c.ublocks)
    return c.val, c.indx, np.asarray(bindx), np.asarray(bpntrb), np.asarray(bpntre), c.ublocks, indptr, indices, csr_val


def convert_sparse_to_vbr(mat, rpntr, cpntr, fname, dst_dir, write: bool = True):
    """utils/convert_real_to_vbr.py:98-199: every (rpntr x cpntr) block with
    stored entries is materialised dense, column-major; returns (val, indx,
    bindx, bpntrb, bpntre) and writes <dst_dir>/<fname>.vbr.  A block row
    without stored blocks gets bpntrb = bpntre = -1 (the reference asserts
    that none exists)."""
    A = scipy.sparse.coo_array(mat)
    rpntr = np.asarray(rpntr, dtype=np.int64)
    cpntr = np.asarray(cpntr, dtype=np.int64)
    nbr, nbc = len(rpntr) - 1, len(cpntr) - 1
    br = np.searchsorted(rpntr, A.row, side="right") - 1
    bc = np.searchsorted(cpntr, A.col, side="right") - 1
    key = br.astype(np.int64) * nbc + bc
    blocks = np.unique(key)
    brow, bcol = blocks // nbc, blocks % nbc
    h = rpntr[brow + 1] - rpntr[brow]
    w = cpntr[bcol + 1] - cpntr[bcol]
    size = h * w
    indx = np.concatenate([[0], np.cumsum(size)]).astype(np.int64)
    val = np.zeros(int(indx[-1]), dtype=np.float64)
    k = np.searchsorted(blocks, key)
    pos = indx[k] + (A.col - cpntr[bc]) * h[k] + (A.row - rpntr[br])
    np.add.at(val, pos, A.data.astype(np.float64))
    bindx = bcol.astype(np.int64)
    counts = np.bincount(brow, minlength=nbr)
    ends = np.cumsum(counts)
    bpntrb = np.where(counts > 0, ends - counts, -1).astype(np.int64)
    bpntre = np.where(counts > 0, ends, -1).astype(np.int64)
    if write:
        os.makedirs(dst_dir, exist_ok=True)
        from .vbr import VBR
        fileio.write_vbr_matrix(fname, VBR(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre), dst_dir)
    return val, indx, bindx, bpntrb, bpntre


def vbr_to_dense(val, indx, bindx, rpntr, cpntr, bpntrb, bpntre) -> np.ndarray:
    """Dense materialisation (utils/mtx_matrices_gen.py:29-49)."""
    bt = block_table(rpntr, cpntr, bpntrb, bpntre, bindx, indx)
    M = np.zeros((int(np.asarray(rpntr)[-1]), int(np.asarray(cpntr)[-1])))
    val = np.asarray(val, dtype=np.float64)
    for k in range(len(bt.off)):
        blk = val[bt.off[k]: bt.off[k] + bt.size[k]].reshape(bt.w[k], bt.h[k]).T
        M[bt.r0[k]: bt.r0[k] + bt.h[k], bt.c0[k]: bt.c0[k] + bt.w[k]] = blk
    return M
