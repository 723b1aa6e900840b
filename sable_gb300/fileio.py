"""Text formats of the reference, plus a binary form (reference: utils/fileio.py).

``.vbr``  seven lines ``name=[v0,v1,...]`` (val, indx, bindx, rpntr, cpntr,
          bpntrb, bpntre), written by write_vbr_matrix (utils/fileio.py:13-35)
          and read by read_vbr (:55-64).
``.vbrc`` eleven lines (val, csr_val, indptr, indices, indx, bindx, rpntr,
          cpntr, bpntrb, bpntre, ublocks), written by
          convert_vbr_to_compressed (utils/convert_real_to_vbr.py:84-95) and
          read by read_vbrc (utils/fileio.py:66-93).
Dense operands: ``Generated_dense_tensors/generated_vector_{n}.vector`` and
``generated_matrix_{m}x{n}.matrix`` under the base path, comma-separated
(utils/fileio.py:37-53).

Values are written with Python's ``str`` of each element, as the reference
does, so the files are byte-identical for identical inputs.  Readers return
numpy arrays (float64 values, int64 indices) instead of lists; parsing is
vectorised.  ``.vbrb`` and ``.vbrcb`` are binary (npz) forms of ``.vbr`` and
``.vbrc`` for large matrices, where text parsing dominates end-to-end time;
read_vbr / read_vbrc accept them, and the *_codegen entry points read the
binary form when the text file is absent (source_path).
"""
from __future__ import annotations

import os
from os.path import exists, join

import numpy as np

from .vbr import VBR

VBR_FIELDS = ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre")
VBRC_FIELDS = ("val", "csr_val", "indptr", "indices", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre", "ublocks")


def base_path() -> str:
    """Directory that holds Generated_dense_tensors/ (the reference uses its repo root)."""
    return os.environ.get("SABLE_BASE_PATH", os.getcwd())


def _fmt(a) -> str:
    if isinstance(a, np.ndarray):
        a = a.tolist()
    return ",".join(map(str, a))


def _parse_line(line: str, dtype) -> np.ndarray:
    body = line.split("=", 1)[1].strip()
    if not (body.startswith("[") and body.endswith("]")):
        raise ValueError(f"malformed line: {line[:60]!r}")
    body = body[1:-1]
    if body == "":
        return np.zeros(0, dtype=dtype)
    if dtype == np.float64:
        out = np.array(body.split(","), dtype=np.float64)
    else:
        out = np.array(body.split(","), dtype=np.int64)
    return out


def write_vbr_matrix(filename: str, vbr_matrix: VBR, dir_name: str) -> None:
    """utils/fileio.py:13-35."""
    assert isinstance(vbr_matrix, VBR)
    assert isinstance(filename, str)
    if not exists(dir_name):
        os.makedirs(dir_name)
    with open(join(dir_name, filename + ".vbr"), "w") as f:
        for name, arr in zip(VBR_FIELDS, vbr_matrix.arrays()):
            f.write(f"{name}=[{_fmt(arr)}]\n")


def write_vbrc(path: str, val2, csr_val, indptr, indices, indx2, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks) -> None:
    """The .vbrc writer of convert_vbr_to_compressed (utils/convert_real_to_vbr.py:84-95)."""
    with open(path, "w") as f:
        for name, arr in zip(VBRC_FIELDS, (val2, csr_val, indptr, indices, indx2, bindx, rpntr, cpntr, bpntrb, bpntre, ublocks)):
            f.write(f"{name}=[{_fmt(arr)}]\n")


def write_dense_vector(val: float, size: int) -> str:
    """utils/fileio.py:37-44; returns the path written."""
    dir_name = join(base_path(), "Generated_dense_tensors")
    os.makedirs(dir_name, exist_ok=True)
    path = join(dir_name, f"generated_vector_{size}.vector")
    with open(path, "w") as f:
        f.write(",".join([str(val)] * size) + "\n")
    return path


def write_dense_matrix(val: float, m: int, n: int) -> str:
    """utils/fileio.py:46-53; returns the path written."""
    dir_name = join(base_path(), "Generated_dense_tensors")
    os.makedirs(dir_name, exist_ok=True)
    path = join(dir_name, f"generated_matrix_{m}x{n}.matrix")
    with open(path, "w") as f:
        f.write(",".join([str(val)] * (n * m)) + "\n")
    return path


def write_vector_values(x, path: str) -> None:
    """Dense operand file with arbitrary values, in the same comma format."""
    with open(path, "w") as f:
        f.write(_fmt(np.asarray(x, dtype=np.float64)) + "\n")


def read_dense_values(path: str) -> np.ndarray:
    """Read a generated_vector / generated_matrix file (comma separated,
    optionally ``name=[...]``), as the generated C reads it with "%lf,"."""
    with open(path) as f:
        text = f.read().strip()
    if "=" in text:
        text = text.split("=", 1)[1].strip()[1:-1]
    text = text.rstrip(",")
    if not text:
        return np.zeros(0)
    return np.array(text.split(","), dtype=np.float64)


def source_path(dir_name: str, filename: str, ext: str) -> str:
    """Path of matrix `filename` in `dir_name` with text suffix `ext` (".vbr"
    or ".vbrc"): the text file when it exists, else its binary form (".vbrb" /
    ".vbrcb") when that exists, else the text path (so that a missing matrix
    is reported under the reference's file name)."""
    text = join(dir_name, filename + ext)
    if exists(text):
        return text
    binary = text + "b"
    return binary if exists(binary) else text


def write_vbr_binary(filename: str, vbr_matrix: VBR, dir_name: str) -> str:
    """Binary counterpart of write_vbr_matrix: <dir_name>/<filename>.vbrb."""
    os.makedirs(dir_name, exist_ok=True)
    path = join(dir_name, filename + ".vbrb")
    write_binary(path, **dict(zip(VBR_FIELDS, vbr_matrix.arrays())))
    return path


def write_vbrc_binary(path: str, val2, csr_val, indptr, indices, indx2, bindx, rpntr, cpntr, bpntrb, bpntre,
                      ublocks) -> None:
    """Binary counterpart of write_vbrc (argument order of the .vbrc lines);
    `path` ends in .vbrcb."""
    write_binary(path, **dict(zip(VBRC_FIELDS, (val2, csr_val, indptr, indices, indx2, bindx, rpntr, cpntr, bpntrb,
                                                bpntre, ublocks))))


def read_vbr(filename: str):
    """utils/fileio.py:55-64 -> (val, indx, bindx, rpntr, cpntr, bpntrb, bpntre)."""
    if filename.endswith(".vbrb") or filename.endswith(".vbrcb"):
        with np.load(filename) as z:
            if "ublocks" in z:
                raise ValueError(f"{filename}: holds a compressed (.vbrc) matrix; read it with read_vbrc")
        return read_binary(filename, VBR_FIELDS)
    with open(filename) as f:
        val = _parse_line(f.readline(), np.float64)
        rest = [_parse_line(f.readline(), np.int64) for _ in range(6)]
    return (val, *rest)


def read_vbrc(filename: str):
    """utils/fileio.py:66-93 -> (val, indx, bindx, rpntr, cpntr, bpntrb,
    bpntre, ublocks, indptr, indices, csr_val)."""
    if filename.endswith(".vbrcb") or filename.endswith(".vbrb"):
        with np.load(filename) as z:
            if "ublocks" not in z:
                raise ValueError(f"{filename}: holds an uncompressed (.vbr) matrix; read it with read_vbr")
        d = read_binary(filename, VBRC_FIELDS)
        got = dict(zip(VBRC_FIELDS, d))
    else:
        with open(filename) as f:
            got = {}
            for name in VBRC_FIELDS:
                line = f.readline()
                key = line.split("=", 1)[0]
                if key != name:
                    raise ValueError(f"{filename}: expected {name}=, found {key}=")
                got[name] = _parse_line(line, np.float64 if name in ("val", "csr_val") else np.int64)
    return (got["val"], got["indx"], got["bindx"], got["rpntr"], got["cpntr"], got["bpntrb"], got["bpntre"],
            got["ublocks"], got["indptr"], got["indices"], got["csr_val"])


def read_vector(filename: str) -> np.ndarray:
    """utils/fileio.py:95-98 (``x=[...]`` form); also accepts the bare comma form."""
    return read_dense_values(filename)


def read_matrix(filename: str) -> np.ndarray:
    """utils/fileio.py:100-103."""
    return read_dense_values(filename)


def write_mm_file(filename: str, M) -> None:
    """utils/fileio.py:105-112: dense matrix -> MatrixMarket coordinate file."""
    M = np.asarray(M)
    rows, cols = np.nonzero(M)
    with open(filename, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{M.shape[0]} {M.shape[1]} {len(rows)}\n")
        for i, j in zip(rows.tolist(), cols.tolist()):
            f.write(f"{i + 1} {j + 1} {M[i][j]}\n")


def write_binary(path: str, **arrays) -> None:
    """Binary (.vbrb, npz) form of a .vbr / .vbrc file: fields by name."""
    with open(path, "wb") as f:
        np.savez(f, **{k: np.asarray(v) for k, v in arrays.items()})


def read_binary(path: str, fields):
    with np.load(path) as z:
        return tuple(np.array(z[name]) if name in z else np.zeros(0) for name in fields)
