"""Build libsable.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

Every translation unit under ``csrc/`` is compiled by nvcc in parallel and
linked into ``sable_gb300/_build/libsable.so``.  Nothing is installed into
site-packages; the Python package loads the library from that path.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
INCLUDE = HERE.parent / "include"
LIB = OUT / "libsable.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsable")


def _sources() -> list[pathlib.Path]:
    return sorted([*CSRC.glob("*.cu"), *CSRC.glob("*.cpp")])


def _fingerprint(srcs: list[pathlib.Path]) -> str:
    h = hashlib.sha256()
    for p in [*srcs, *sorted(CSRC.glob("*.h")), *sorted(CSRC.glob("*.cuh")), *sorted(INCLUDE.glob("*.h")),
              pathlib.Path(__file__)]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> pathlib.Path:
    """Compile libsable.so if any source changed; return its path."""
    srcs = _sources()
    OUT.mkdir(exist_ok=True)
    stamp = OUT / "libsable.stamp"
    fp = _fingerprint(srcs)
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    nvcc = _nvcc()
    incs = [f"-I{INCLUDE}", f"-I{CSRC}"]

    def compile_one(src: pathlib.Path) -> pathlib.Path:
        obj = OUT / (src.name + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *incs, "-c", str(src), "-o", str(obj)]
        if ptxas_verbose and src.suffix == ".cu":
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = OUT / "libsable.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libsable.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(fp)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
