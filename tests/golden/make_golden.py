"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run in a container that holds the reference tree (read-only), naming its root
as the argument or in SABLE_REFERENCE_ROOT:

    python tests/golden/make_golden.py <reference root>

Steps (harness shims only, all inside a scratch copy in a temporary
directory):
  1. copy the reference tree to the scratch directory;
  2. stub `numba` (only `njit` is used, src/autopartition.py:76) so that the
     reference's test module imports;
  3. build the MKL stand-in of oracle/mkl_standin (plain CSR loop behind
     mkl_sparse_d_create_csr / mkl_sparse_d_mv / mkl_set_num_threads) and
     point the scratch src/consts.py MKL_PATH at it;
  4. in the scratch src/codegen.py replace the SpMM width literal 512 by a
     module global SPMM_N, and prepend `#define SPMM_N <N>` to generated C;
  5. rewrite the printf formats of the generated C to %.17g (FP64) / %.9g
     (FP32) so that every printed value round-trips;
  6. run the reference's own generator (vbr_spmv_codegen, vbr_spmm_codegen,
     convert_vbr_to_compressed, and its test functions for the example
     matrices), compile the generated C with the reference CFLAGS
     (src/consts.py:6) and run it under `ulimit -s unlimited`;
  7. run the reference's synthetic matrix generator (vbr_matrix_gen,
     synthesize_matrices/vbr_matrices_gen.py:36-113) after random.seed(s)
     and store the arrays of the .vbr file it writes;
  8. run the reference's partitioning steps, cut_indices2 with similarity2
     and with similarity2_numba (src/autopartition.py:34-107) and
     convert_sparse_to_vbr (utils/convert_real_to_vbr.py:98-199), on the
     seeded matrices of synth.PARTITION_CASES, and cut_indices2 on the
     MatrixMarket files of its manual_mtx/ directory (stored: the cuts, the
     VBR index arrays and a sha256 of each file, not the matrices).
The fixtures store the reference's inputs (or the seeds that regenerate
them, with a sha256 of the arrays) and its outputs.

    python tests/golden/make_golden.py --generator-only <reference root>
    python tests/golden/make_golden.py --partition-only <reference root>

add (or refresh) only the cases of step 7 / step 8 in the existing fixture
files.
"""
from __future__ import annotations

import hashlib
import importlib
import json
import os
import pathlib
import re
import shutil
import subprocess
import sys
import tempfile
import types

import numpy as np

REPO = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
OUT = pathlib.Path(__file__).resolve().parent
SCRATCH = None   # the scratch copy of the reference (prepare)


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(np.asarray(a))
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def reference_root(argv_root=None) -> pathlib.Path:
    root = argv_root or os.environ.get("SABLE_REFERENCE_ROOT")
    if not root:
        sys.exit("name the reference root as the argument or in SABLE_REFERENCE_ROOT")
    return pathlib.Path(root)


def prepare(ref_root: pathlib.Path):
    global SCRATCH
    SCRATCH = pathlib.Path(tempfile.mkdtemp(prefix="sable_ref_golden_")) / "ref"
    shutil.copytree(ref_root, SCRATCH, ignore=shutil.ignore_patterns(".git"))
    for p in SCRATCH.rglob("*"):
        try:
            p.chmod(p.stat().st_mode | 0o200)
        except OSError:
            pass
    # MKL stand-in
    from oracle import build as ob
    ob.build()
    mkl = SCRATCH / "_mkl"
    (mkl / "include").mkdir(parents=True)
    (mkl / "lib" / "intel64").mkdir(parents=True)
    for h in ("mkl.h", "mkl_spblas.h"):
        shutil.copy(REPO / "oracle" / "mkl_standin" / h, mkl / "include" / h)
    shutil.copy(ob.MKL_STANDIN, mkl / "lib" / "intel64" / "libmkl_rt.so")
    consts = SCRATCH / "src" / "consts.py"
    txt = consts.read_text()
    txt = re.sub(r'MKL_PATH = .*', f'MKL_PATH = "{mkl}"', txt)
    consts.write_text(txt)
    # SpMM width
    cg = SCRATCH / "src" / "codegen.py"
    src = cg.read_text()
    src = re.sub(r"\b512\b", "SPMM_N", src)
    src = src.replace("curr_block_instructions = []\n", "curr_block_instructions = []\nSPMM_N = 512\n", 1)
    cg.write_text(src)
    # numba stub
    stub = types.ModuleType("numba")
    stub.njit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    sys.modules["numba"] = stub
    sys.path.insert(0, str(SCRATCH))
    os.chdir(SCRATCH)


def run_c(c_path: pathlib.Path, fp64: bool, spmm_n: int | None = None) -> list[str]:
    consts = importlib.import_module("src.consts")
    text = c_path.read_text()
    text = text.replace('printf("%lf\\n"', 'printf("%.17g\\n"').replace('printf("%.2f\\n"', 'printf("%.17g\\n"')
    text = text.replace('printf("%f\\n"', 'printf("%.9g\\n"')
    if spmm_n is not None:
        text = f"#define SPMM_N {spmm_n}\n" + text
    c_path.write_text(text)
    exe = c_path.with_suffix("")
    cmd = ["gcc", "-o", str(exe), str(c_path)] + consts.CFLAGS + consts.MKL_FLAGS
    subprocess.check_call(cmd, cwd=c_path.parent)
    env = dict(os.environ, LD_LIBRARY_PATH=str(SCRATCH / "_mkl" / "lib" / "intel64"))
    out = subprocess.check_output(["bash", "-c", f"ulimit -s unlimited; {exe}"], cwd=c_path.parent, env=env)
    return out.decode().split("\n")


def write_vector_file(x):
    d = SCRATCH / "Generated_dense_tensors"
    d.mkdir(exist_ok=True)
    (d / f"generated_vector_{len(x)}.vector").write_text(",".join(map(str, np.asarray(x, np.float64).tolist())) + "\n")


def write_matrix_file(X):
    d = SCRATCH / "Generated_dense_tensors"
    d.mkdir(exist_ok=True)
    (d / f"generated_matrix_{X.shape[0]}x512.matrix").write_text(
        ",".join(map(str, np.asarray(X, np.float64).ravel().tolist())) + "\n")


def spmv_case(name, arrays, x, density, threads, fixtures, meta):
    conv = importlib.import_module("utils.convert_real_to_vbr")
    cg = importlib.import_module("src.codegen")
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = arrays
    vdir = SCRATCH / "golden_vbr"
    vdir.mkdir(exist_ok=True)
    res = conv.convert_vbr_to_compressed(list(map(float, val)), list(map(int, rpntr)), list(map(int, cpntr)),
                                         list(map(int, indx)), list(map(int, bindx)), list(map(int, bpntrb)),
                                         list(map(int, bpntre)), name, str(vdir), density)
    write_vector_file(x)
    cdir = SCRATCH / "golden_c"
    cg.vbr_spmv_codegen(name, str(cdir), str(vdir), threads, bench=3)
    lines = run_c(cdir / f"{name}.c", fp64=True)
    y = np.array([float(s) for s in lines[1:] if s.strip()], dtype=np.float64)
    val2, indx2, _, _, _, ublocks, indptr, indices, csr_val = res
    fixtures[name] = {
        "kind": "spmv", "density": density, "threads": threads, **meta,
        "y": y, "ublocks": np.asarray(ublocks, np.int64), "indx2": np.asarray(indx2, np.int64),
        "indptr": np.asarray(indptr, np.int64), "indices": np.asarray(indices, np.int64),
        "csr_val": np.asarray(csr_val, np.float64), "val2_sha": sha(np.asarray(val2, np.float64)),
    }


def spmm_case(name, arrays, X, density, fixtures, meta):
    cg = importlib.import_module("src.codegen")
    fio = importlib.import_module("utils.fileio")
    vbrmod = importlib.import_module("src.vbr")
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = arrays
    vdir = SCRATCH / "golden_vbr"
    vdir.mkdir(exist_ok=True)
    fio.write_vbr_matrix(name, vbrmod.VBR(list(map(float, val)), list(map(int, indx)), list(map(int, bindx)),
                                          list(map(int, rpntr)), list(map(int, cpntr)), list(map(int, bpntrb)),
                                          list(map(int, bpntre))), str(vdir))
    N = X.shape[1]
    cg.SPMM_N = N
    write_matrix_file(X)
    cdir = SCRATCH / "golden_c"
    v, ix, bi, rp, cp, bb, be = fio.read_vbr(str(vdir / f"{name}.vbr"))
    cg.gen_single_threaded_spmm(v, ix, bi, rp, cp, bb, be, density, str(cdir), name, str(vdir))
    lines = run_c(cdir / f"{name}.c", fp64=False, spmm_n=N)
    Y = np.array([float(s) for s in lines[1:] if s.strip()], dtype=np.float64).reshape(-1, N)
    fixtures[name] = {"kind": "spmm", "density": density, "N": N, **meta, "Y": Y}


# vbr_matrix_gen cases: (seed, m, n, partitioning, row_split, col_split, num_dense,
# perc_dense_zeros, num_sparse, dense_blocks_only)
GEN_CASES = [
    (11, 60, 60, "uniform", 6, 5, 8, 20, 6, False),
    (12, 60, 60, "nonuniform", 6, 5, 8, 20, 0, False),   # random partitions: sparse blocks may hold < 10 entries
    (13, 120, 90, "nonuniform", 8, 6, 12, 0, 0, True),
    (14, 120, 90, "uniform", 4, 6, 3, 50, 9, False),
]


def generator_cases(fixtures):
    """Step 7: the reference generator's matrices for GEN_CASES."""
    import random
    gen = importlib.import_module("synthesize_matrices.vbr_matrices_gen")
    fio = importlib.import_module("utils.fileio")
    out_dir = SCRATCH / "_gen"
    for case in GEN_CASES:
        seed, args = case[0], case[1:]
        random.seed(seed)
        name = gen.vbr_matrix_gen(*args, vbr_dir=str(out_dir))
        sub = out_dir if args[-1] else pathlib.Path(str(out_dir) + "_Sparse")
        arrays = fio.read_vbr(str(sub / (name + ".vbr")))
        fixtures[f"vbrgen_{seed}"] = {"kind": "arrays", "seed": seed, "args": list(args), "name": name,
                                      **{k: np.asarray(v) for k, v in zip(
                                          ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre"), arrays)}}


def write(fixtures):
    index = {}
    arrays_out = {}
    for name, f in fixtures.items():
        index[name] = {k: v for k, v in f.items() if not isinstance(v, np.ndarray)}
        for k, v in f.items():
            if isinstance(v, np.ndarray):
                arrays_out[f"{name}__{k}"] = v
    np.savez_compressed(OUT / "golden.npz", **arrays_out)
    (OUT / "golden.json").write_text(json.dumps(index, indent=1, default=str))
    print("wrote", OUT / "golden.npz", "cases:", ", ".join(fixtures))


def partition_cases(fixtures, ref_root: pathlib.Path):
    """Step 8: the reference's partitioning steps on the seeded partition
    matrices and on its manual_mtx files."""
    import scipy.io
    import scipy.sparse
    from sable_gb300 import synth
    ap = importlib.import_module("src.autopartition")
    conv = importlib.import_module("utils.convert_real_to_vbr")
    out_dir = SCRATCH / "_part"
    out_dir.mkdir(exist_ok=True)

    def run(name, A, meta, store_val):
        csc = scipy.sparse.csc_matrix(A)
        col, row = ap.cut_indices2(csc, 0.2, ap.similarity2)
        col_n, row_n = ap.cut_indices2(csc, 0.2, ap.similarity2_numba)
        f = {"kind": "partition", **meta, "col": np.asarray(col, np.int64), "row": np.asarray(row, np.int64),
             "col_numba": np.asarray(col_n, np.int64), "row_numba": np.asarray(row_n, np.int64)}
        try:
            val, indx, bindx, bpntrb, bpntre = conv.convert_sparse_to_vbr(csc, row, col, name, str(out_dir))
            f.update(vbr_ok=True, val_sha=sha(np.asarray(val, np.float64)), indx=np.asarray(indx, np.int64),
                     bindx=np.asarray(bindx, np.int64), bpntrb=np.asarray(bpntrb, np.int64),
                     bpntre=np.asarray(bpntre, np.int64))
            if store_val:
                f["val"] = np.asarray(val, np.float64)
        except AssertionError:
            f["vbr_ok"] = False   # a block row without stored blocks: the reference asserts
        fixtures[name] = f

    for case in synth.PARTITION_CASES:
        A = synth.partition_case(*case)
        run(f"part_{case[0]}", A, {"case": list(case), "sha": sha(A.indptr, A.indices, A.data)}, True)
    for path in sorted((ref_root / "manual_mtx").glob("*.mtx")):
        data = path.read_bytes()
        A = scipy.io.mmread(str(path))
        run(f"mtx_{path.stem}", A, {"file": f"manual_mtx/{path.name}",
                                    "file_sha": hashlib.sha256(data).hexdigest()}, False)


def _load_existing(drop_prefix):
    index = json.loads((OUT / "golden.json").read_text())
    with np.load(OUT / "golden.npz") as z:
        stored = {k: z[k] for k in z.files}
    fixtures = {name: dict(meta) for name, meta in index.items() if not name.startswith(drop_prefix)}
    for key, v in stored.items():
        name, field = key.split("__", 1)
        if name in fixtures:
            fixtures[name][field] = v
    return fixtures


def generator_only(ref_root=None):
    """Refresh only the step-7 cases in the existing fixture files."""
    fixtures = _load_existing("vbrgen_")
    prepare(reference_root(ref_root))
    generator_cases(fixtures)
    write(fixtures)


def partition_only(ref_root=None):
    """Refresh only the step-8 cases in the existing fixture files."""
    root = reference_root(ref_root)
    fixtures = {k: v for k, v in _load_existing("part_").items() if not k.startswith("mtx_")}
    prepare(root)
    partition_cases(fixtures, root)
    write(fixtures)


def main(ref_root=None):
    ref_root = reference_root(ref_root)
    from sable_gb300 import synth
    prepare(ref_root)
    fixtures = {}

    # (1) the reference's own example and its canonical outputs
    fio = importlib.import_module("utils.fileio")
    ex = fio.read_vbr(str(SCRATCH / "tests" / "example.vbr"))
    canon_spmv = np.loadtxt(SCRATCH / "tests" / "output_spmv_canon.txt")
    canon_sparse = np.loadtxt(SCRATCH / "tests" / "output_spmv_canon_sparse.txt")
    canon_spmm = np.loadtxt(SCRATCH / "tests" / "output_spmm_canon.txt")
    fixtures["example_arrays"] = {"kind": "arrays", **{k: np.asarray(v) for k, v in zip(
        ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre"), ex)}}
    fixtures["example_canon"] = {"kind": "canon", "spmv": canon_spmv, "spmv_sparse": canon_sparse,
                                 "spmm_rows": canon_spmm.reshape(11, 512)[:, 0],
                                 "spmm_rows_constant": bool(np.all(canon_spmm.reshape(11, 512) ==
                                                                   canon_spmm.reshape(11, 512)[:, :1]))}
    # the reference test that builds example2 (density 80) and its outputs
    test = importlib.import_module("test")
    test.test_compression()
    ex2 = fio.read_vbr(str(SCRATCH / "tests" / "example2.vbr"))
    ex2c = fio.read_vbrc(str(SCRATCH / "tests" / "example2.vbrc"))
    fixtures["example2_arrays"] = {"kind": "arrays", **{k: np.asarray(v) for k, v in zip(
        ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre"), ex2)}}
    fixtures["example2_vbrc"] = {"kind": "arrays", **{k: np.asarray(v) for k, v in zip(
        ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre", "ublocks", "indptr", "indices", "csr_val"),
        ex2c)}}
    ones11 = np.ones(11)
    spmv_case("example_d0", ex, ones11, 0, 1, fixtures, {"source": "tests/example.vbr"})
    spmv_case("example2_d80", ex2, ones11, 80, 1, fixtures, {"source": "tests/example2.vbr"})
    spmm_case("example_spmm512", ex, np.ones((11, 512)), 0, fixtures, {"source": "tests/example.vbr"})

    # (2) seeded synthetic cases, random x
    m = synth.spmv_1000()
    x = synth.vector(m.n_cols, 2000)
    meta = {"workload": "spmv_1000", "seed": 1000, "x_seed": 2000, "sha": sha(*m.arrays(), x)}
    arrays = (m.val.astype(np.float64), *m.arrays()[1:])
    spmv_case("spmv1000_d0", arrays, x, 0, 1, fixtures, meta)
    spmv_case("spmv1000_d50", arrays, x, 50, 1, fixtures, meta)
    spmv_case("spmv1000_rf", arrays, x, None, 1, fixtures, meta)
    if int(np.diff(m.rpntr).min()) > 1 and int(np.diff(m.cpntr).min()) > 1:
        spmv_case("spmv1000_d0_t4", arrays, x, 0, 4, fixtures, meta)

    s = synth.spmm_50k(seed=1010, n=400, parts=10, p=0.3)
    for N, dens, xs in ((32, 0, 2010), (8, 30, 2011)):
        X = synth.dense_operand(s.n_cols, N, xs)
        meta = {"workload": "spmm_50k", "seed": 1010, "n": 400, "parts": 10, "p": 0.3, "x_seed": xs,
                "sha": sha(*s.arrays(), X)}
        spmm_case(f"spmm400_N{N}_d{dens}", (s.val.astype(np.float64), *s.arrays()[1:]), X, dens, fixtures, meta)

    generator_cases(fixtures)
    partition_cases(fixtures, ref_root)
    write(fixtures)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--generator-only"]:
        generator_only(*sys.argv[2:])
    elif sys.argv[1:2] == ["--partition-only"]:
        partition_only(*sys.argv[2:])
    else:
        main(*sys.argv[1:])
