"""ORACLE / CPU baseline — test infrastructure only: the reference's own
generated SpMV executor for the 100000 x 100000 workload, timed on the host.

Only bench.py's reference arm and CPU-baseline leg (and tests) use it; the
product never imports it.

generate(reference_root)  (run where the reference tree is present; build()
    calls it): imports the reference's src/codegen.py from that tree and runs
    its own gen_single_threaded_spmv (src/codegen.py:293-452) and
    gen_multi_threaded_spmv (:454-643, THREADS OpenMP sections, block rows
    split by split_chunks :165-186) on the workload with the reference's
    block choice (its RandomForest), writing the C sources to
    oracle/_ref/spmv_100k/.  The compressed arrays passed to the generators
    come from sable_gb300.convert (identical, array for array, to the
    reference's convert_vbr_to_compressed; tests/test_oracle.py).
    Harness shims, applied to the generated text (each one a plain string
    substitution, listed here):
      - the two input paths (its .vbrc file and its vector file) become
        placeholders, replaced at compile time by the files run() writes
        beside the build;
      - the iteration count `bench` is read at run time from the environment
        variable SABLE_BENCH (at most SABLE_BENCH_MAX; the reference bakes it
        in), so that one compiled program serves every iteration count;
      - y is printed with %.17g instead of %lf / %.2f, so that the result can
        be checked against the FP64 oracle.
compile()  (on any host, the GPU machine included): writes the .vbrc text
    (sable_gb300.fileio.write_vbrc, the reference's format byte for byte) and
    the vector file, and compiles both programs (in parallel; about four
    minutes each at these flags) with the reference's CFLAGS for this host
    (oracle.build.reference_cflags) against the MKL stand-in (a plain CSR
    loop, threaded like MKL's); the executables are kept beside the inputs
    and reused while source, flags and host architecture stay the same.
run(steps)  compiles if needed, runs each program under `ulimit -s
    unlimited` (its arrays live on the stack) and returns the per-iteration
    times it prints (ns) and its y.  Parsing its 660 MB text input takes the
    program about a minute before the timed loop.
"""
from __future__ import annotations

import hashlib
import json
import os
import pathlib
import subprocess
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_ref" / "spmv_100k"
NAME = "spmv_100k"
THREADS = 16            # OpenMP sections of the multi-threaded program (the GPU machine's host cores)
BENCH_MARK = 97531      # iteration count at generation time, replaced by the run-time count
BENCH_MAX = 1000        # largest run-time iteration count


def _workload():
    sys.path.insert(0, str(ROOT))
    from sable_gb300 import blockmodel, convert, synth
    m = synth.spmv_100k()
    x = synth.vector(m.n_cols, 31)
    bt = convert.block_table(m.rpntr, m.cpntr, m.bpntrb, m.bpntre, m.bindx, m.indx)
    choice = blockmodel.RFTableModel().choose_dense(convert.block_features(m.val, bt, 1))
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, choice, bt=bt,
                            value_dtype=np.float64)
    return m, x, comp


def _signature(comp) -> str:
    h = hashlib.sha256()
    for a in (comp.val, comp.indx, comp.bindx, comp.rpntr, comp.cpntr, comp.bpntrb, comp.bpntre, comp.ublocks):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(f"{THREADS}/{BENCH_MARK}".encode())
    return h.hexdigest()


def generated() -> bool:
    """True when the generated sources for the current workload are present."""
    meta = OUT / "meta.json"
    return meta.exists() and (OUT / "st.c").exists() and (OUT / "mt.c").exists()


def _shim(text: str, vbrc_path: str, vector_path: str) -> str:
    """The harness substitutions listed in the module docstring."""
    # input paths: the generated program fopen()s absolute paths
    lines = text.split("\n")
    for i, ln in enumerate(lines):
        if "FILE *file1 = fopen(" in ln:
            lines[i] = f'\tFILE *file1 = fopen("{vbrc_path}", "r");'
        elif "FILE *file2 = fopen(" in ln:
            lines[i] = f'\tFILE *file2 = fopen("{vector_path}", "r");'
    text = "\n".join(lines)
    # iteration count, read at run time
    text = text.replace(f"long times[{BENCH_MARK}]", f"long times[{BENCH_MAX}]")
    text = text.replace(f"i<{BENCH_MARK + 1};", "i<sable_bench+1;").replace(f"i<{BENCH_MARK};", "i<sable_bench;")
    text = ("#include <stdlib.h>\nstatic int sable_bench = 1;\n"
            "__attribute__((constructor)) static void sable_read_bench(void) {\n"
            "\tconst char *s = getenv(\"SABLE_BENCH\");\n"
            f"\tsable_bench = s ? atoi(s) : 1;\n\tif (sable_bench < 1) sable_bench = 1;\n"
            f"\tif (sable_bench > {BENCH_MAX}) sable_bench = {BENCH_MAX};\n}}\n") + text
    # full-precision y
    text = text.replace('printf("%lf\\n", y[i])', 'printf("%.17g\\n", y[i])')
    text = text.replace('printf("%.2f\\n", y[i])', 'printf("%.17g\\n", y[i])')
    return text


def generate(reference_root: str | os.PathLike) -> None:
    """Run the reference's generators (see module docstring); writes
    oracle/_ref/spmv_100k/{st,mt}.c and meta.json.  Skipped when present for
    the same workload."""
    m, x, comp = _workload()
    sig = _signature(comp)
    meta = OUT / "meta.json"
    if generated() and json.loads(meta.read_text()).get("signature") == sig:
        return
    OUT.mkdir(parents=True, exist_ok=True)
    sys.dont_write_bytecode = True
    sys.path.insert(0, str(pathlib.Path(reference_root).resolve()))
    cg = __import__("src.codegen", fromlist=["gen_single_threaded_spmv"])
    args = [comp.val.tolist(), comp.indx.tolist(), comp.bindx.tolist(), comp.rpntr.tolist(), comp.cpntr.tolist(),
            comp.bpntrb.tolist(), comp.bpntre.tolist(), comp.ublocks.tolist(),
            comp.indptr.tolist() if comp.indptr is not None else [],
            comp.indices.tolist() if comp.indices is not None else [],
            comp.csr_val.tolist() if comp.csr_val is not None else []]
    tmp = OUT / "gen"
    tmp.mkdir(exist_ok=True)
    cg.gen_single_threaded_spmv(*args, str(tmp), "st", str(OUT), bench=BENCH_MARK)
    cg.gen_multi_threaded_spmv(THREADS, *args, str(tmp), "mt", str(OUT), bench=BENCH_MARK)
    for kind in ("st", "mt"):
        (OUT / f"{kind}.c").write_text(_shim((tmp / f"{kind}.c").read_text(), "@VBRC_PATH@", "@VECTOR_PATH@"))
        (tmp / f"{kind}.c").unlink()
    tmp.rmdir()
    meta.write_text(json.dumps({"signature": sig, "threads": THREADS, "n_blocks": int(len(comp.bindx)),
                                "dense_blocks": int(len(comp.indx) - 1), "csr_nnz": int(len(comp.csr_val))
                                if comp.csr_val is not None else 0}))


def _cflags() -> list:
    from oracle import build as ob
    return [*ob.reference_cflags(), f"-I{HERE / 'mkl_standin'}", f"-L{ob.OUT}", "-lmkl_rt", f"-Wl,-rpath,{ob.OUT}"]


def compiled(kinds=("st", "mt")) -> bool:
    """True when executables for the current sources, flags and host are present."""
    work = OUT / "run"
    for kind in kinds:
        sig = work / f"{kind}.sig"
        if not ((work / kind).exists() and sig.exists() and sig.read_text() == _exe_signature(kind)):
            return False
    return True


def _exe_signature(kind: str) -> str:
    import platform
    h = hashlib.sha256()
    h.update((OUT / f"{kind}.c").read_bytes() if (OUT / f"{kind}.c").exists() else b"")
    h.update(" ".join(_cflags()).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def compile(kinds=("st", "mt")) -> None:
    """Write the inputs and compile the programs (see module docstring)."""
    from oracle import build as ob
    from sable_gb300 import fileio
    if not generated():
        raise FileNotFoundError("the reference's generated C is not present (oracle/_ref/spmv_100k)")
    m, x, comp = _workload()
    meta = json.loads((OUT / "meta.json").read_text())
    if meta["signature"] != _signature(comp):
        raise RuntimeError("oracle/_ref/spmv_100k was generated for another workload")
    ob.build()
    work = OUT / "run"
    work.mkdir(exist_ok=True)
    vbrc, vec = work / f"{NAME}.vbrc", work / "x.vector"
    stamp = work / "inputs.sig"
    if not (vbrc.exists() and vec.exists() and stamp.exists() and stamp.read_text() == meta["signature"]):
        empty = np.zeros(0)
        fileio.write_vbrc(str(vbrc), comp.val, comp.csr_val if comp.csr_val is not None else empty,
                          comp.indptr if comp.indptr is not None else empty,
                          comp.indices if comp.indices is not None else empty, comp.indx, comp.bindx, comp.rpntr,
                          comp.cpntr, comp.bpntrb, comp.bpntre, comp.ublocks)
        fileio.write_vector_values(np.asarray(x, np.float64), str(vec))
        stamp.write_text(meta["signature"])
    procs = {}
    for kind in kinds:
        if compiled((kind,)):
            continue
        src = work / f"{kind}.c"
        src.write_text((OUT / f"{kind}.c").read_text().replace("@VBRC_PATH@", str(vbrc))
                       .replace("@VECTOR_PATH@", str(vec)))
        procs[kind] = subprocess.Popen(["gcc", "-o", str(work / kind), str(src), *_cflags()], stdout=subprocess.PIPE,
                                       stderr=subprocess.PIPE, text=True)
    for kind, pr in procs.items():
        _, err = pr.communicate()
        if pr.returncode:
            raise RuntimeError(f"gcc failed on the generated {kind}.c:\n{err[-2000:]}")
        (work / f"{kind}.sig").write_text(_exe_signature(kind))


def run(steps: int, kinds=("st", "mt"), timeout: float = 900.0) -> dict:
    """Run the generated programs for `steps` timed iterations each (after the
    reference's own dropped first iteration), compiling them first if needed.
    Returns {kind: {"times_ns": [...], "y": array, "threads": n}}."""
    compile(kinds)
    meta = json.loads((OUT / "meta.json").read_text())
    work = OUT / "run"
    out = {}
    for kind in kinds:
        env = dict(os.environ, SABLE_BENCH=str(int(steps)))
        r = subprocess.run(["bash", "-c", f"ulimit -s unlimited; exec {work / kind}"], capture_output=True,
                           text=True, timeout=timeout, env=env)
        if r.returncode:
            raise RuntimeError(f"generated {kind} program exited {r.returncode}: {r.stdout[:200]} {r.stderr[-500:]}")
        lines = r.stdout.split("\n")
        times = [int(t) for t in lines[0].split("=", 1)[1].strip().rstrip(",").split(",") if t]
        y = np.array([float(v) for v in lines[1:] if v.strip()], dtype=np.float64)
        out[kind] = {"times_ns": times, "y": y, "threads": 1 if kind == "st" else meta["threads"]}
    return out
