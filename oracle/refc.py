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

The reference's generated SpMM for the 50000 x 50000 SpMM workload, at the
widths N = 32 and 128 (oracle/_ref/spmm_50k/n<N>/):
generate_spmm(reference_root)  runs the reference's own
    gen_multi_threaded_spmm (src/codegen.py:939-1075: THREADS pthreads, block
    rows split by split_chunks) with density 0, the setting its own benchmark
    passes (bench.py:66-91: every block runs as a dense loop nest).  Its SpMM
    width is the literal 512 throughout the generator; the generator's source
    is loaded as a private module with that literal replaced by the name
    SPMM_N, set to N (the recipe tests/golden/make_golden.py uses for the
    reference's SpMM fixtures; the tree is not modified).  Harness
    substitutions, each a plain string substitution:
      - `#define SPMM_N <N>` in front of the program (its C text names the
        width as SPMM_N after the replacement above);
      - the two input paths become placeholders, and the text parses of its
        inputs (val from its .vbr file, char by char; X from its matrix file)
        become one fread each of the same FP32 values from binary files
        written beside the build (both before the timed region; the text
        parse of 25 M values took longer than the timed work);
      - the timed region (pthread_create .. pthread_join of its functions)
        runs SABLE_BENCH times, y set to zero before each run, one time
        printed per run; the time is printed as an integer (the generated
        printf passes a double to %lu, which prints an undefined value);
      - y is printed with %.9g instead of %f.
    The program is then cut, as text, into one translation unit per thread
    function and one for main; all are compiled with the same flags and
    linked together (the same code: the functions reach x, val and y through
    the same global pointers and are started through pthread_create; one
    2.4 MB unit took about nine minutes to compile, the units compile in
    parallel).
run_spmm(N, steps)  compiles if needed and returns the per-run times (ns)
    and the last run's Y.
"""
from __future__ import annotations

import builtins
import concurrent.futures as cf
import hashlib
import json
import os
import pathlib
import re
import subprocess
import sys
import types

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_ref" / "spmv_100k"
NAME = "spmv_100k"
THREADS = 16            # OpenMP sections of the multi-threaded program (the GPU machine's host cores)
BENCH_MARK = 97531      # iteration count at generation time, replaced by the run-time count
BENCH_MAX = 1000        # largest run-time iteration count
SPMM_OUT = HERE / "_ref" / "spmm_50k"
SPMM_WIDTHS = (32, 128)
SPMM_DENSITY = 0        # the density argument of the reference's own SpMM benchmark: every block dense
SPMM_X_SEED = 7         # the dense operand of the GPU bench (synth.dense_operand(n, N, 7))


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


def _spmv_jobs(kinds) -> tuple[list, list]:
    """Writes the SpMV inputs and sources of the programs in `kinds` not yet
    compiled; returns their gcc commands and the steps that mark them done."""
    from sable_gb300 import fileio
    if not generated():
        raise FileNotFoundError("the reference's generated C is not present (oracle/_ref/spmv_100k)")
    m, x, comp = _workload()
    meta = json.loads((OUT / "meta.json").read_text())
    if meta["signature"] != _signature(comp):
        raise RuntimeError("oracle/_ref/spmv_100k was generated for another workload")
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
    cmds, done = [], []
    for kind in kinds:
        if compiled((kind,)):
            continue
        src = work / f"{kind}.c"
        src.write_text((OUT / f"{kind}.c").read_text().replace("@VBRC_PATH@", str(vbrc))
                       .replace("@VECTOR_PATH@", str(vec)))
        cmds.append(["gcc", "-o", str(work / kind), str(src), *_cflags()])
        done.append(lambda kind=kind: (work / f"{kind}.sig").write_text(_exe_signature(kind)))
    return cmds, done


def _gcc_all(cmds: list) -> None:
    """Runs gcc commands in parallel on the host cores, in the given order."""
    def one(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            src = next((a for a in cmd if a.endswith(".c")), " ".join(cmd[:3]))
            raise RuntimeError(f"gcc failed on {src}:\n{r.stderr[-2000:]}")
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
            list(ex.map(one, cmds))


def compile(kinds=("st", "mt"), spmm_widths=()) -> None:
    """Write the inputs and compile the programs (see module docstring): the
    SpMV programs in `kinds` and the SpMM programs of `spmm_widths`, all
    translation units in one pool over the host cores (the SpMV programs,
    the longest, first)."""
    from oracle import build as ob
    ob.build()
    cmds, done = _spmv_jobs(kinds) if kinds else ([], [])
    links = []
    for N in spmm_widths:
        c, link, d = _spmm_jobs(N)
        cmds += c
        if link:
            links.append(link)
        done += d
    _gcc_all(cmds)
    _gcc_all(links)
    for d in done:
        d()


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


# ---------------------------------------------------------------------------
# The reference's generated SpMM (50000 x 50000, N = 32 and 128)
# ---------------------------------------------------------------------------
def _spmm_workload():
    sys.path.insert(0, str(ROOT))
    from sable_gb300 import synth
    return synth.spmm_50k()


def _spmm_operand(m, N: int) -> np.ndarray:
    from sable_gb300 import synth
    return synth.dense_operand(m.n_cols, N, SPMM_X_SEED)


def _spmm_signature(m, N: int) -> str:
    h = hashlib.sha256()
    for a in m.arrays():
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(f"{THREADS}/{N}/{SPMM_DENSITY}/{SPMM_X_SEED}".encode())
    return h.hexdigest()


def _spmm_dir(N: int) -> pathlib.Path:
    return SPMM_OUT / f"n{N}"


def spmm_generated(N: int) -> bool:
    """True when the generated SpMM sources for width N are present."""
    d = _spmm_dir(N)
    return (d / "meta.json").exists() and (d / "main.c").exists()


def _spmm_codegen(reference_root, N: int):
    """The reference's src/codegen.py with its SpMM width (the literal 512)
    replaced by the module variable SPMM_N = N, loaded as a private module."""
    root = pathlib.Path(reference_root).resolve()
    path = root / "src" / "codegen.py"
    src = re.sub(r"\b512\b", "SPMM_N", path.read_text())
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))        # its `from utils.fileio import read_vbrc`
    mod = types.ModuleType("sable_reference_codegen_spmm")
    mod.__file__ = str(path)
    # this module's compile() is the C build; dont_inherit keeps this file's
    # `from __future__ import annotations` out of the reference's code
    exec(builtins.compile(src, str(path), "exec", dont_inherit=True), mod.__dict__)
    mod.SPMM_N = N
    return mod


def _one(pattern: str, text: str, flags=0) -> re.Match:
    found = list(re.finditer(pattern, text, flags))
    if len(found) != 1:
        raise RuntimeError(f"expected one match of {pattern!r} in the generated SpMM, found {len(found)}")
    return found[0]


def _spmm_shim(text: str, N: int, n_val: int) -> str:
    """The harness substitutions listed in the module docstring (SpMM)."""
    lines = text.split("\n")
    for i, ln in enumerate(lines):
        if "FILE *file1 = fopen(" in ln:
            lines[i] = '\tFILE *file1 = fopen("@VAL_PATH@", "rb");'
        elif "FILE *file2 = fopen(" in ln:
            lines[i] = '\tFILE *file2 = fopen("@X_PATH@", "rb");'
    text = "\n".join(lines)
    # inputs: one fread each instead of the text parses
    m = _one(r'\n[ \t]*assert\(fscanf\(file1, "val=\[%f", &val\[val_size\]\) == 1\.0\);.*?fclose\(file1\);', text,
             re.S)
    text = (text[:m.start()] + f'\n\tif (fread(val, sizeof(float), {n_val}, file1) != {n_val}) '
            '{ printf("Error reading file1"); return 1; }\n\tfclose(file1);' + text[m.end():])
    m = _one(r'\tfor\(int i = 0; i < (\d+); i\+\+\) \{\s*for\(int j = 0; j < SPMM_N; j\+\+\) \{\s*'
             r'assert\(fscanf\(file2, "%f,", &x\[i\*SPMM_N\+j\]\) == 1\);\s*\}\s*\}\s*fclose\(file2\);', text)
    cnt = f"(size_t){m.group(1)} * SPMM_N"
    text = (text[:m.start()] + f'\tif (fread(x, sizeof(float), {cnt}, file2) != {cnt}) '
            '{ printf("Error reading file2"); return 1; }\n\tfclose(file2);' + text[m.end():])
    # the timed region, SABLE_BENCH times, y cleared before each run, the time as an integer
    zero = _one(r'\tmemset\(y, 0, [^\n]*\);\n', text).group(0)
    m = _one(r'(\tstruct timespec t1;\n.*?\tprintf\("\w+ = %lu\\n", )'
             r'(\(t2\.tv_sec - t1\.tv_sec\) \* 1e9 \+ \(t2\.tv_nsec - t1\.tv_nsec\))(\);\n)', text, re.S)
    text = (text[:m.start()] + "\tfor (int sable_it = 0; sable_it < sable_bench; sable_it++) {\n" + zero
            + m.group(1) + f"(unsigned long)({m.group(2)})" + m.group(3) + "\t}\n" + text[m.end():])
    # full-precision y
    text = text.replace('printf("%f\\n", y[i*SPMM_N + j])', 'printf("%.9g\\n", y[i*SPMM_N + j])')
    return (f"#define SPMM_N {N}\n#include <stdlib.h>\nstatic int sable_bench = 1;\n"
            "__attribute__((constructor)) static void sable_read_bench(void) {\n"
            "\tconst char *s = getenv(\"SABLE_BENCH\");\n"
            f"\tsable_bench = s ? atoi(s) : 1;\n\tif (sable_bench < 1) sable_bench = 1;\n"
            f"\tif (sable_bench > {BENCH_MAX}) sable_bench = {BENCH_MAX};\n}}\n") + text


def _spmm_split(text: str) -> dict:
    """Cuts the program into {"main.c": ..., "func<k>.c": ...}: each thread
    function in a unit of its own (with the global pointers declared extern),
    main with everything before the first function."""
    starts = [m.start() for m in re.finditer(r"^void \*func\d+\(\)\{\n", text, re.M)]
    main_at = _one(r"^int main\(\) \{\n", text, re.M).start()
    if not starts or starts[-1] > main_at:
        raise RuntimeError("unexpected layout of the generated SpMM")
    pre = text[:starts[0]]
    _one(r"^float \*x, \*val, \*y;\n", pre, re.M)
    units, protos = {}, []
    bounds = starts + [main_at]
    for k in range(len(starts)):
        body = text[bounds[k]:bounds[k + 1]]
        name = re.match(r"void \*(func\d+)\(\)", body).group(1)
        units[f"{name}.c"] = "extern float *x, *val, *y;\n\n" + body
        protos.append(f"void *{name}();\n")
    units["main.c"] = pre + "".join(protos) + "\n" + text[main_at:]
    return units


def generate_spmm(reference_root, widths=SPMM_WIDTHS) -> None:
    """Run the reference's SpMM generator (see module docstring); writes
    oracle/_ref/spmm_50k/n<N>/{main,func<k>}.c and meta.json.  Skipped where
    present for the same workload."""
    m = _spmm_workload()
    a = m.arrays()
    args = [list(map(float, a[0]))] + [list(map(int, v)) for v in a[1:]]
    for N in widths:
        d = _spmm_dir(N)
        sig = _spmm_signature(m, N)
        if spmm_generated(N) and json.loads((d / "meta.json").read_text()).get("signature") == sig:
            continue
        d.mkdir(parents=True, exist_ok=True)
        for old in d.glob("*.c"):
            old.unlink()
        sys.dont_write_bytecode = True
        cg = _spmm_codegen(reference_root, N)
        tmp = d / "gen"
        tmp.mkdir(exist_ok=True)
        cg.gen_multi_threaded_spmm(THREADS, *args, SPMM_DENSITY, str(tmp), "spmm", str(tmp))
        text = _spmm_shim((tmp / "spmm.c").read_text(), N, len(args[0]))
        (tmp / "spmm.c").unlink()
        tmp.rmdir()
        units = _spmm_split(text)
        for name, body in units.items():
            (d / name).write_text(body)
        (d / "meta.json").write_text(json.dumps({"signature": sig, "threads": THREADS, "N": N,
                                                 "units": sorted(units), "n_val": len(args[0]),
                                                 "n_rows": int(m.n_rows), "density": SPMM_DENSITY}))


def _spmm_exe_signature(N: int) -> str:
    import platform
    d = _spmm_dir(N)
    h = hashlib.sha256()
    for p in sorted(d.glob("*.c")):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(_cflags()).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def spmm_compiled(N: int) -> bool:
    """True when the SpMM program of width N is compiled for the current sources, flags and host."""
    work = _spmm_dir(N) / "run"
    sig = work / "spmm.sig"
    return (spmm_generated(N) and (work / "spmm").exists() and sig.exists()
            and sig.read_text() == _spmm_exe_signature(N))


def _spmm_jobs(N: int) -> tuple[list, list | None, list]:
    """Writes the inputs of width N and the units with their paths; returns
    the unit compiles, the link and the step that marks the program done."""
    if not spmm_generated(N):
        raise FileNotFoundError(f"the reference's generated SpMM is not present (oracle/_ref/spmm_50k/n{N})")
    d = _spmm_dir(N)
    meta = json.loads((d / "meta.json").read_text())
    m = _spmm_workload()
    if meta["signature"] != _spmm_signature(m, N):
        raise RuntimeError(f"oracle/_ref/spmm_50k/n{N} was generated for another workload")
    work = d / "run"
    work.mkdir(exist_ok=True)
    valf, xf, stamp = work / "val.f32", work / "x.f32", work / "inputs.sig"
    if not (valf.exists() and xf.exists() and stamp.exists() and stamp.read_text() == meta["signature"]):
        np.ascontiguousarray(m.val, np.float32).tofile(valf)
        np.ascontiguousarray(_spmm_operand(m, N), np.float32).tofile(xf)
        stamp.write_text(meta["signature"])
    if spmm_compiled(N):
        return [], None, []
    cmds, objs = [], []
    for name in meta["units"]:
        src = work / name
        src.write_text((d / name).read_text().replace("@VAL_PATH@", str(valf)).replace("@X_PATH@", str(xf)))
        obj = work / (name[:-2] + ".o")
        cmds.append(["gcc", *_cflags(), "-c", str(src), "-o", str(obj)])
        objs.append(str(obj))
    link = ["gcc", "-o", str(work / "spmm"), *objs, *_cflags()]
    return cmds, link, [lambda: (work / "spmm.sig").write_text(_spmm_exe_signature(N))]


def run_spmm(N: int, steps: int, timeout: float = 900.0) -> dict:
    """Run the SpMM program of width N for `steps` timed runs (compiling it
    first if needed).  Returns {"times_ns": [...], "Y": (rows, N) array,
    "threads": n}."""
    if not spmm_compiled(N):
        compile((), spmm_widths=(N,))
    meta = json.loads((_spmm_dir(N) / "meta.json").read_text())
    exe = _spmm_dir(N) / "run" / "spmm"
    env = dict(os.environ, SABLE_BENCH=str(int(steps)))
    r = subprocess.run(["bash", "-c", f"ulimit -s unlimited; exec {exe}"], capture_output=True, text=True,
                       timeout=timeout, env=env)
    if r.returncode:
        raise RuntimeError(f"generated SpMM program exited {r.returncode}: {r.stdout[:200]} {r.stderr[-500:]}")
    lines = r.stdout.split("\n", int(steps))
    times = [int(ln.split("=", 1)[1]) for ln in lines[:int(steps)]]
    Y = np.array(lines[int(steps)].split(), dtype=np.float64).reshape(meta["n_rows"], N)
    return {"times_ns": times, "Y": Y, "threads": meta["threads"]}
