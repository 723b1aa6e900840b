"""The reference's generated CPU executor used as the timed baseline
(oracle/refc.py): the listed harness substitutions, and nothing else, were
applied to the sources it generated (present where the build container ran
the reference's generator)."""
import re

import pytest

from oracle import refc


def test_generated_sources_carry_only_the_listed_shims():
    if not refc.generated():
        pytest.skip("the reference's generated C is not present on this host")
    for kind in ("st", "mt"):
        text = (refc.OUT / f"{kind}.c").read_text()
        assert str(refc.BENCH_MARK) not in text and str(refc.BENCH_MARK + 1) not in text
        assert 'fopen("@VBRC_PATH@", "r")' in text and 'fopen("@VECTOR_PATH@", "r")' in text
        assert f"long times[{refc.BENCH_MAX}]" in text
        assert text.count("i<sable_bench+1;") == 1 and text.count("i<sable_bench;") == 1
        assert 'printf("%.17g\\n", y[i])' in text
        # the block calls of the reference's generator are untouched
        assert len(re.findall(r"spmv_kernel(_2|_3)?\(y, x, val,", text)) > 1000
        assert "mkl_sparse_d_mv(SPARSE_OPERATION_NON_TRANSPOSE" in text
    assert "#pragma omp section" in (refc.OUT / "mt.c").read_text()


def test_generated_spmm_sources_carry_only_the_listed_shims():
    """The reference's SpMM program per width: the width macro, binary input
    reads, the repeated timed region and the output format are the only
    changes; every block of the matrix appears as one dense loop nest in the
    thread functions, and the units together hold all thread functions."""
    widths = [N for N in refc.SPMM_WIDTHS if refc.spmm_generated(N)]
    if not widths:
        pytest.skip("the reference's generated SpMM is not present on this host")
    import json
    from sable_gb300 import synth
    m = synth.spmm_50k()
    for N in widths:
        d = refc._spmm_dir(N)
        meta = json.loads((d / "meta.json").read_text())
        assert meta["signature"] == refc._spmm_signature(m, N) and meta["density"] == 0
        main = (d / "main.c").read_text()
        assert main.startswith(f"#define SPMM_N {N}\n")
        assert 'fopen("@VAL_PATH@", "rb")' in main and 'fopen("@X_PATH@", "rb")' in main
        assert "fscanf" not in main and main.count("fread(") == 2
        assert main.count("for (int sable_it = 0; sable_it < sable_bench; sable_it++) {") == 1
        assert main.count("(unsigned long)((t2.tv_sec - t1.tv_sec) * 1e9 + (t2.tv_nsec - t1.tv_nsec))") == 1
        assert 'printf("%.9g\\n", y[i*SPMM_N + j])' in main and 'printf("%f' not in main
        funcs = sorted(u for u in meta["units"] if u != "main.c")
        assert len(funcs) == refc.THREADS
        nests = 0
        for u in funcs:
            body = (d / u).read_text()
            assert body.startswith("extern float *x, *val, *y;\n")
            assert f"void *{u[:-2]}();" in main and f"pthread_create(&tid[{u[4:-2]}], NULL, &{u[:-2]}, NULL);" in main
            nests += len(re.findall(rf"for \(int k = 0; k < {N}; k\+\+\) \{{;y\[", body))
        assert nests == len(m.bindx)


def test_spmm_program_pipeline_on_a_small_matrix(tmp_path):
    """The SpMM harness end to end on a 400 x 400 matrix (where the reference
    tree is present): the reference's generator with the width as SPMM_N, the
    listed substitutions, the cut into one unit per thread function, binary
    inputs, three timed runs; Y of the last run against the FP64 oracle."""
    import subprocess

    import numpy as np

    from oracle import build as ob
    from oracle import oracle
    from sable_gb300 import synth
    root = ob.reference_root()
    if root is None:
        pytest.skip("the reference tree is not present on this host")
    ob.build()
    m = synth.spmm_50k(seed=1010, n=400, parts=10, p=0.3)
    N = 8
    a = m.arrays()
    args = [list(map(float, a[0]))] + [list(map(int, v)) for v in a[1:]]
    gen = tmp_path / "gen"
    gen.mkdir()
    refc._spmm_codegen(root, N).gen_multi_threaded_spmm(4, *args, 0, str(gen), "spmm", str(gen))
    units = refc._spmm_split(refc._spmm_shim((gen / "spmm.c").read_text(), N, len(args[0])))
    assert sorted(units) == ["func0.c", "func1.c", "func2.c", "func3.c", "main.c"]
    valf, xf = tmp_path / "val.f32", tmp_path / "x.f32"
    np.asarray(m.val, np.float32).tofile(valf)
    X = synth.dense_operand(m.n_cols, N, 3)
    X.tofile(xf)
    objs = []
    for name, body in units.items():
        src = tmp_path / name
        src.write_text(body.replace("@VAL_PATH@", str(valf)).replace("@X_PATH@", str(xf)))
        objs.append(str(tmp_path / (name[:-2] + ".o")))
        subprocess.run(["gcc", "-O1", "-c", str(src), "-o", objs[-1]], check=True, capture_output=True)
    exe = tmp_path / "spmm"
    subprocess.run(["gcc", "-o", str(exe), *objs, "-lpthread"], check=True, capture_output=True)
    r = subprocess.run([str(exe)], env={"SABLE_BENCH": "3"}, capture_output=True, text=True, check=True)
    lines = r.stdout.split("\n", 3)
    assert all(re.fullmatch(r"spmm = \d+", ln) for ln in lines[:3]), lines[:3]
    Y = np.array(lines[3].split(), dtype=np.float64).reshape(m.n_rows, N)
    Yr, Ya = oracle.spmm_vbr(m, X.astype(np.float64))
    rep = oracle.report(Y, Yr, Ya, 1e-5)
    assert rep["pass"], rep
