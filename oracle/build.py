"""ORACLE build recipe — test infrastructure only.

Compiles the C restatement of the reference's generated executor
(vbr_oracle.c) twice into oracle/_build/:
  liboracle.so  the parity checker: -O2, no fast-math, so every sum runs in
                the reference's order in IEEE FP64;
  libcpuref.so  the timed CPU baseline port: the reference's CFLAGS
                (src/consts.py:6: -O3 -march=native -funroll-all-loops
                -mprefer-vector-width=512 -mavx -ffast-math -lpthread
                -fopenmp) as reference_cflags() adapts them to the host:
                all of them on x86-64, without the two x86-only ones
                (-mprefer-vector-width=512 -mavx) elsewhere (Arm hosts);
and the MKL stand-in (mkl_standin/) used to run the reference's own
generated C (tests/golden/make_golden.py, oracle/refc.py).  Where the
reference tree is present (SABLE_REFERENCE_ROOT, else REFERENCE_ROOT), build()
also runs the reference's own code generators (SpMV and SpMM) for the timed
CPU baselines (oracle/refc.py, into oracle/_ref/).
"""
import os
import pathlib
import platform
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
REFERENCE_ROOT = "/root/reference"   # where the reference tree is mounted in the build container
OUT = HERE / "_build"
CHECKER = OUT / "liboracle.so"
CPUREF = OUT / "libcpuref.so"
MKL_STANDIN = OUT / "libmkl_rt.so"
REFERENCE_CFLAGS = ["-O3", "-march=native", "-funroll-all-loops", "-mprefer-vector-width=512", "-mavx", "-ffast-math",
                    "-lpthread", "-fopenmp"]
X86_ONLY = ("-mprefer-vector-width=512", "-mavx")


def reference_cflags() -> list:
    """The reference's CFLAGS for this host (x86-only flags dropped elsewhere)."""
    if platform.machine() in ("x86_64", "AMD64"):
        return list(REFERENCE_CFLAGS)
    return [f for f in REFERENCE_CFLAGS if f not in X86_ONLY]


CPU_CFLAGS = [f for f in reference_cflags() if f != "-lpthread"]


def _cc(args):
    r = subprocess.run(["gcc", *args], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("gcc failed: " + " ".join(args) + "\n" + r.stderr)


def reference_root():
    root = pathlib.Path(os.environ.get("SABLE_REFERENCE_ROOT", REFERENCE_ROOT))
    return root if (root / "src" / "codegen.py").exists() else None


def build(force: bool = False, generate: bool = False) -> None:
    """Compile the checker, the CPU-baseline port and the MKL stand-in;
    with generate=True also run the reference's generator when its tree is
    present (oracle/refc.py)."""
    OUT.mkdir(exist_ok=True)
    src = HERE / "vbr_oracle.c"
    mtime = src.stat().st_mtime
    if force or not CHECKER.exists() or CHECKER.stat().st_mtime < mtime:
        _cc(["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", str(src), "-o", str(CHECKER), "-lm"])
    if force or not CPUREF.exists() or CPUREF.stat().st_mtime < mtime:
        _cc([*CPU_CFLAGS, "-std=c11", "-fPIC", "-shared", str(src), "-o", str(CPUREF), "-lm"])
    ms = HERE / "mkl_standin" / "mkl_standin.c"
    if force or not MKL_STANDIN.exists() or MKL_STANDIN.stat().st_mtime < ms.stat().st_mtime:
        _cc(["-O2", "-fPIC", "-shared", "-fopenmp", f"-I{HERE / 'mkl_standin'}", str(ms), "-o", str(MKL_STANDIN)])
    if generate and reference_root() is not None:
        from oracle import refc
        refc.generate(reference_root())
        refc.generate_spmm(reference_root())


if __name__ == "__main__":
    build(force=True)
    print("built", CHECKER, CPUREF, MKL_STANDIN)
