"""ORACLE build recipe — test infrastructure only.

Compiles the C restatement of the reference's generated executor
(vbr_oracle.c) twice into oracle/_build/:
  liboracle.so  the parity checker: -O2, no fast-math, so every sum runs in
                the reference's order in IEEE FP64;
  libcpuref.so  the timed CPU baseline: the reference's CFLAGS
                (src/consts.py:6: -O3 -funroll-all-loops -ffast-math -fopenmp)
                without its x86- and host-specific flags (-march=native -mavx
                -mprefer-vector-width=512), so the same recipe builds on x86
                and on Arm hosts.
and the MKL stand-in (mkl_standin/) used to run the reference's own
generated C in the fixture script tests/golden/make_golden.py.
"""
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build"
CHECKER = OUT / "liboracle.so"
CPUREF = OUT / "libcpuref.so"
MKL_STANDIN = OUT / "libmkl_rt.so"
CPU_CFLAGS = ["-O3", "-funroll-all-loops", "-ffast-math", "-fopenmp"]


def _cc(args):
    r = subprocess.run(["gcc", *args], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("gcc failed: " + " ".join(args) + "\n" + r.stderr)


def build(force: bool = False) -> None:
    OUT.mkdir(exist_ok=True)
    src = HERE / "vbr_oracle.c"
    mtime = src.stat().st_mtime
    if force or not CHECKER.exists() or CHECKER.stat().st_mtime < mtime:
        _cc(["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", str(src), "-o", str(CHECKER), "-lm"])
    if force or not CPUREF.exists() or CPUREF.stat().st_mtime < mtime:
        _cc([*CPU_CFLAGS, "-std=c11", "-fPIC", "-shared", str(src), "-o", str(CPUREF), "-lm"])
    ms = HERE / "mkl_standin" / "mkl_standin.c"
    if force or not MKL_STANDIN.exists() or MKL_STANDIN.stat().st_mtime < ms.stat().st_mtime:
        _cc(["-O2", "-fPIC", "-shared", f"-I{HERE / 'mkl_standin'}", str(ms), "-o", str(MKL_STANDIN)])


if __name__ == "__main__":
    build(force=True)
    print("built", CHECKER, CPUREF, MKL_STANDIN)
