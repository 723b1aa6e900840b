"""The SpMM entry point that allocates nothing (sable_spmm_noalloc).

Callers that cannot let a library allocate device memory during a call (a
runtime whose pool allocator owns all device memory, a real-time loop that
must not block on the driver's allocator) use this entry point; call after
call, it must give the result of sable_spmm, within the parity tolerance of
the FP64 oracle, with its scratch in the library's fixed device array.  This file is collected last so
that a failure here cannot hide the other tests in a run that stops at the
first failure; it also passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import _lib, convert, synth
from sable_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def _matrix(seed=41):
    rng = np.random.default_rng(seed)
    rs = np.array([1, 300, 64, 2, 100, 37, 128])
    cs = np.array([1, 250, 3, 64, 77, 2, 31, 90])
    present = rng.random((len(rs), len(cs))) < 0.7

    def fill(rng, h, w, a, b):
        v = rng.uniform(-1, 1, (h, w)).astype(np.float32)
        return v if rng.random() < 0.5 else v * synth.block_pattern(rng, h, w, rng.uniform(0.05, 0.4), "uniform")

    return synth.assemble(rng, rs, cs, present, fill)


@pytest.mark.parametrize("N,tc", [(8, "off"), (32, "off"), (64, "off"), (32, "split3"), (64, "split3")])
def test_noalloc_matches_spmm_twice(cuda, N, tc):
    import torch
    m = _matrix()
    rng = np.random.default_rng(42)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, rng.random(m.n_blocks) < 0.5)
    plan = Plan(comp, chunk_bytes=4096, spmm_tc=tc)   # small items: many split tiles use the scratch
    assert plan.stats()["scratch_floats"] > 0
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        X = torch.as_tensor(synth.dense_operand(m.n_cols, N, 100 + call)).cuda()
        Y_spmm = torch.empty(m.n_rows, N, device="cuda")
        Y_new = torch.full((m.n_rows, N), float("nan"), device="cuda")
        _lib.check(lib.sable_spmm(plan.handle, X.data_ptr(), N, Y_spmm.data_ptr(), N, N, stream), "sable_spmm")
        _lib.check(lib.sable_spmm_noalloc(plan.handle, X.data_ptr(), N, Y_new.data_ptr(), N, N, stream),
                   "sable_spmm_noalloc")
        torch.cuda.synchronize()
        Yn = Y_new.cpu().numpy()
        Yr, Ya = oracle.spmm_vbr(m, X.cpu().numpy())
        r = oracle.report(Yn, Yr, Ya)            # against FP64: tolerance 1e-5 * (|A||X|)
        assert r["pass"], (call, r)
        # the same kernels as sable_spmm: bit-identical output
        assert np.array_equal(Yn, Y_spmm.cpu().numpy()), call
    plan.close()


def test_noalloc_rejects_oversized_plan(cuda):
    import torch
    m = synth.spmm_50k(seed=1011, n=3000, parts=60, p=0.5)
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, np.ones(m.n_blocks, bool))
    plan = Plan(comp, chunk_bytes=4096)
    N = 512
    need = plan.stats()["scratch_floats"] * 128 * (N // 128)
    assert need > (2 << 20), "test plan must exceed the fixed scratch"
    X = torch.zeros(m.n_cols, N, device="cuda")
    Y = torch.zeros(m.n_rows, N, device="cuda")
    rc = _lib.load().sable_spmm_noalloc(plan.handle, X.data_ptr(), N, Y.data_ptr(), N, N,
                                        torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.SABLE_ERR_UNSUPPORTED
    assert b"fixed scratch" in _lib.load().sable_last_error()
    plan.close()
