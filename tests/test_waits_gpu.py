"""The failure path of the kernels' bounded waits, exercised without a fault:
a wait on an mbarrier phase that nothing completes runs out after its limit,
the call reports SABLE_ERR_TIMEOUT (as sable_plan_check and
sable_batch_check report a kernel's wait that ran out), and the context
stays usable for the next SpMV."""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from sable_gb300 import _lib, convert, synth
from sable_gb300.plan import Plan

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_context_stays_usable(cuda):
    import torch
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    el = ctypes.c_int64(0)
    rc = lib.sable_selftest_wait(50000, 0, ctypes.byref(el), stream)          # 50 ms, nothing arrives
    assert rc == _lib.SABLE_ERR_TIMEOUT
    assert b"ran out" in lib.sable_last_error()
    assert 50_000_000 <= el.value < 1_500_000_000, el.value
    rc = lib.sable_selftest_wait(50000, 1, ctypes.byref(el), stream)          # the phase completes
    assert rc == _lib.SABLE_OK and el.value < 50_000_000, (rc, el.value)
    assert lib.sable_selftest_wait(0, 0, None, stream) == _lib.SABLE_ERR_ARG
    # the context is still usable: a plan, an SpMV, the FP64 oracle's result
    m = synth.spmv_1000()
    x = synth.vector(m.n_cols, 3)
    dense = np.random.default_rng(4).random(m.n_blocks) < 0.5
    comp = convert.compress(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, dense)
    plan = Plan(comp, schedule="warp_items", row_tile=16, chunk_bytes=4096)
    y = plan.spmv(torch.as_tensor(x).cuda()).cpu().numpy()
    plan.check()
    yr, ya = oracle.spmv_vbrc(comp, x)
    assert oracle.report(y, yr, ya)["pass"]
    plan.close()
