"""Host emulation of the split-BF16 products used by the tensor-core SpMM:
the error the kernel can reach, on the reference's seeded 400 x 400 SpMM case,
against the FP64 oracle.  The two-term split (three products) stays within
3 * 2^-16 (|A||X|) but not within the 1e-5 parity tolerance; the three-term
split (six products) stays within 1e-5."""
import numpy as np

from oracle import oracle
from sable_gb300 import convert, synth


def bf16_rn(a):
    """Round FP32 to the nearest BF16 (ties to even), returned as FP32."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def split(a, terms):
    out, r = [], np.asarray(a, np.float32)
    for _ in range(terms):
        t = bf16_rn(r)
        out.append(t.astype(np.float64))
        r = (r - t).astype(np.float32)
    return out


def emulate(A, X, terms):
    a, x = split(A, terms), split(X, terms)
    pairs = [(0, 0), (0, 1), (1, 0)] if terms == 2 else [(0, 0), (0, 1), (1, 0), (0, 2), (2, 0), (1, 1)]
    return sum(a[i] @ x[j] for i, j in pairs)


def test_split_error_bounds(golden):
    meta = golden.meta("spmm400_N32_d0")
    m = synth.spmm_50k(meta["seed"], n=meta["n"], parts=meta["parts"], p=meta["p"])
    X = synth.dense_operand(m.n_cols, meta["N"], meta["x_seed"])
    A = convert.vbr_to_dense(*m.arrays()).astype(np.float32)
    Yr, Ya = oracle.spmm_vbr(m, X)
    r2 = oracle.report(emulate(A, X, 2), Yr, Ya, oracle.TOL_SPLIT2)
    r3 = oracle.report(emulate(A, X, 3), Yr, Ya)
    assert r2["pass"] and r2["max"] > oracle.TOL, r2
    assert r3["pass"] and r3["max"] < 1e-6, r3


def test_split_terms_exact():
    """Three BF16 terms hold every FP32 value in [-1, 1] exactly (24 bits)."""
    v = np.random.default_rng(0).uniform(-1, 1, 100000).astype(np.float32)
    s = split(v, 3)
    np.testing.assert_array_equal((s[0] + s[1] + s[2]).astype(np.float32), v)
    assert np.all(np.abs(s[0] + s[1] + s[2] - v.astype(np.float64)) <= 2.0 ** -24 * np.abs(v))
