"""The drop-in synthetic matrix generator (synth.vbr_matrix_gen) against the
reference's generator (synthesize_matrices/vbr_matrices_gen.py:36-113): with
the same random.seed it writes the same .vbr file name and the same arrays,
fixtures of tests/golden/ made by running the reference's own generator."""
import pathlib
import random

import numpy as np
import pytest

from sable_gb300 import fileio, synth

KEYS = ("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre")


def gen_cases(golden):
    return sorted(k for k in golden.index if k.startswith("vbrgen_"))


def test_fixtures_present(golden):
    assert len(gen_cases(golden)) >= 4


@pytest.mark.parametrize("k", range(4))
def test_seeded_generator_matches_reference(golden, tmp_path, k):
    name = gen_cases(golden)[k]
    meta = golden.meta(name)
    args = meta["args"]
    random.seed(meta["seed"])
    fname = synth.vbr_matrix_gen(*args, vbr_dir=str(tmp_path / "gen"))
    assert fname == meta["name"]
    sub = tmp_path / ("gen" if args[-1] else "gen_Sparse")
    got = fileio.read_vbr(str(sub / (fname + ".vbr")))
    for key, a in zip(KEYS, got):
        np.testing.assert_array_equal(np.asarray(a), golden.arr(name, key), err_msg=key)


def test_generator_structure(tmp_path):
    """Structure of an unseeded call: stored blocks = num_dense + num_sparse,
    dense blocks with the asked share of zeros, sparse blocks with 10
    nonzeros, values 0 or 1, a valid VBR (block rows cover bindx in order)."""
    random.seed(3)
    m, n, rs, cs, nd, pz, nsp = 100, 80, 5, 4, 6, 25, 5
    fname = synth.vbr_matrix_gen(m, n, "uniform", rs, cs, nd, pz, nsp, False, vbr_dir=str(tmp_path / "g"))
    val, indx, bindx, rpntr, cpntr, bpntrb, bpntre = fileio.read_vbr(str(tmp_path / "g_Sparse" / (fname + ".vbr")))
    assert len(bindx) == nd + nsp and indx[-1] == len(val)
    assert set(np.unique(val)) <= {0.0, 1.0}
    nnz = np.add.reduceat(np.asarray(val), np.asarray(indx[:-1])) if len(val) else np.zeros(0)
    size = np.diff(indx)
    assert np.sum(nnz == 10) >= nsp
    assert np.sum(nnz == size - size * pz // 100) >= nd
    k = 0
    for a in range(rs):
        if bpntrb[a] == -1:
            assert bpntre[a] == -1
            continue
        assert bpntrb[a] == k and bpntre[a] > k
        assert np.all(np.diff(bindx[bpntrb[a]:bpntre[a]]) > 0)
        k = bpntre[a]
    assert k == len(bindx)


def test_generator_rejects_bad_partitioning(tmp_path):
    with pytest.raises(ValueError):
        synth.vbr_matrix_gen(10, 10, "diagonal", 2, 2, 1, 0, 0, True, vbr_dir=str(tmp_path))
