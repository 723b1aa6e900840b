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
