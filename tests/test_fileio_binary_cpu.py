"""Binary (.vbrb / .vbrcb) forms of the reference's text files
(utils/fileio.py:13-35, 55-93): round trips, the entry points' choice of
file (text first, then binary), and refusal of the wrong kind of file."""
import os

import numpy as np
import pytest

from sable_gb300 import convert, fileio, synth
from sable_gb300.vbr import VBR


def test_vbr_binary_round_trip(tmp_path):
    m = synth.spmv_1000(1000)
    arrays = [np.asarray(a) for a in m.arrays()]
    path = fileio.write_vbr_binary("m", VBR(*arrays), str(tmp_path))
    assert path.endswith(".vbrb")
    for a, b in zip(arrays, fileio.read_vbr(path)):
        np.testing.assert_array_equal(a, b)
    assert fileio.source_path(str(tmp_path), "m", ".vbr") == path
    fileio.write_vbr_matrix("m", VBR(*[a.tolist() for a in arrays]), str(tmp_path))
    assert fileio.source_path(str(tmp_path), "m", ".vbr") == os.path.join(str(tmp_path), "m.vbr")


def test_vbrc_binary_matches_text(tmp_path):
    m = synth.spmv_1000(1000)
    for binary in (False, True):
        convert.convert_vbr_to_compressed(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, "m",
                                          str(tmp_path), density=50, binary=binary)
    t = fileio.read_vbrc(os.path.join(str(tmp_path), "m.vbrc"))
    b = fileio.read_vbrc(os.path.join(str(tmp_path), "m.vbrcb"))
    for x, y in zip(t, b):
        np.testing.assert_array_equal(np.asarray(x, np.float64), np.asarray(y, np.float64))


def test_wrong_kind_refused(tmp_path):
    m = synth.spmv_1000(1000)
    path = fileio.write_vbr_binary("m", VBR(*[np.asarray(a) for a in m.arrays()]), str(tmp_path))
    with pytest.raises(ValueError, match="uncompressed"):
        fileio.read_vbrc(path)
    convert.convert_vbr_to_compressed(m.val, m.rpntr, m.cpntr, m.indx, m.bindx, m.bpntrb, m.bpntre, "c",
                                      str(tmp_path), density=50, binary=True)
    with pytest.raises(ValueError, match="compressed"):
        fileio.read_vbr(os.path.join(str(tmp_path), "c.vbrcb"))
