import json
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


class Golden:
    def __init__(self):
        self.index = json.loads((GOLDEN / "golden.json").read_text())
        self._z = np.load(GOLDEN / "golden.npz")

    def meta(self, name):
        return self.index[name]

    def arr(self, name, key):
        return self._z[f"{name}__{key}"]

    def arrays(self, name, keys=("val", "indx", "bindx", "rpntr", "cpntr", "bpntrb", "bpntre")):
        return tuple(self.arr(name, k) for k in keys)


@pytest.fixture(scope="session")
def golden():
    return Golden()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
