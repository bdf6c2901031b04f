import os
import random
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer-running case")


@pytest.fixture(autouse=True)
def _seed():
    random.seed(0)
    np.random.seed(0)
    try:
        import torch
        torch.manual_seed(0)
    except Exception:
        pass
    yield


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def unpack_spectra(lens, flat):
    out, o = [], 0
    for n in lens:
        out.append(flat[o:o + int(n)])
        o += int(n)
    return out


def unpack_tensors(shapes, flat):
    out, o = [], 0
    for s in shapes:
        sz = int(np.prod(s))
        out.append(flat[o:o + sz].reshape(tuple(int(x) for x in s)))
        o += sz
    return out
