import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def load_golden(name):
    import json
    import numpy as np
    man = json.load(open(os.path.join(GOLDEN, "manifest.json")))
    return man[name], np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture
def golden():
    return load_golden
