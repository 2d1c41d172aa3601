import ctypes
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through libvkhel's C ABI")
    config.addinivalue_line("markers", "slow: long-running")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    return pyoracle.load()


@pytest.fixture(scope="session")
def vk():
    import vkhel_gb300
    vkhel_gb300.lib()
    return vkhel_gb300


@pytest.fixture(scope="session")
def ctx(vk):
    c = vk.Context()
    yield c


def u64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64))
