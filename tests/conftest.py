"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
CPU-only machine."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "sat_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: large full-size cases")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()  # liboracle.so, and the reference's own CPU code where the reference is present
    return O


@pytest.fixture(scope="session")
def golden():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["__meta__"]).decode())
    return z, meta


@pytest.fixture(scope="session")
def golden_scans():
    """The reference's own row, transposed-row and column scans on seeded inputs."""
    z = np.load(os.path.join(os.path.dirname(GOLDEN), "scans_golden.npz"))
    meta = json.loads(bytes(z["__meta__"]).decode())
    return z, meta


@pytest.fixture(scope="session")
def satlib():
    from sat_gb300 import build as B
    B.build()
    from sat_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(satlib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
