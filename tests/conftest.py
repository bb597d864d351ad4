import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built libnrc.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    enc = np.load(os.path.join(GOLDEN, "encode_golden.npz"))
    ev = np.load(os.path.join(GOLDEN, "evaluate_golden.npz"))
    return {"encode": dict(enc), "evaluate": dict(ev)}


@pytest.fixture(scope="session")
def nrclib():
    from vknrc_gb300 import nrc

    return nrc.lib()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test needs CUDA; run with -m 'not gpu' on a machine without a GPU")
    torch.cuda.init()
    return torch
