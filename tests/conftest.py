import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def golden(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("golden fixture %s not present" % name)
    return np.load(path)


@pytest.fixture(scope="session")
def golden_o5v19():
    return golden("o5v19.npz")


@pytest.fixture(scope="session")
def ham_o5v19():
    from pycc_gb300.synth import SyntheticFactors
    fac = SyntheticFactors(5, 19, 0)
    F, ERI, L = fac.hamiltonian()
    return fac, F, ERI, L


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pycc_gb300._lib as lib
    lib.load()       # fails loudly when the CUDA library is missing
    return torch.device("cuda:0")
