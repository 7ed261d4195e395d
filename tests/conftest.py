import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.build_oracle import build_oracle_lib
    build_oracle_lib()
    from oracle import pyoracle
    return pyoracle


@pytest.fixture(scope="session")
def engine_lib():
    from metallic_glasses_gb300 import build
    build.build()
    from metallic_glasses_gb300 import api
    return api.load_library()


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
