import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")
    config.addinivalue_line("markers", "slow: longer CPU test")


def _lib_built() -> bool:
    return os.path.exists(os.path.join(ROOT, "cryoim_gb300", "_lib", "libcryoim_gb300.so"))


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library (cross-compiles without a GPU) and the oracle once."""
    from cryoim_gb300 import build as b
    if not _lib_built() or os.environ.get("CRYOIM_REBUILD"):
        b.build_library()
    b.build_oracle()
    return True


@pytest.fixture(scope="session")
def orc(built):
    import pyoracle
    return pyoracle


@pytest.fixture(scope="session")
def golden_ops():
    import json
    d = json.load(open(os.path.join(ROOT, "tests", "golden", "icos2f_sym_mat.json")))
    return np.array(d["rot"], np.float64)


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
