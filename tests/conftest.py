import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "lbm-dem_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    import lbdem
    if not os.path.exists(lbdem.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()


@pytest.fixture(scope="session")
def lib():
    _ensure_built()
    import lbdem
    return lbdem.load_library()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle_ffi
    oracle_ffi.build_oracle()
    return oracle_ffi.load()


def golden_case(name):
    """(cfg path, npz) of a committed golden case."""
    import numpy as np
    return (os.path.join(GOLDEN, name, "parameters.cfg"),
            np.load(os.path.join(GOLDEN, f"{name}.npz")))


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
