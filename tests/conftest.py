import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

# Root of the reference tree (read only); tests that need its files skip when
# it is absent.  TDM_REFERENCE_ROOT overrides the default mount point.
REFERENCE = os.environ.get("TDM_REFERENCE_ROOT", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def tdm():
    import __graft_entry__ as ge
    return ge.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def golden(name):
    return os.path.join(ROOT, "tests", "golden", name)


def reference_path(*parts):
    return os.path.join(REFERENCE, *parts)


@pytest.fixture(scope="session")
def scene():
    """Seeded synthetic room fragments (the stand-in for 3DMatch fragments)."""
    import __graft_entry__ as ge
    ge.load()
    from tdm_gb300 import synth
    return synth
