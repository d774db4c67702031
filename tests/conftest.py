import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsegfock.so")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


class CGF:
    """Reference-style contracted function from a golden record."""

    def __init__(self, d):
        self.coefs = d["coefs"]
        self.expns = d["expns"]
        self.shell = d["shell"]
        self.normalize_factors = d["nf"]
        self.center = d["center"]


@pytest.fixture(scope="session")
def h2o_golden():
    return load_golden("h2o_sto3g.json")


@pytest.fixture(scope="session")
def quartet_golden():
    return load_golden("quartets_mmd.json")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import torch
    return torch.device("cuda:0")
