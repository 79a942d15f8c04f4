"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on the CPU."""
import importlib
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("mesh-ferrofluid_gb300")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O._load()
    return O


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


@pytest.fixture(scope="session")
def golden():
    return {n: load_golden(n) for n in ("ico0", "ico1", "ell1")}


@pytest.fixture(scope="session")
def gauss_golden():
    return load_golden("gauss_tables")


@pytest.fixture(scope="session")
def cuda(pkg):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    pkg.load_library()
    return torch.device("cuda:0")


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
