"""Shared pytest configuration: the `gpu` marker and common fixtures."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "minife_golden.npz"))


@pytest.fixture(scope="session")
def golden_hashes():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "golden_hashes.json")) as f:
        return json.load(f)
