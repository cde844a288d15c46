import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a) and the built library")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def golden_trees():
    return load_golden("golden_trees.npz")


@pytest.fixture(scope="session")
def golden_walk():
    return load_golden("golden_walk.npz")


@pytest.fixture(scope="session")
def golden_bruteforce():
    return load_golden("golden_bruteforce.npz")


@pytest.fixture(scope="session")
def golden_bigtree():
    return load_golden("golden_bigtree.npz")


@pytest.fixture(scope="session")
def golden_column():
    return load_golden("golden_column.npz")
