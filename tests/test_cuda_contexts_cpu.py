"""pytreegrav_gb300.cuda without a GPU: the names pytreegrav.cuda exports, the missing-device error
(cuda.py:70-80, 553-557) and the packed-row format (cuda.py:299-357). No GPU work."""

import numpy as np
import pytest

from pytreegrav_gb300 import cuda


def test_names_of_pytreegrav_cuda():
    for name in ("is_available", "pack_tree_gravity", "CudaPotential", "CudaAccel", "CudaPotentialBruteforce",
                 "CudaAccelBruteforce", "CudaColumnDensity", "THREADS_X", "GRAV_ROW"):
        assert hasattr(cuda, name), name


def test_no_device_raises_runtime_error(monkeypatch):
    monkeypatch.setattr(cuda, "is_available", lambda: False)
    x = np.zeros((4, 3))
    with pytest.raises(RuntimeError, match="no CUDA device available"):
        cuda.CudaAccelBruteforce(x, np.ones(4))
    with pytest.raises(RuntimeError, match="no CUDA device available"):
        cuda.CudaPotential(object())


def test_is_available_is_false_without_a_gpu():
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is visible")
    assert cuda.is_available() is False


class _Tree:
    """The attributes pytreegrav's Octree exposes, two particles and one node."""

    NumNodes = 3
    Coordinates = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.5, 0.0, 0.0]])
    Masses = np.array([1.0, 1.0, 2.0])
    Softenings = np.array([0.1, 0.2, 0.2])
    Sizes = np.array([0.0, 0.0, 2.0])
    Deltas = np.array([0.0, 0.0, 0.5])
    NextBranch = np.array([1, -1, -1])
    FirstSubnode = np.array([-1, -1, 0])


def test_pack_tree_gravity_rows_and_links():
    rows, links = cuda.pack_tree_gravity(_Tree())
    assert rows.dtype == np.float32 and rows.shape == (3, cuda.GRAV_ROW)
    assert links.dtype == np.int32 and links.shape == (3, 2)
    np.testing.assert_array_equal(rows[2], np.float32([0.5, 0.0, 0.0, 2.0, 0.2, 2.0, 0.5, 0.0]))
    np.testing.assert_array_equal(links[:, 0], [1, -1, -1])
    np.testing.assert_array_equal(links[:, 1], [-1, -1, 0])


def test_pack_tree_gravity_overflow_is_value_error():
    t = _Tree()
    t.Masses = np.array([1.0, 1e300, 2.0])
    with pytest.raises(ValueError, match="packing overflowed float32"):
        cuda.pack_tree_gravity(t)
