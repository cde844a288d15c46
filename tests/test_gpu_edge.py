"""Edge cases through the public API on the GPU, against the oracle and FP64 brute force: one and two
particles, coincident points, empty target sets, far and offset coordinates, negative masses, extreme
opening angles.

Tolerances: the FP32 walk is held to 1e-5 relative RMS against the oracle's FP64 walk of the same
accepted node set (pytreegrav's bar for its FP32 path), except where noted; FP64 brute force is
bit-exact.
"""


import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RMS = 1e-5


@pytest.fixture(scope="module")
def tg():
    import pytreegrav_gb300 as tg

    return tg


def rel_rms(a, b):
    a, b = np.asarray(a).reshape(len(a), -1), np.asarray(b).reshape(len(b), -1)
    s = np.sqrt(np.mean(np.sum(b**2, 1)))
    return np.sqrt(np.mean(np.sum((a - b) ** 2, 1))) / (s if s > 0 else 1.0)


def test_single_particle_has_no_self_force(tg):
    x, m, h = np.array([[0.3, -0.2, 0.1]]), np.array([2.0]), np.array([0.1])
    for method in ("tree", "bruteforce"):
        assert np.all(tg.Accel(x, m, h, method=method) == 0)
        assert np.all(tg.Potential(x, m, h, method=method) == 0)
        assert np.all(tg.TidalTensor(x, m, h, method=method) == 0)


@pytest.mark.parametrize("soft", [0.0, 0.5])
def test_two_particles_equal_brute_force(tg, soft):
    x = np.array([[0.0, 0.0, 0.0], [0.3, 0.1, -0.2]])
    m = np.array([1.0, 3.0])
    h = np.full(2, soft)
    ref = O.bruteforce(x, h, x, m, h, potential=True, accel=True, tidal=True, mutual=True)
    for key, fn in (("potential", tg.Potential), ("accel", tg.Accel), ("tidal", tg.TidalTensor)):
        assert rel_rms(fn(x, m, h, method="tree"), ref[key]) < RMS, key
        assert np.array_equal(fn(x, m, h, method="bruteforce"), ref[key]), key


def test_coincident_points_warn_and_match_the_oracle(tg):
    rng = np.random.default_rng(1)
    x = np.vstack([np.tile([[0.5, 0.5, 0.5]], (40, 1)), rng.random((200, 3))])
    m = np.full(len(x), 1.0 / len(x))
    h = np.full(len(x), 0.02)
    with pytest.warns(UserWarning, match="non-unique"):
        t = tg.ConstructTree(x, m, h)
    assert t.HasCoincidentPoints
    got = tg.Accel(x, m, h, method="tree", tree=t)
    ref, _ = O.self_fields(x, m, h, accel=True, tree=O.OracleTree(x, m, h))
    assert np.all(np.isfinite(got))
    assert rel_rms(got, ref["accel"]) < RMS


def test_empty_target_set(tg):
    rng = np.random.default_rng(2)
    x, m = rng.random((500, 3)), np.full(500, 0.002)
    for fn, w in ((tg.AccelTarget, (0, 3)), (tg.PotentialTarget, (0,)), (tg.TidalTensorTarget, (0, 3, 3))):
        out = fn(np.zeros((0, 3)), x, m, method="tree")
        assert out.shape == w


def test_far_targets_see_a_point_mass(tg):
    rng = np.random.default_rng(3)
    x, m = rng.normal(size=(2000, 3)), rng.random(2000) / 2000
    far = np.array([[1e6, 0.0, 0.0], [0.0, -3e5, 4e5]])
    com = (m[:, None] * x).sum(0) / m.sum()
    phi = tg.PotentialTarget(far, x, m, method="tree", quadrupole=True)
    ref = -m.sum() / np.linalg.norm(far - com, axis=1)
    assert np.allclose(phi, ref, rtol=1e-7)


def test_offset_coordinates_keep_fp32_accuracy(tg):
    """A system far from the origin: the walk works on offsets from each group's reference point,
    so FP32 keeps its relative accuracy although the coordinates carry 1e8."""
    rng = np.random.default_rng(4)
    x = rng.normal(size=(5000, 3)) + np.array([1e8, -2e8, 3e7])
    m, h = np.full(5000, 1.0 / 5000), np.full(5000, 0.01)
    got = tg.Accel(x, m, h, method="tree", quadrupole=True)
    ref, _ = O.self_fields(x, m, h, accel=True, quadrupole=True)
    assert rel_rms(got, ref["accel"]) < RMS


def test_negative_masses_match_the_oracle(tg):
    rng = np.random.default_rng(5)
    x = rng.random((3000, 3))
    m = rng.normal(size=3000) / 3000
    h = np.full(3000, 0.01)
    got = tg.Accel(x, m, h, method="tree", quadrupole=True)
    ref, _ = O.self_fields(x, m, h, accel=True, quadrupole=True)
    assert rel_rms(got, ref["accel"]) < RMS


@pytest.mark.parametrize("theta", [0.05, 2.0])
def test_extreme_opening_angles(tg, theta):
    rng = np.random.default_rng(6)
    x, m, h = rng.normal(size=(3000, 3)), np.full(3000, 1.0 / 3000), np.full(3000, 0.02)
    got = tg.Accel(x, m, h, method="tree", theta=theta)
    ref, _ = O.self_fields(x, m, h, accel=True, theta=theta)
    assert rel_rms(got, ref["accel"]) < RMS
    if theta < 0.1:  # nearly every node opened: close to the direct sum
        bf = O.bruteforce(x, h, x, m, h, accel=True, mutual=True)["accel"]
        assert rel_rms(got, bf) < 1e-4
