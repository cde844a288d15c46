"""CPU-side checks of the drop-in boundary: the C ABI library loads and exports every symbol the
header declares, and the frontend validates arguments exactly like pytreegrav before any GPU work."""

import ctypes
import os
import re

import numpy as np
import pytest

from pytreegrav_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols(name="pytreegrav_gb300.h"):
    src = open(os.path.join(ROOT, "include", name)).read()
    return sorted(set(re.findall(r"^(?:tg_status|const char \*|int64_t|double|int)\s*(tg_\w+)\s*\(", src, re.M)))


def test_header_and_binding_agree():
    assert header_symbols() == sorted(_lib.EXPORTS)
    assert header_symbols("pytreegrav_gb300_theta.h") == sorted(_lib.THETA_EXPORTS)
    assert header_symbols("pytreegrav_gb300_measure.h") == sorted(_lib.MEASURE_EXPORTS)


def test_theta_constants_agree_with_header():
    src = open(os.path.join(ROOT, "include", "pytreegrav_gb300_theta.h")).read()
    consts = dict(re.findall(r"^#define (TG_THETA_NFEAT|TG_MLP_H|TG_THETA_FEAT_LAMBDA) (\d+)", src, re.M))
    assert int(consts["TG_THETA_NFEAT"]) == _lib.TG_THETA_NFEAT
    assert int(consts["TG_MLP_H"]) == _lib.TG_MLP_H
    assert int(consts["TG_THETA_FEAT_LAMBDA"]) == _lib.TG_THETA_FEAT_LAMBDA


def test_corr_constants_agree_with_header():
    src = open(os.path.join(ROOT, "include", "pytreegrav_gb300.h")).read()
    assert int(re.search(r"^#define TG_CORR_MAX_BINS (\d+)", src, re.M).group(1)) == _lib.TG_CORR_MAX_BINS
    kinds = re.search(r"enum \{ TG_CORR_DENSITY = (\d), TG_CORR_VELOCITY = (\d), TG_CORR_STRUCTURE = (\d) \}", src)
    assert [int(k) for k in kinds.groups()] == [_lib.TG_CORR_KINDS[k] for k in ("density", "velocity", "structure")]


def test_library_builds_loads_and_exports_every_symbol():
    from pytreegrav_gb300 import build

    path = build.build()
    L = ctypes.CDLL(path)
    for name in (header_symbols() + header_symbols("pytreegrav_gb300_theta.h")
                 + header_symbols("pytreegrav_gb300_measure.h")):
        assert hasattr(L, name), name


def test_status_mapping():
    with pytest.raises(ValueError):
        _lib.check(_lib.TG_ERR_BAD_ARG)
    with pytest.raises(ValueError, match="quadrupole"):
        _lib.check(_lib.TG_ERR_NO_QUADRUPOLES)
    with pytest.raises(MemoryError):
        _lib.check(_lib.TG_ERR_OOM)
    with pytest.raises(RuntimeError, match="Invalid input"):
        _lib.check(_lib.TG_ERR_NONFINITE)
    with pytest.raises(_lib.GravityError, match="stack"):
        _lib.check(_lib.TG_ERR_STACK_OVERFLOW)


@pytest.mark.parametrize("fn", ["Potential", "Accel", "TidalTensor"])
def test_invalid_method_raises(fn):
    import pytreegrav_gb300 as tg

    x = np.random.default_rng(0).random((10, 3))
    m = np.ones(10)
    with pytest.raises(ValueError):
        getattr(tg, fn)(x, m, method="nonsense")
    with pytest.raises(TypeError):
        getattr(tg, fn)(x, m, method=3)


@pytest.mark.parametrize("fn", ["PotentialTarget", "AccelTarget", "TidalTensorTarget"])
def test_target_forms_need_sources_or_tree(fn):
    import pytreegrav_gb300 as tg

    x = np.random.default_rng(0).random((10, 3))
    with pytest.raises(ValueError, match="Must pass either"):
        getattr(tg, fn)(x, None, None)
    with pytest.raises(ValueError):
        getattr(tg, fn)(x, x, np.ones(10), method="nonsense")


@pytest.mark.parametrize("fn", ["Potential", "Accel"])
def test_frontend_rejects_bad_device_combinations(fn):
    import pytreegrav_gb300 as tg

    x = np.random.default_rng(0).random((500, 3))
    m = np.ones(500)
    with pytest.raises(ValueError, match="must be 'cpu' or 'cuda'"):
        getattr(tg, fn)(x, m, device="gpu")
    with pytest.raises(ValueError, match="monopole only"):
        getattr(tg, fn)(x, m, device="cuda", quadrupole=True)


def test_nonfinite_status_prints_and_raises_like_construct_tree(monkeypatch, capsys):
    """The library's device-side check reports TG_ERR_NONFINITE; ConstructTree then prints and raises
    as frontend.py:123-125 does. The device call is replaced by its status here (no GPU)."""
    import pytreegrav_gb300 as tg
    from pytreegrav_gb300 import frontend

    def fake_octree(*a, **k):
        _lib.check(_lib.TG_ERR_NONFINITE, "ConstructTree")

    monkeypatch.setattr(frontend, "Octree", fake_octree)
    x = np.random.default_rng(0).random((100, 3))
    x[3, 1] = np.nan
    with pytest.raises(RuntimeError, match="^Invalid input detected - aborting treebuild"):
        tg.ConstructTree(x, np.ones(100))
    assert "Invalid input detected" in capsys.readouterr().out


def test_quadrupole_guard():
    import pytreegrav_gb300 as tg

    class Fake:
        HasQuads = False

    with pytest.raises(ValueError, match="quadrupole"):
        tg.checkTreeQuadrupoles(Fake(), True)
    tg.checkTreeQuadrupoles(Fake(), False)


class _FakeColumnTree:
    """Records the column-density calls the frontend makes; results encode the call."""

    def __init__(self, n):
        self.n = n
        self.calls = []

    def column_density_self(self, rays=None, theta=0.5, group_size=0):
        self.calls.append(("self", None if rays is None else np.shape(rays), theta, group_size))
        w = 6 if rays is None else np.shape(rays)[-2]
        return np.arange(self.n * w, dtype=float).reshape(self.n, w)

    def column_density(self, pos, rays=None, theta=0.5, group_size=0):
        self.calls.append(("explicit", np.array(pos), None if rays is None else np.shape(rays), theta, group_size))
        w = 6 if rays is None else np.shape(rays)[-2]
        return np.arange(len(pos) * w, dtype=float).reshape(len(pos), w)


def test_column_density_dispatch_own_and_given_trees(monkeypatch):
    """ColumnDensity on a tree it builds asks the library for the tree's own particles (rows come back
    in the caller's order, so no host gather or scatter); on a given tree it Morton-orders the targets,
    walks them and undoes the order (frontend.py:1440-1452). Dispatch only, no GPU work."""
    from pytreegrav_gb300 import frontend

    n = 1200
    x = np.random.default_rng(3).normal(size=(n, 3))
    fake = _FakeColumnTree(n)
    monkeypatch.setattr(frontend, "ConstructTree", lambda *a, **k: fake)
    monkeypatch.setattr(frontend, "_check_tree", lambda t: None)
    perm = np.random.default_rng(4).permutation(n)
    monkeypatch.setattr(frontend, "morton_order", lambda p: perm)
    m, h = np.ones(n), np.full(n, 0.1)

    out = frontend.ColumnDensity(x, m, h, rays=6)
    assert fake.calls[-1] == ("self", (6, 3), 0.5, 0)
    assert np.array_equal(out, np.arange(n * 6, dtype=float).reshape(n, 6))
    frontend.ColumnDensity(x, m, h)  # binned, grouped from 1000 targets with pytreegrav's group size 16
    assert fake.calls[-1] == ("self", None, 0.5, 16)

    out = frontend.ColumnDensity(x, m, h, rays=6, tree=fake)
    kind, pos, shape, theta, gs = fake.calls[-1]
    assert kind == "explicit" and shape == (6, 3) and np.array_equal(pos, x[perm])
    expect = np.empty((n, 6))
    expect[perm] = np.arange(n * 6, dtype=float).reshape(n, 6)
    assert np.array_equal(out, expect)
