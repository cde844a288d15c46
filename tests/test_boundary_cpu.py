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
