"""The library after a device reset of its own process (cudaDeviceReset, which ends only this
process's CUDA context): the streams, events and device memory it pools, and the no-alloc entry's
cached scratch address, belong to the old context, so the library must make them anew instead of
reusing dead handles.

A child process (no torch, so that nothing else holds the context) builds a tree from host arrays,
walks it, orders points with tg_morton_order and tg_morton_order_noalloc, resets the device, and
does all of it again: every call must succeed and give the same results bit for bit."""

import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent(r"""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, ROOT)
    from pytreegrav_gb300 import _lib, synthetic

    L = _lib.load()
    rt = ctypes.CDLL("libcudart.so.13")  # the runtime instance the library is linked against
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    H2D, D2H = 1, 2

    x = synthetic.plummer(20_000, 23)
    n = len(x)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)

    def once():
        t = ctypes.c_void_p()
        _lib.check(L.tg_tree_build(_lib.ptr(x), _lib.ptr(m), _lib.ptr(h), n, 1, 1, _lib.TG_MEM_HOST, None,
                                   ctypes.byref(t)), "build")
        acc = np.empty((n, 3))
        _lib.check(L.tg_tree_fields(t, None, None, n, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                                    _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_HOST, _lib.ptr(acc), None),
                   "walk")
        _lib.check(L.tg_tree_free(t), "free")
        perm = np.empty(n, np.int64)
        _lib.check(L.tg_morton_order(_lib.ptr(x), n, _lib.TG_MEM_HOST, _lib.ptr(perm), None), "morton")
        dpos, dperm = ctypes.c_void_p(), ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(dpos), x.nbytes) == 0 and rt.cudaMalloc(ctypes.byref(dperm), perm.nbytes) == 0
        assert rt.cudaMemcpy(dpos, x.ctypes.data, x.nbytes, H2D) == 0
        _lib.check(L.tg_morton_order_noalloc(dpos, n, dperm, None), "noalloc")
        perm2 = np.empty(n, np.int64)
        assert rt.cudaMemcpy(perm2.ctypes.data, dperm, perm2.nbytes, D2H) == 0
        rt.cudaFree(dpos)
        rt.cudaFree(dperm)
        assert np.array_equal(perm, perm2)
        return acc, perm

    a0, p0 = once()
    a1, p1 = once()  # pooled resources reused within one context
    assert rt.cudaDeviceSynchronize() == 0
    assert rt.cudaDeviceReset() == 0
    a2, p2 = once()  # a new context: the pools and the cached address are made again
    assert np.array_equal(a0, a1) and np.array_equal(p0, p1)
    assert np.array_equal(a0, a2) and np.array_equal(p0, p2)
    print("reset ok")
""").replace("ROOT", repr(ROOT))


def test_library_after_a_device_reset():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    r = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "reset ok" in r.stdout
