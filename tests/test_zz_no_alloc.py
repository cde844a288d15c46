"""tg_morton_order_noalloc (the entry point that allocates nothing) against tg_morton_order.

Both are called through the C ABI. The no-alloc call gets device buffers made here by torch (the
caller owns all memory); the reference result comes from tg_morton_order on host arrays. A Morton
permutation is index work, so the tolerance is zero: the two permutations must be identical.

Calls are made back to back on one stream with inputs of different sizes and contents, so a
result that depended on what the previous call left in the shared scratch array would show.
This file is named to be collected last, and it also passes run alone in a fresh process (where
its first call is the one that looks up the scratch array)."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MISMATCHES = 0  # integer permutation: bit-exact


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from pytreegrav_gb300 import _lib

    return torch, _lib, _lib.load()


def points(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "plummer":
        u = rng.uniform(0.0, 1.0, n)
        r = np.minimum(1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0), 50.0)
        v = rng.normal(size=(n, 3))
        return v / np.linalg.norm(v, axis=1)[:, None] * r[:, None]
    if kind == "duplicates":  # few distinct points: stability of equal keys decides the order
        base = rng.uniform(-1.0, 1.0, (7, 3))
        return base[rng.integers(0, 7, n)]
    return rng.uniform(-3.0, 5.0, (n, 3))


def order_existing(L, _lib, pos):
    perm = np.empty(len(pos), np.int64)
    _lib.check(L.tg_morton_order(_lib.ptr(pos), len(pos), _lib.TG_MEM_HOST, _lib.ptr(perm), None), "morton_order")
    return perm


def order_noalloc(torch, L, pos):
    dpos = torch.from_numpy(pos).cuda()
    dperm = torch.full((len(pos),), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    rc = L.tg_morton_order_noalloc(ctypes.c_void_p(dpos.data_ptr()), len(pos), ctypes.c_void_p(dperm.data_ptr()),
                                   ctypes.c_void_p(stream))
    return rc, dperm.cpu().numpy()


def test_noalloc_matches_existing_entry_point_on_consecutive_calls(env):
    torch, _lib, L = env
    cases = [("plummer", 200_000, 1), ("duplicates", 5_000, 2), ("uniform", _lib.TG_NOALLOC_MAX_POINTS, 3),
             ("plummer", 4_097, 4), ("uniform", 1, 5)]
    for kind, n, seed in cases:
        pos = np.ascontiguousarray(points(kind, n, seed))
        want = order_existing(L, _lib, pos)
        for call in range(2):  # two calls in a row on the same input
            rc, got = order_noalloc(torch, L, pos)
            assert rc == _lib.TG_OK, (kind, n, call, L.tg_last_error())
            mismatches = int(np.count_nonzero(got != want))
            assert mismatches <= TOL_MISMATCHES, f"{kind} n={n} call {call}: {mismatches} entries differ"


def test_noalloc_rejects_too_many_points(env):
    torch, _lib, L = env
    n = _lib.TG_NOALLOC_MAX_POINTS + 1
    dpos = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    dperm = torch.zeros(n, dtype=torch.int64, device="cuda")
    rc = L.tg_morton_order_noalloc(ctypes.c_void_p(dpos.data_ptr()), n, ctypes.c_void_p(dperm.data_ptr()), None)
    assert rc == _lib.TG_ERR_BAD_ARG
    assert b"exceeds the fixed scratch capacity" in L.tg_last_error()


def test_noalloc_rejects_host_memory_and_nonfinite(env):
    torch, _lib, L = env
    pos = np.zeros((10, 3))
    perm = np.zeros(10, np.int64)
    rc = L.tg_morton_order_noalloc(_lib.ptr(pos), 10, _lib.ptr(perm), None)
    assert rc == _lib.TG_ERR_BAD_ARG
    assert b"not device memory" in L.tg_last_error()
    bad = np.ascontiguousarray(points("uniform", 1000, 6))
    bad[500, 1] = np.nan
    rc, _ = order_noalloc(torch, L, bad)
    assert rc == _lib.TG_ERR_NONFINITE
    # the shared scratch is usable again right after a rejected call
    good = np.ascontiguousarray(points("plummer", 3000, 7))
    rc, got = order_noalloc(torch, L, good)
    assert rc == _lib.TG_OK
    assert np.array_equal(got, order_existing(L, _lib, good))
