"""The library's integer binary64 -> binary32 conversion (used by the kernels that repack FP64 tree
data as FP32: the walk arena, the walk's targets, the learned-angle features and the column-density
screen) against the GPU's own conversion, bit for bit: random bit patterns over every exponent,
values around the float range's edges (overflow, the smallest normal, subnormals, underflow to
zero), exact ties in both rounding positions, signed zeros, infinities and NaN."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def conversion_cases(seed=0):
    rng = np.random.default_rng(seed)
    n = 200_000
    bits = rng.integers(0, 2**63, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    anybits = bits.view(np.float64)  # includes double subnormals, infinities and NaNs
    sign = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    near = rng.random(n) * 2.0 ** rng.integers(-160, 135, n) * sign  # the float range and its edges
    # ties: the 29 dropped bits exactly half (hi rounds to even), and ties in the residual's rounding
    t = rng.integers(0, 2**52, 20_000, dtype=np.uint64) & ~np.uint64((1 << 29) - 1)
    t |= np.uint64(1 << 28)
    t |= rng.integers(880, 1160, 20_000).astype(np.uint64) << np.uint64(52)
    ties = t.view(np.float64)
    fmax = float(np.finfo(np.float32).max)
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.0**-149, 2.0**-150, -(2.0**-150), 3 * 2.0**-151,
                        2.0**-126, 2.0**-126 * (1 - 2.0**-30), fmax, np.nextafter(fmax, np.inf),
                        fmax * (1 + 2.0**-25), -fmax * (1 + 2.0**-24), 1e39, -1e300, 1.0, 1e8 + 0.1, 2.0**-1022,
                        np.inf, -np.inf, np.nan])
    return np.concatenate([anybits, near, ties, special])


def test_integer_conversion_matches_the_hardware():
    import torch

    from pytreegrav_gb300 import _lib

    L = _lib.load()
    L.tg_check_f32_conversion.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.c_void_p]
    L.tg_check_f32_conversion.restype = ctypes.c_int
    x = torch.from_numpy(conversion_cases()).cuda()
    bad = ctypes.c_int64(-1)
    assert L.tg_check_f32_conversion(ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.byref(bad), None) == 0
    assert bad.value == 0
