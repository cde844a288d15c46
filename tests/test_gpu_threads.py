"""Concurrent use from several host threads, each on its own CUDA stream: builds, plain and learned
walks and frees running at the same time must give each thread exactly the results it gets alone.
The library's shared state (memory pool, pooled side streams and events, per-thread build side
streams, error strings) is per device behind a lock or per thread; ctypes releases the GIL during
each call, so the calls do overlap on the host and on the GPU."""

import ctypes
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 60_000
THREADS = 4
ROUNDS = 4


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from pytreegrav_gb300 import _lib, synthetic, theta

    return torch, _lib, _lib.load(), synthetic, theta


def one_step(torch, _lib, L, x, m, h, out, stream, model_handle, l10):
    vp = ctypes.c_void_p
    t = vp()
    _lib.check(L.tg_tree_build(vp(x.data_ptr()), vp(m.data_ptr()), vp(h.data_ptr()), N, 1, 1, _lib.TG_MEM_DEVICE,
                               vp(stream.cuda_stream), ctypes.byref(t)), "build")
    try:
        _lib.check(L.tg_tree_fields(t, None, None, N, _lib.TG_FIELD_ACCEL, 1, 0.7, 1.0, 32, _lib.TG_GROUP_TREE,
                                    _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(out[0].data_ptr()),
                                    vp(stream.cuda_stream)), "walk")
        _lib.check(L.tg_tree_fields_learned(t, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, model_handle, l10, 0.7,
                                            _lib.TG_MEM_DEVICE, vp(out[1].data_ptr()), vp(stream.cuda_stream)),
                   "learned")
    finally:
        L.tg_tree_free(t)
    stream.synchronize()
    return out[0].cpu().numpy(), out[1].cpu().numpy()


def test_threads_on_their_own_streams(env):
    torch, _lib, L, synthetic, theta = env
    model = theta.ThetaModel.load()
    mh = model.handle()
    l10 = float(theta.default_lambda(model, True))
    inputs, alone = [], []
    for k in range(THREADS):
        x = synthetic.plummer(N, 100 + k)
        args = tuple(torch.from_numpy(a).cuda() for a in (x, np.full(N, 1.0 / N), np.full(N, 0.005)))
        out = (torch.empty((N, 3), dtype=torch.float64, device="cuda"),
               torch.empty((N, 3), dtype=torch.float64, device="cuda"))
        s = torch.cuda.Stream()
        inputs.append((args, out, s))
        alone.append(one_step(torch, _lib, L, *args, out, s, mh, l10))
    errors, results = [], [[None] * ROUNDS for _ in range(THREADS)]
    barrier = threading.Barrier(THREADS)

    def work(k):
        try:
            torch.cuda.set_device(0)
            args, out, s = inputs[k]
            barrier.wait()
            for r in range(ROUNDS):
                results[k][r] = one_step(torch, _lib, L, *args, out, s, mh, l10)
        except Exception as e:  # reported below
            errors.append((k, repr(e)))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(THREADS)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=300)
    model.close()
    assert not errors, errors
    for k in range(THREADS):
        for r in range(ROUNDS):
            plain, learned = results[k][r]
            assert np.array_equal(plain, alone[k][0]), (k, r)
            assert np.array_equal(learned, alone[k][1]), (k, r)
