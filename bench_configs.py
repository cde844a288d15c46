"""The benchmark's other configurations, one JSON line each (``python bench.py --config NAME``).

* ``uniform``: N = 1e5 uniform in the unit cube (float64, seeded), m = 1/N, h = 0.01, theta = 0.7,
  monopole; Accel and Potential via method='tree', judged by method='bruteforce' on a 1e4-target
  subset.
* ``precision``: N = 1e6 Plummer sphere (a = 1, r < 50), m = 1/N, h = 0.005, quadrupole, theta in
  {0.4, 0.7}; FP32 walk with FP64 tree and moments; Accel, Potential and the tidal tensor; RMS/max
  error against FP64 brute force on 1e4 sampled targets.
* ``clustered``: N = 4e6 mixture of 64 Plummer subclusters (centres uniform in a cube of side 20,
  scale radii lognormal mu = ln 0.3, sigma = 0.5, Dirichlet(1) member counts), m = 1/N, h = 0.002,
  quadrupole; the learned acceptance test and the plain walk each tuned to an RMS force error of
  1e-3 against FP64 brute force (1e4 sampled targets), then timed at that equal error.
* ``largest``: AccelTarget/PotentialTarget with 3.2e7 Plummer sources (float32 positions, m = 1/N,
  softenings lognormal mu = ln 0.003, sigma = 0.7) and 2e6 uniform targets in the ball r < 5; the
  learned walk for external targets (plain-theta fallback for groups over the error budget) next to
  the plain theta = 0.7 walk on the same target groups; errors against FP32 Kahan-compensated direct
  sums, over all sources on 1e4 sampled targets and over a 2e5-source subset.
* ``corr``: VelocityStructFunc with pytreegrav's defaults on N = 1e6 Plummer particles with velocities
  (0.3 x + unit normal noise): tree build, velocity moments and the FP64 walk of every particle.
* ``build``: the octree build alone (quadrupole moments) of the headline's 1e6 Plummer sphere, from
  device arrays: build time, particles/s, and the build's algorithmic bytes per second against the
  measured HBM copy rate.

Every input is seeded synthetic data with the configuration's shapes and distributions. Steps are
timed with CUDA events on the launching stream, inputs resident in HBM, L2 flushed (256 MiB
written) between timed steps outside the events.
"""

import ctypes
import json
import os
import statistics
import time

import numpy as np

SEED = 20261203
FLOPS = {"mono_acc": 18, "quad_acc": 56}  # algorithmic FP32 flops per interaction (see bench.py)


def _env():
    import torch

    from pytreegrav_gb300 import _lib

    L = _lib.load()
    L.tg_tree_last_walk_kernel_ms.restype = ctypes.c_double
    L.tg_tree_last_walk_kernel_ms.argtypes = [ctypes.c_void_p]
    L.tg_tree_last_walk_quad_interactions.restype = ctypes.c_int64
    L.tg_tree_last_walk_quad_interactions.argtypes = [ctypes.c_void_p]
    L.tg_launch_count.restype = ctypes.c_int64
    L.tg_launch_count.argtypes = []
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return torch, _lib, L, st


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def timed(torch, step, steps, warmup):
    """Mean CUDA-event time of `step` (ms) over `steps` runs after `warmup`, L2 flushed before each."""
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    res = []
    for a, b in ev:
        flush.zero_()
        a.record()
        res.append(step())
        b.record()
    torch.cuda.synchronize()
    return statistics.mean(a.elapsed_time(b) for a, b in ev), res


def errs(a, ref):
    """(RMS, max) per-target error norm relative to the RMS norm of ref."""
    a, ref = np.asarray(a).reshape(len(a), -1), np.asarray(ref).reshape(len(ref), -1)
    d = np.sqrt(np.sum((a - ref) ** 2, 1))
    s = np.sqrt(np.mean(np.sum(ref**2, 1)))
    return {"rms": float(np.sqrt(np.mean(d**2)) / s), "max": float(d.max() / s)}


def pot_errs(p, ref):
    d = (p - ref) - np.mean(p - ref)
    return {"rms": float(np.std(p - ref) / np.std(ref)), "max": float(np.abs(d).max() / np.std(ref))}


def walk_stats(L, h):
    v = [ctypes.c_int64() for _ in range(4)]
    L.tg_tree_last_walk_stats(h, *[ctypes.byref(x) for x in v])
    return {"interactions": v[0].value, "quad_interactions": L.tg_tree_last_walk_quad_interactions(h),
            "kernel_ms": L.tg_tree_last_walk_kernel_ms(h), "groups": v[3].value}


def flops_of(s, quad):
    q = s["quad_interactions"] if quad else 0
    return FLOPS["mono_acc"] * (s["interactions"] - q) + FLOPS["quad_acc"] * q


def build(L, _lib, st, dx, dm, dh, n, quad):
    h = ctypes.c_void_p()
    _lib.check(L.tg_tree_build(_vp(dx), _vp(dm), _vp(dh), n, int(quad), 1, _lib.TG_MEM_DEVICE, st, ctypes.byref(h)),
               "build")
    return h


def fp32_peak(L, st):
    L.tg_measure_fp32_fma.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                      ctypes.c_void_p]
    tf, ms = ctypes.c_double(), ctypes.c_double()
    L.tg_measure_fp32_fma(ctypes.byref(tf), ctypes.byref(ms), st)
    return tf.value


# The build's algorithmic bytes: 638 B per particle and 969 B per node, summed over its kernels (keys,
# eight sort passes, gather, split round, numbering sort, final arrays, moment pass; the per-kernel
# figures are in profiles/build_plummer1e6.md).
BUILD_BYTES_PER_PARTICLE, BUILD_BYTES_PER_NODE = 638, 969


def build_roofline(n, nodes, build_ms):
    alg = BUILD_BYTES_PER_PARTICLE * n + BUILD_BYTES_PER_NODE * nodes
    hbm = None
    try:
        hbm = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json"))).get(
            "hbm_gbs")
    except Exception:
        pass
    gbs = alg / (build_ms * 1e-3) / 1e9
    return {"ms": round(build_ms, 4), "nodes": nodes, "algorithmic_bytes": alg, "achieved_gbs": round(gbs, 1),
            "hbm_peak_gbs": hbm, "frac_of_hbm": round(gbs / hbm, 4) if hbm else None,
            "bound": "latency at this size (dependent launches) and FP64 issue in the moment pass; per-kernel "
                     "traffic in profiles/build_plummer1e6.md"}


def ball(n, seed, radius=5.0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return np.ascontiguousarray(d * (radius * rng.random(n) ** (1 / 3))[:, None])


# ---------------------------------------------------------------------------------------------


def run_uniform(args):
    torch, _lib, L, st = _env()
    import pytreegrav_gb300 as tg
    from oracle import oracle as O

    n = 100_000
    x = np.random.default_rng(0).random((n, 3))
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    dx, dm, dh = (torch.from_numpy(a).cuda() for a in (x, m, h))
    out = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    fields = _lib.TG_FIELD_POTENTIAL | _lib.TG_FIELD_ACCEL
    res = {}
    for grouping, gs in (("blocks", 8), ("tree", 32)):
        gcode = _lib.TG_GROUP_BLOCKS if grouping == "blocks" else _lib.TG_GROUP_TREE

        def step():
            t = build(L, _lib, st, dx, dm, dh, n, False)
            _lib.check(L.tg_tree_fields(t, None, None, n, fields, 0, 0.7, 1.0, gs, gcode, _lib.TG_ORDER_TREE,
                                        _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, _vp(out), st), "walk")
            s = walk_stats(L, t)
            L.tg_tree_free(t)
            return s

        ms, stats = timed(torch, step, args.steps, args.warmup)
        res[grouping] = {"ms_per_step": round(ms, 4), "value": round(n / (ms * 1e-3), 1), "group_size": gs,
                         "walk_kernel_ms": round(statistics.mean(s["kernel_ms"] for s in stats), 4),
                         "interactions_per_target": stats[-1]["interactions"] / n, "out": out.cpu().numpy().copy()}
    sub = np.random.default_rng(1).choice(n, 10_000, replace=False)
    bf = tg.bruteforce(x[sub], h[sub], x, m, h, potential=True, accel=True, precision="fp64")
    for r in res.values():
        o = r.pop("out")
        r["accuracy_vs_fp64_bruteforce"] = {"accel": errs(o[sub, 1:], bf["accel"]),
                                            "potential": pot_errs(o[sub, 0], bf["potential"])}
    # end to end: the public calls a pytreegrav user makes, from host arrays
    tg.Accel(x, m, h, method="tree")
    e2e = []
    for _ in range(5):
        t0 = time.perf_counter()
        tg.Accel(x, m, h, theta=0.7, method="tree")
        tg.Potential(x, m, h, theta=0.7, method="tree")
        e2e.append(time.perf_counter() - t0)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ot = O.OracleTree(x, m, h)
    idx = ot.TreewalkIndices
    ot.fields(x[idx], h[idx], potential=True, accel=True, group_size=8, theta=0.7, nthreads=cores)
    cpu_s = time.perf_counter() - t0
    return {"metric": "Accel+Potential particles/s, 1e5 uniform cube", "value": res["blocks"]["value"],
            "unit": "particles/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["blocks"]["ms_per_step"], "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded uniform cube, float64)",
            "config": {"workload": "N=1e5 uniform in the unit cube, m=1/N, h=0.01, theta=0.7, monopole, Accel and "
                                   "Potential from one walk (FP32 interactions, FP64 tree)",
                       "step": "tree build + walk, inputs resident in HBM", "l2": "flushed between timed steps"},
            "groupings": res,
            "e2e": {"value": round(n / statistics.median(e2e), 1), "unit": "particles/s",
                    "api": "Accel(x, m, h, method='tree') then Potential(x, m, h, method='tree')",
                    "h2d_bytes_per_step": int(2 * (x.nbytes + m.nbytes + h.nbytes)),
                    "d2h_bytes_per_step": int(8 * 4 * n), "ms_per_step": round(1e3 * statistics.median(e2e), 3)},
            "cpu_baseline": {"value": round(n / cpu_s, 1), "unit": "particles/s", "cores": cores, "kind": "port",
                             "sample": f"one full step: oracle build + FP64 walk of all N (groups of 8), {cpu_s:.2f} s"}}


def run_precision(args):
    torch, _lib, L, st = _env()
    import pytreegrav_gb300 as tg

    from bench import plummer

    n = 1_000_000
    x = plummer(n, SEED)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.005)
    dx, dm, dh = (torch.from_numpy(a).cuda() for a in (x, m, h))
    out = torch.empty((n, 13), dtype=torch.float64, device="cuda")
    sub = np.random.default_rng(7).choice(n, 10_000, replace=False)
    bf = tg.bruteforce(x[sub], h[sub], x, m, h, potential=True, accel=True, tidal=True, precision="fp64")
    peak = fp32_peak(L, st)
    res = {}
    for theta in (0.4, 0.7):
        for grouping, gs in (("blocks", 8), ("tree", 32)):
            gcode = _lib.TG_GROUP_BLOCKS if grouping == "blocks" else _lib.TG_GROUP_TREE

            def step(fields=7):
                t = build(L, _lib, st, dx, dm, dh, n, True)
                _lib.check(L.tg_tree_fields(t, None, None, n, fields, 1, theta, 1.0, gs, gcode, _lib.TG_ORDER_TREE,
                                            _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, _vp(out), st), "walk")
                s = walk_stats(L, t)
                L.tg_tree_free(t)
                return s

            ms, stats = timed(torch, step, max(3, args.steps // 3), args.warmup)
            o = out.cpu().numpy()
            # the acceleration alone, for its FP32 rate at the counted flops
            ms_a, st_a = timed(torch, lambda: step(_lib.TG_FIELD_ACCEL), max(3, args.steps // 3), 1)
            s_a = st_a[-1]
            kms = statistics.mean(s["kernel_ms"] for s in st_a)
            res[f"theta_{theta}_{grouping}"] = {
                "group_size": gs, "all_fields": {"ms_per_step": round(ms, 3), "value": round(n / (ms * 1e-3), 1),
                                                 "walk_kernel_ms": round(statistics.mean(s["kernel_ms"] for s in stats), 3)},
                "accel_only": {"ms_per_step": round(ms_a, 3), "value": round(n / (ms_a * 1e-3), 1),
                               "walk_kernel_ms": round(kms, 3),
                               "interactions_per_target": s_a["interactions"] / n,
                               "interactions_per_s": round(s_a["interactions"] / (kms * 1e-3), 1),
                               "fp32_frac_of_probe_peak": round(flops_of(s_a, True) / (kms * 1e-3) / 1e12 / peak, 4)},
                "accuracy_vs_fp64_bruteforce": {"accel": errs(o[sub, 1:4], bf["accel"]),
                                                "potential": pot_errs(o[sub, 0], bf["potential"]),
                                                "tidal": errs(o[sub, 4:], bf["tidal"].reshape(-1, 9))}}
    r = res["theta_0.7_blocks"]["all_fields"]
    return {"metric": "Accel+Potential+tidal particles/s, 1e6 Plummer (precision form)", "value": r["value"],
            "unit": "particles/s", "n_gpus": 1, "steps": max(3, args.steps // 3), "warmup": args.warmup,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded Plummer sphere, a=1, r<50)",
            "config": {"workload": "N=1e6 Plummer, m=1/N, h=0.005, quadrupole, theta in {0.4, 0.7}, FP32 walk with FP64 "
                                   "tree and moments; potential, acceleration and tidal tensor from one walk",
                       "headline": "theta=0.7, pytreegrav's grouping (8 consecutive targets)",
                       "step": "tree build + walk, inputs resident in HBM", "l2": "flushed between timed steps",
                       "judge": "FP64 brute force on 1e4 sampled targets; accel by rms|a|, potential by std(phi), "
                                "tidal by rms|T|"},
            "fp32_probe_peak_tflops": round(peak, 3), "results": res}


def run_clustered(args):
    torch, _lib, L, st = _env()
    import pytreegrav_gb300 as tg
    from pytreegrav_gb300 import synthetic
    from pytreegrav_gb300 import theta as th

    n = 4_000_000
    target = 1e-3
    x = synthetic.clustered(n, SEED + 4)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.002)
    dx, dm, dh = (torch.from_numpy(a).cuda() for a in (x, m, h))
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    sub = np.random.default_rng(11).choice(n, 10_000, replace=False)
    dsub = torch.from_numpy(sub).cuda()
    ref = tg.bruteforce(x[sub], h[sub], x, m, h, accel=True, precision="fp64")["accel"]
    model = th.ThetaModel.load()
    mh = model.handle()

    def walk(t, kind, v):
        if kind == "plain":
            _lib.check(L.tg_tree_fields(t, None, None, n, _lib.TG_FIELD_ACCEL, 1, float(v), 1.0, 32, _lib.TG_GROUP_TREE,
                                        _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, _vp(out), st),
                       "walk")
        else:
            _lib.check(L.tg_tree_fields_learned(t, _lib.TG_FIELD_ACCEL, 1, 1.0, 32, mh, float(v), 0.7,
                                                _lib.TG_MEM_DEVICE, _vp(out), st), "learned walk")

    def err_of(kind, v, t):
        walk(t, kind, v)
        return errs(out.index_select(0, dsub).cpu().numpy(), ref)["rms"], walk_stats(L, t)

    t = build(L, _lib, st, dx, dm, dh, n, True)
    scan = {"plain": [], "learned": []}
    for v in np.round(np.arange(0.4, 1.0001, 0.05), 3):
        e, s = err_of("plain", v, t)
        scan["plain"].append((float(v), e, s["interactions"] / n))
    for v in np.round(np.arange(-1.5, 2.5001, 0.25), 3):
        e, s = err_of("learned", v, t)
        scan["learned"].append((float(v), e, s["interactions"] / n))
    L.tg_tree_free(t)
    # the cheapest setting of each within the target error (plain: largest theta; learned: smallest lambda)
    ok_p = [r for r in scan["plain"] if r[1] <= target]
    ok_l = [r for r in scan["learned"] if r[1] <= target]
    theta_eq = max(ok_p, key=lambda r: r[0])[0] if ok_p else min(r[0] for r in scan["plain"])
    lam_eq = min(ok_l, key=lambda r: r[0])[0] if ok_l else max(r[0] for r in scan["learned"])

    def step(kind, v):
        t = build(L, _lib, st, dx, dm, dh, n, True)
        walk(t, kind, v)
        s = walk_stats(L, t)
        L.tg_tree_free(t)
        return s

    ms_p, sp = timed(torch, lambda: step("plain", theta_eq), args.steps, args.warmup)
    e_p = errs(out.index_select(0, dsub).cpu().numpy(), ref)
    ms_l, sl = timed(torch, lambda: step("learned", lam_eq), args.steps, args.warmup)
    e_l = errs(out.index_select(0, dsub).cpu().numpy(), ref)
    ms_07, s07 = timed(torch, lambda: step("plain", 0.7), args.steps, args.warmup)
    e_07 = errs(out.index_select(0, dsub).cpu().numpy(), ref)
    kp = statistics.mean(s["kernel_ms"] for s in sp)
    kl = statistics.mean(s["kernel_ms"] for s in sl)
    return {"metric": "Accel particles/s, 4e6 clustered mixture: learned vs plain at RMS force error 1e-3",
            "value": round(n / (ms_l * 1e-3), 1), "unit": "particles/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_l, 3), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded mixture of 64 Plummer subclusters)",
            "config": {"workload": "N=4e6 clustered mixture, m=1/N, h=0.002, quadrupole, FP32 walk, tree grouping 32",
                       "equal_error": f"each variant at its cheapest setting with RMS force error <= {target} against "
                                      "FP64 brute force on 1e4 sampled targets (plain: theta scanned in 0.05 steps; "
                                      "learned: log10 lambda in 0.25 steps)",
                       "step": "tree build + walk, inputs resident in HBM", "l2": "flushed between timed steps"},
            "learned": {"log10_lambda": lam_eq, "accuracy": e_l, "ms_per_step": round(ms_l, 3),
                        "walk_kernel_ms": round(kl, 3), "interactions_per_target": sl[-1]["interactions"] / n},
            "plain_equal_error": {"theta": theta_eq, "accuracy": e_p, "ms_per_step": round(ms_p, 3),
                                  "value": round(n / (ms_p * 1e-3), 1), "walk_kernel_ms": round(kp, 3),
                                  "interactions_per_target": sp[-1]["interactions"] / n},
            "plain_theta_0.7": {"accuracy": e_07, "ms_per_step": round(ms_07, 3),
                                "walk_kernel_ms": round(statistics.mean(s["kernel_ms"] for s in s07), 3),
                                "interactions_per_target": s07[-1]["interactions"] / n},
            "speedup_vs_plain_equal_error": {"step": round(ms_p / ms_l, 3), "walk": round(kp / kl, 3)},
            "scan": scan}


def run_largest(args):
    torch, _lib, L, st = _env()
    import pytreegrav_gb300 as tg
    from oracle import oracle as O
    from pytreegrav_gb300 import synthetic
    from pytreegrav_gb300 import theta as th

    ns = int(args.sources)
    nt = ns // 16
    x = synthetic.plummer(ns, SEED + 5).astype(np.float32).astype(np.float64)
    m = np.full(ns, 1.0 / ns)
    h = np.exp(np.random.default_rng(SEED + 6).normal(np.log(0.003), 0.7, ns))
    xt = ball(nt, SEED + 7)
    ht = np.zeros(nt)
    dx, dm, dh, dxt, dht = (torch.from_numpy(a).cuda() for a in (x, m, h, xt, ht))
    out = torch.empty((nt, 4), dtype=torch.float64, device="cuda")
    fields = _lib.TG_FIELD_POTENTIAL | _lib.TG_FIELD_ACCEL
    model = th.ThetaModel.load()
    mh = model.handle()
    l10 = th.default_lambda(model, True, targets=True)

    def step(learned):
        t = build(L, _lib, st, dx, dm, dh, ns, True)
        ts = ctypes.c_void_p()
        _lib.check(L.tg_targets_create(t, _vp(dxt), _vp(dht), nt, 32, _lib.TG_MEM_DEVICE, st, ctypes.byref(ts)),
                   "target set")
        if learned:
            _lib.check(L.tg_targets_fields_learned(ts, fields, 1, 1.0, mh, float(l10), 0.7, _lib.TG_MEM_DEVICE,
                                                   _vp(out), st), "learned target walk")
        else:
            _lib.check(L.tg_targets_fields(ts, fields, 1, 0.7, 1.0, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, _vp(out),
                                           st), "target walk")
        s = walk_stats(L, t)
        L.tg_targets_free(ts)
        L.tg_tree_free(t)
        return s

    steps = max(3, min(args.steps, 10))
    l0 = L.tg_launch_count()
    ms_l, sl = timed(torch, lambda: step(True), steps, args.warmup)
    launches = L.tg_launch_count() - l0
    o_l = out.cpu().numpy().copy()
    ms_p, sp = timed(torch, lambda: step(False), steps, args.warmup)
    o_p = out.cpu().numpy().copy()
    # judges: FP32 Kahan-compensated direct sums (tg_bruteforce FP32)
    samp = np.random.default_rng(SEED + 8).choice(nt, 10_000, replace=False)
    bf = tg.bruteforce(xt[samp], ht[samp], x, m, h, potential=True, accel=True, precision="fp32")

    def acc(o):
        return {"accel": errs(o[samp, 1:], bf["accel"]), "potential": pot_errs(o[samp, 0], bf["potential"])}

    acc_l, acc_p = acc(o_l), acc(o_p)
    # the 2e5-source subset, masses scaled to the same total: learned and plain against its direct sum
    k = 200_000
    si = np.random.default_rng(SEED + 9).choice(ns, k, replace=False)
    xs, ms_, hs = x[si], np.full(k, 1.0 / k), h[si]
    sub_tree = tg.ConstructTree(xs, ms_, hs, quadrupole=True)
    sub_ts = tg.TargetSet(sub_tree, xt[samp], ht[samp])
    bf_s = tg.bruteforce(xt[samp], ht[samp], xs, ms_, hs, accel=True, precision="fp32")["accel"]
    sub_acc = {"learned": errs(sub_ts.fields_learned(accel=True, quadrupole=True, theta=0.7)["accel"], bf_s),
               "plain": errs(sub_ts.fields(accel=True, quadrupole=True, theta=0.7)["accel"], bf_s)}
    sub_ts.close()
    # end to end: the public target calls on pinned host arrays (one tree build, two walks)
    pins = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True) for a in (x, m, h, xt, ht)]
    for p, a in zip(pins, (x, m, h, xt, ht)):
        p.numpy()[:] = a
    px, pm, ph, pxt, pht = (p.numpy() for p in pins)
    kw = dict(theta=0.7, quadrupole=True, method="tree", learned=True)
    e2e = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a, tree = tg.AccelTarget(pxt, px, pm, pht, ph, return_tree=True, **kw)
        p = tg.PotentialTarget(pxt, None, None, pht, tree=tree, **kw)
        torch.cuda.synchronize()
        e2e.append(time.perf_counter() - t0)
        del tree
    # CPU baseline: the oracle's build of all sources + the FP64 walk of every 64th block of 8 targets
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ot = O.OracleTree(x, m, h, quadrupole=True)
    t1 = time.perf_counter()
    ts_ = O.morton_order(xt)
    starts = np.arange(0, nt, 8 * 64, dtype=np.int64)
    counts = np.minimum(8, nt - starts)
    O.fields_groups(ot, xt[ts_], ht[ts_], starts, counts, potential=True, accel=True, quadrupole=True, theta=0.7,
                    nthreads=cores)
    t2 = time.perf_counter()
    cpu_s = (t1 - t0) + (t2 - t1) * nt / counts.sum()
    peak = fp32_peak(L, st)
    s = sl[-1]
    kl = statistics.mean(v["kernel_ms"] for v in sl)
    kp = statistics.mean(v["kernel_ms"] for v in sp)
    return {"metric": "AccelTarget+PotentialTarget targets/s, 3.2e7 Plummer sources, 2e6 targets (learned walk)",
            "value": round(nt / (ms_l * 1e-3), 1), "unit": "targets/s", "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "ms_per_step": round(ms_l, 3), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded Plummer sources, float32 positions; uniform targets in a ball)",
            "config": {"workload": f"{ns} Plummer sources (m=1/N, h lognormal mu=ln 0.003 sigma=0.7, quadrupole), "
                                   f"{nt} uniform targets in r<5; potential and acceleration from one walk, FP32",
                       "step": "source tree build + target set (the targets' own octree and grouping) + learned "
                               "walk; inputs resident in HBM", "l2": "flushed between timed steps"},
            "learned": {"ms_per_step": round(ms_l, 3), "walk_kernel_ms": round(kl, 3),
                        "interactions_per_target": s["interactions"] / nt, "accuracy_vs_fp32_compensated_direct_sum":
                        acc_l, "log10_lambda": l10},
            "plain": {"ms_per_step": round(ms_p, 3), "value": round(nt / (ms_p * 1e-3), 1),
                      "walk_kernel_ms": round(kp, 3), "interactions_per_target": sp[-1]["interactions"] / nt,
                      "accuracy_vs_fp32_compensated_direct_sum": acc_p},
            "speedup_vs_plain": {"step": round(ms_p / ms_l, 3), "walk": round(kp / kl, 3)},
            "subset_2e5_sources": {"targets": len(samp), "rms_vs_fp32_compensated_direct_sum": sub_acc},
            "roofline": {"bound": "fp32", "achieved": round(flops_of(s, True) / (kl * 1e-3) / 1e12, 3),
                         "peak": round(peak, 3), "unit": "TFLOP/s",
                         "frac": round(flops_of(s, True) / (kl * 1e-3) / 1e12 / peak, 4), "kernel": "k_walk",
                         "interactions_per_s": round(s["interactions"] / (kl * 1e-3), 1)},
            "e2e": {"value": round(nt / statistics.median(e2e), 1), "unit": "targets/s",
                    "api": "AccelTarget(xt, x, m, ht, h, learned=True, return_tree=True) then "
                           "PotentialTarget(xt, None, None, ht, tree=tree, learned=True)",
                    "h2d_bytes_per_step": int(x.nbytes + m.nbytes + h.nbytes + 2 * (xt.nbytes + ht.nbytes)),
                    "d2h_bytes_per_step": int(8 * 4 * nt), "ms_per_step": round(1e3 * statistics.median(e2e), 3)},
            "cpu_baseline": {"value": round(nt / cpu_s, 1), "unit": "targets/s", "cores": cores, "kind": "port",
                             "sample": f"oracle build of all {ns} sources ({t1 - t0:.1f} s) + FP64 walk of every 64th "
                                       f"block of 8 Morton-ordered targets, walk time scaled to all {nt}: "
                                       f"{cpu_s:.1f} s per step"},
            "gpu_launches_per_step": int(launches / (steps + args.warmup))}


def run_corr(args):
    """VelocityStructFunc on 1e6 Plummer particles with velocities (0.3 x + unit normal noise, seeded),
    pytreegrav's defaults: rbins from the N^(1/3) heuristic, theta = 1, max_bin_size_ratio = 100,
    jittered binning. A step is the tree build, the node velocity moments and the FP64 walk of all N
    targets (the tree's own particles), inputs resident in HBM; e2e is the public call from host arrays."""
    import pytreegrav_gb300 as tg
    from oracle import oracle as O
    from pytreegrav_gb300.frontend import _default_rbins

    torch, _lib, L, st = _env()
    n = args.n
    rng = np.random.default_rng(SEED + 5)
    import bench

    x = bench.plummer(n, SEED)
    m = np.full(n, 1.0 / n)
    v = 0.3 * x + rng.normal(size=(n, 3))
    rb = _default_rbins(x)
    nb = len(rb) - 1
    dx, dm, dv, drb = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (x, m, v, rb))
    dz = torch.zeros(n, dtype=torch.float64, device="cuda")
    bins = torch.zeros(2 * nb, dtype=torch.float64, device="cuda")
    vp = ctypes.c_void_p
    walk_ev = []

    def step():
        t = vp()
        _lib.check(L.tg_tree_build(_vp(dx), _vp(dm), _vp(dz), n, 0, 1, _lib.TG_MEM_DEVICE, st, ctypes.byref(t)), "build")
        _lib.check(L.tg_tree_set_velocities(t, _vp(dv), _lib.TG_MEM_DEVICE, st), "velocities")
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        _lib.check(L.tg_tree_correlation(t, _lib.TG_CORR_KINDS["structure"], None, None, None, 0, _vp(drb), nb, 100.0,
                                         1.0, 0.0, 0, 12345, _lib.TG_MEM_DEVICE, _vp(bins),
                                         vp(bins.data_ptr() + 8 * nb), st), "correlation")
        b.record()
        walk_ev.append((a, b))
        L.tg_tree_free(t)

    l0 = L.tg_launch_count()
    steps = max(3, min(args.steps, 10))
    ms, _ = timed(torch, step, steps, args.warmup)
    launches = (L.tg_launch_count() - l0) // (steps + args.warmup)
    walk_ms = statistics.mean(a.elapsed_time(b) for a, b in walk_ev[-steps:])
    sv = (bins[:nb] / bins[nb:]).cpu().numpy()
    # end to end through the public call
    tg.VelocityStructFunc(x, m, v, seed=12345)
    e2e_t = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, sv_e2e = tg.VelocityStructFunc(x, m, v, seed=12345)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    # CPU baseline: the oracle (pytreegrav's walk in C, FP64, OpenMP on all host cores): build and
    # moments of all N, the walk of every 64th target, extrapolated
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ot = O.OracleTree(x, m, np.zeros(n))
    otv = O.tree_velocities(ot, v)
    t1 = time.perf_counter()
    idx = ot.TreewalkIndices[::64]
    O.correlation(ot, "structure", x[idx], rb, vel=v[idx], weight=m[idx], tree_vel=otv, theta=1.0, seed=12345,
                  nthreads=cores)
    t2 = time.perf_counter()
    cpu_s = (t1 - t0) + (t2 - t1) * 64
    return {"metric": "VelocityStructFunc targets/s, 1e6 Plummer with velocities (pytreegrav defaults)",
            "value": round(n / (ms * 1e-3), 1), "unit": "targets/s", "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded Plummer sphere a=1 r<50; velocities 0.3 x + N(0,1))",
            "config": {"workload": f"VelocityStructFunc, N={n}, m=1/N, {nb} log bins from the N^(1/3) heuristic, "
                                   "theta=1, max_bin_size_ratio=100, jittered binning",
                       "step": "tree build + node velocity moments + FP64 walk of all N targets, inputs resident in HBM",
                       "l2": "flushed between timed steps"},
            "walk_ms": round(walk_ms, 3), "walk_targets_per_s": round(n / (walk_ms * 1e-3), 1),
            "same_as_e2e_call": bool(np.allclose(sv, sv_e2e, rtol=1e-12, equal_nan=True)),
            "e2e": {"value": round(n / e2e_s, 1), "unit": "targets/s",
                    "h2d_bytes_per_step": int(x.nbytes + m.nbytes + v.nbytes + rb.nbytes),
                    "d2h_bytes_per_step": int(16 * nb), "api": "pytreegrav_gb300.VelocityStructFunc(pos, m, v, seed=...)",
                    "ms_per_step": round(1e3 * e2e_s, 3)},
            "cpu_baseline": {"value": round(n / cpu_s, 1), "unit": "targets/s", "cores": cores, "kind": "port",
                             "sample": "oracle build and velocity moments of all N + the structure-function walk "
                                       f"(C, FP64, OpenMP) of every 64th target, extrapolated; {cpu_s:.2f} s per step"},
            "gpu_launches": int(launches)}


def run_build(args):
    """The octree build alone (see the module docstring)."""
    torch, _lib, L, st = _env()
    import bench

    n = args.n
    x = bench.plummer(n, SEED)
    dx = torch.from_numpy(x).cuda()
    dm = torch.from_numpy(np.full(n, 1.0 / n)).cuda()
    dh = torch.from_numpy(np.full(n, bench.SOFT)).cuda()
    nodes = [0]

    def step():
        h = build(L, _lib, st, dx, dm, dh, n, True)
        info = _lib.TreeInfo()
        L.tg_tree_info_get(h, ctypes.byref(info))
        nodes[0] = int(info.node_hi) - n
        L.tg_tree_free(h)

    l0 = L.tg_launch_count()
    ms, _ = timed(torch, step, args.steps, args.warmup)
    launches = (L.tg_launch_count() - l0) // (args.steps + args.warmup)
    roof = build_roofline(n, nodes[0], ms)
    return {"metric": f"octree build particles/s, {n:.2g}-particle Plummer sphere (quadrupole moments)",
            "value": round(n / (ms * 1e-3), 1),
            "unit": "particles/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Plummer sphere, a=1, r<50)",
            "config": {"workload": f"tg_tree_build of N={n} Plummer particles (m=1/N, h={bench.SOFT}) from device arrays, "
                                   "quadrupole moments", "l2": "flushed (256 MiB written) before each step"},
            "build": roof, "gpu_launches": launches}
