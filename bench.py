"""Benchmark: Accel particles/s on a 1e6-particle Plummer sphere (GB300).

One step = build the octree of 1e6 Plummer particles (a=1, r<50, m=1/N, h=0.005, quadrupoles) on
the GPU and evaluate the acceleration of every particle with the FP32 grouped walk at theta=0.7,
inputs resident in HBM. Prints one JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores (the C restatement under oracle/,
all threads): pytreegrav's own implementation is numba-compiled Python and numba is absent here.
Multi-GPU runs are independent replicas (one system per rank, no collective in the data path).
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Accel particles/s, 1e6 Plummer: learned-θ vs plain walk at same RMS force error"
UNIT = "particles/s"
N_DEFAULT = 1_000_000
THETA = 0.7
SOFT = 0.005
GROUP = 32
SEED = 20261203

# FP32 flops per interaction: the algorithmic count of the interaction as the monopole and
# quadrupole terms are written (pytreegrav_gb300/csrc/tg_walk.cu, point_mass and quad_terms, which
# the walk evaluates for potential and tidal fields), with add/sub/mul = 1, FMA = 2, rsqrt = 1:
#   monopole acceleration: 3 sub + r^2 (1 mul + 2 fma) + rsqrt + rinv^2, m*rinv, *rinv^2 (3 mul)
#   + 3 fma = 18; quadrupole node, acceleration: +38 (Q.dx 15, A 5, r^-5 and r^-7 4, 2.5*A*r^-7 2,
#   three components of qf*dx - qdx*r^-5 accumulated, 12).
# The fused FP32 acceleration sweep computes the same quantities in fewer operations (48 for a
# quadrupole node); the fixed algorithmic count keeps rates comparable across kernel versions.
FLOPS_MONO_ACC = 18
FLOPS_QUAD_ACC = 18 + 38


def plummer(n, seed):
    """Plummer sphere, a=1, truncated at r<50, isotropic directions (seeded)."""
    rng = np.random.default_rng(seed)
    out = np.empty((0, 3))
    while len(out) < n:
        k = n - len(out)
        u = rng.random(k)
        r = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        d = rng.normal(size=(k, 3))
        p = d / np.linalg.norm(d, axis=1)[:, None] * r[:, None]
        out = np.vstack([out, p[r < 50]])
    return np.ascontiguousarray(out[:n])


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi sampling (every 20 ms, timestamped) around the timed region; only the samples
    taken inside the region (or, for a region shorter than the interval, the nearest ones) count."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"tg_clocks_{os.getpid()}.csv")
        self.t_begin = self.t_end = None

    def start(self):
        """Start sampling; returns once it is underway."""
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.5)

    def begin(self):
        self.t_begin = time.time()

    def end(self):
        self.t_end = time.time()

    def stop(self):
        import datetime

        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                continue
            rows.append((t, parts[1:]))
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        inside = [r for t, r in rows if self.t_begin is None or self.t_begin <= t <= self.t_end]
        if not inside:  # region shorter than the interval: the samples just before and after it
            inside = [r for t, r in rows if t < self.t_begin][-1:] + [r for t, r in rows if t > self.t_end][:1]
        sm = [float(r[1]) for r in inside if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in inside if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


def read_traffic():
    """DRAM bytes per walk launch from the committed ncu summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", "walk_plummer1e6.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip().split()[0]))
            except ValueError:
                return None
    return None


def _bind(L):
    i64, dbl, vp = ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
    L.tg_launch_count.restype = i64
    L.tg_launch_count.argtypes = []
    L.tg_measure_fp32_fma.argtypes = [ctypes.POINTER(dbl), ctypes.POINTER(dbl), vp]
    L.tg_tree_last_walk_kernel_ms.restype = dbl
    L.tg_tree_last_walk_kernel_ms.argtypes = [vp]
    L.tg_tree_last_walk_quad_interactions.restype = i64
    L.tg_tree_last_walk_quad_interactions.argtypes = [vp]
    return L


def gpu_step(L, _lib, dpos, dm, dh, out, n, stream, model=None, log10_lambda=0.0):
    """One step on device-resident arrays: build + FP32 quadrupole Accel walk (tree grouping), with
    the learned acceptance test when `model` (a library model handle) is given, else plain theta."""
    vp = ctypes.c_void_p
    h = vp()
    rc = L.tg_tree_build(vp(dpos.data_ptr()), vp(dm.data_ptr()), vp(dh.data_ptr()), n, 1, 1, _lib.TG_MEM_DEVICE,
                         vp(stream), ctypes.byref(h))
    _lib.check(rc, "build")
    if model is not None:
        rc = L.tg_tree_fields_learned(h, _lib.TG_FIELD_ACCEL, 1, 1.0, GROUP, model, float(log10_lambda), THETA,
                                      _lib.TG_MEM_DEVICE, vp(out.data_ptr()), vp(stream))
    else:
        rc = L.tg_tree_fields(h, None, None, n, _lib.TG_FIELD_ACCEL, 1, THETA, 1.0, GROUP, _lib.TG_GROUP_TREE,
                              _lib.TG_ORDER_TREE, _lib.TG_FP32, None, _lib.TG_MEM_DEVICE, vp(out.data_ptr()), vp(stream))
    _lib.check(rc, "walk")
    v = [ctypes.c_int64() for _ in range(4)]
    L.tg_tree_last_walk_stats(h, *[ctypes.byref(x) for x in v])
    st = {"interactions": v[0].value, "node_tests": v[1].value, "groups": v[3].value,
          "quad_interactions": L.tg_tree_last_walk_quad_interactions(h),
          "kernel_ms": L.tg_tree_last_walk_kernel_ms(h)}
    L.tg_tree_free(h)
    return st


def cpu_step(x, m, h, nthreads):
    """One step of the reference algorithm on the host cores (oracle/, FP64, OpenMP): the full tree
    build and the grouped walk (pytreegrav's consecutive groups of 8, theta=0.7, quadrupole) of every
    particle, as Accel(x, m, h, method='tree', quadrupole=True) does. Returns (build s, walk s)."""
    from oracle import oracle as O

    t0 = time.perf_counter()
    t = O.OracleTree(x, m, h, quadrupole=True)
    t1 = time.perf_counter()
    idx = t.TreewalkIndices
    t.fields(x[idx], h[idx], accel=True, quadrupole=True, group_size=8, theta=THETA, nthreads=nthreads)
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1


def cpu_baseline(x, m, h, nthreads):
    """The reference algorithm timed on the host cores: one full step (no sampling, no extrapolation)."""
    n = len(x)
    tb, tw = cpu_step(x, m, h, nthreads)
    step = tb + tw
    return {"value": n / step, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"one full step: oracle build of all N={n} particles + FP64 grouped walk of all of them "
                      f"(group_size=8, theta={THETA}, quadrupole), timed whole: {step:.2f} s per step "
                      f"(build {tb:.2f} s, walk {tw:.2f} s)"}


def run_ours(args):
    import torch

    from pytreegrav_gb300 import _lib

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = _bind(_lib.load())
    stream = torch.cuda.current_stream().cuda_stream
    n = args.n
    x = plummer(n, SEED + rank)  # one independent replica per rank
    m = np.full(n, 1.0 / n)
    h = np.full(n, SOFT)
    dpos = torch.from_numpy(x).cuda()
    dm = torch.from_numpy(m).cuda()
    dh = torch.from_numpy(h).cuda()
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    out_plain = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2 (129 MB)
    from pytreegrav_gb300 import theta as th

    model = th.ThetaModel.load()
    mh = model.handle()
    l10 = th.default_lambda(model, True)
    # FP64 direct sums on 1e4 sampled targets: the accuracy of both walks (rank 0 reports it)
    import pytreegrav_gb300 as tg

    rng = np.random.default_rng(7)
    samp = rng.choice(n, 10_000, replace=False)
    ref = tg.bruteforce(x[samp], h[samp], x, m, h, accel=True, precision="fp64")["accel"]
    rms_ref = np.sqrt(np.mean(np.sum(ref**2, 1)))

    def rms_err(o):
        err = o.cpu().numpy()[samp] - ref
        return float(np.sqrt(np.mean(np.sum(err**2, 1))) / rms_ref)

    # equal accuracy: the learned test's lambda is lowered along the model's calibration grid (a lower
    # lambda accepts more, cheaper, nodes) for as long as the learned walk's RMS error on these targets
    # stays within the plain theta = 0.7 walk's, then refined between grid values; untimed
    gpu_step(L, _lib, dpos, dm, dh, out_plain, n, stream)
    e_plain = rms_err(out_plain)
    grid = [g for g in model.meta.get("calibration", {}).get("grid", []) if g <= l10 + 1e-9]
    l10_default = l10
    g_fail = None
    for g in sorted(grid, reverse=True):
        gpu_step(L, _lib, dpos, dm, dh, out, n, stream, mh, g)
        if rms_err(out) <= e_plain:
            l10 = g
        else:
            g_fail = g
            break
    # then bisected between the last grid value that stayed within and the first that did not
    if g_fail is not None and g_fail < l10:
        lo, hi = g_fail, l10
        for _ in range(4):
            mid = 0.5 * (lo + hi)
            gpu_step(L, _lib, dpos, dm, dh, out, n, stream, mh, mid)
            if rms_err(out) <= e_plain:
                hi = mid
            else:
                lo = mid
        l10 = hi

    def timed(step_fn, dest, sampler=None):
        for _ in range(args.warmup):
            step_fn(dest)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        stats = []
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = L.tg_launch_count()
        if sampler:
            sampler.begin()
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()  # evict the previous step's data from L2 (outside the step events)
            ev[k][0].record()
            stats.append(step_fn(dest))
            ev[k][1].record()
        torch.cuda.synchronize()
        region = time.perf_counter() - t0
        if sampler:
            sampler.end()
        if dist:
            dist.barrier()
        ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
        if dist:
            tt = torch.tensor([ms], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            ms = float(tt.item())
        return ms, stats, region, L.tg_launch_count() - l0

    learned_step = lambda dest: gpu_step(L, _lib, dpos, dm, dh, dest, n, stream, mh, l10)
    plain_step = lambda dest: gpu_step(L, _lib, dpos, dm, dh, dest, n, stream)
    clocks = ClockSampler(local)
    clocks.start()
    ms, stats, t_region, launches = timed(learned_step, out, clocks)
    clk = clocks.stop()
    ms_plain, stats_plain, _, _ = timed(plain_step, out_plain)
    value = n * ws / (ms * 1e-3)
    if rank != 0:
        return None

    # accuracy of both walks against FP64 direct summation on the same 1e4 sampled targets
    def accuracy(o):
        err = o.cpu().numpy()[samp] - ref
        return {"rms_rel_vs_fp64_bruteforce": float(np.sqrt(np.mean(np.sum(err**2, 1))) / rms_ref),
                "max_rel_vs_fp64_bruteforce": float(np.max(np.sqrt(np.sum(err**2, 1))) / rms_ref),
                "sample_targets": len(samp)}

    acc_learned, acc_plain = accuracy(out), accuracy(out_plain)

    # roofline of the dominant kernel (the walk): algorithmic FP32 flops / its own device time
    st = stats[-1]
    walk_ms = statistics.mean(s["kernel_ms"] for s in stats)
    flops = FLOPS_MONO_ACC * (st["interactions"] - st["quad_interactions"]) + FLOPS_QUAD_ACC * st["quad_interactions"]
    peak_tf, peak_ms = ctypes.c_double(), ctypes.c_double()
    L.tg_measure_fp32_fma(ctypes.byref(peak_tf), ctypes.byref(peak_ms), ctypes.c_void_p(stream))
    achieved = flops / (walk_ms * 1e-3) / 1e12
    # the arithmetic FP32 peak at the clock sampled during the timed region: SMs x 128 FMA lanes x 2
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk.get("sm_mhz") or 2070.0
    arith_tf = sms * 128 * 2 * mhz * 1e6 / 1e12
    roofline = {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(peak_tf.value, 3), "unit": "TFLOP/s",
                "frac": round(achieved / peak_tf.value, 4), "traffic": read_traffic(), "kernel": "k_walk",
                "peak_source": "measured: FFMA-chain probe on this GPU (tg_measure_fp32_fma); MEASURED_PEAKS.json "
                               "has no FP32 CUDA-core figure",
                "arith_peak": round(arith_tf, 3), "frac_of_arith_peak": round(achieved / arith_tf, 4),
                "arith_peak_source": f"{sms} SMs x 128 FP32 lanes x 2 flops x {mhz:.0f} MHz (median sampled SM clock)",
                "kernel_ms": round(walk_ms, 4), "flops_per_launch": flops,
                "interactions_per_s": round(st["interactions"] / (walk_ms * 1e-3), 1)}
    sp = stats_plain[-1]
    walk_ms_plain = statistics.mean(s["kernel_ms"] for s in stats_plain)
    flops_plain = (FLOPS_MONO_ACC * (sp["interactions"] - sp["quad_interactions"])
                   + FLOPS_QUAD_ACC * sp["quad_interactions"])
    plain = {"value": round(n / (ms_plain * 1e-3), 1), "ms_per_step": round(ms_plain, 4),
             "walk_kernel_ms": round(walk_ms_plain, 4), "walk_particles_per_s": round(n / (walk_ms_plain * 1e-3), 1),
             "interactions_per_target": sp["interactions"] / n, "accuracy": acc_plain,
             "walk_frac_of_fp32_peak": round(flops_plain / (walk_ms_plain * 1e-3) / 1e12 / peak_tf.value, 4),
             "walk_frac_of_arith_fp32_peak": round(flops_plain / (walk_ms_plain * 1e-3) / 1e12 / arith_tf, 4)}
    learned = {"walk_kernel_ms": round(walk_ms, 4), "walk_particles_per_s": round(n / (walk_ms * 1e-3), 1),
               "walk_speedup_vs_plain": round(walk_ms_plain / walk_ms, 3),
               "step_speedup_vs_plain": round(ms_plain / ms, 3),
               "error_ratio_vs_plain": round(acc_learned["rms_rel_vs_fp64_bruteforce"]
                                             / acc_plain["rms_rel_vs_fp64_bruteforce"], 3),
               "log10_lambda": l10, "log10_lambda_calibrated_default": l10_default,
               "lambda_choice": "the lowest lambda on the model's calibration grid at which the learned walk's RMS "
                                "error on the sampled targets stays within the plain walk's, then bisected four "
                                "times towards the next grid value (searched before timing)",
               "model": os.path.relpath(th.DEFAULT_MODEL, ROOT), "theta_cap": model.theta_max}

    # end to end through the public API, inputs in pinned host memory, result read back
    pin_x = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
    pin_m = torch.empty(n, dtype=torch.float64, pin_memory=True)
    pin_h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    pin_x.numpy()[:] = x
    pin_m.numpy()[:] = m
    pin_h.numpy()[:] = h
    model_eq = th.ThetaModel.load()  # the public call with the same lambda: a model object carrying it
    model_eq.log10_lambda = l10
    kw = dict(theta=THETA, method="tree", quadrupole=True, learned=model_eq)
    for _ in range(2):
        tg.Accel(pin_x.numpy(), pin_m.numpy(), pin_h.numpy(), **kw)
    e2e_t = []
    for _ in range(max(3, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a = tg.Accel(pin_x.numpy(), pin_m.numpy(), pin_h.numpy(), **kw)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e = {"value": n / statistics.median(e2e_t), "unit": UNIT, "h2d_bytes_per_step": int(x.nbytes + m.nbytes + h.nbytes),
           "d2h_bytes_per_step": int(a.nbytes), "api": "pytreegrav_gb300.Accel(pos, m, h, theta=0.7, quadrupole=True, "
           "method='tree', learned=model) with the packaged model at the lambda above",
           "ms_per_step": round(1e3 * statistics.median(e2e_t), 3)}

    # the reference's own configuration on the GPU: pytreegrav's consecutive groups of 8, plain
    # theta=0.7, FP32 and FP64 interactions (build + walk, device-resident inputs, L2 flushed)
    def blocks_step(dest, prec):
        vp = ctypes.c_void_p
        th = vp()
        _lib.check(L.tg_tree_build(vp(dpos.data_ptr()), vp(dm.data_ptr()), vp(dh.data_ptr()), n, 1, 1,
                                   _lib.TG_MEM_DEVICE, vp(stream), ctypes.byref(th)), "build")
        _lib.check(L.tg_tree_fields(th, None, None, n, _lib.TG_FIELD_ACCEL, 1, THETA, 1.0, 8, _lib.TG_GROUP_BLOCKS,
                                    _lib.TG_ORDER_TREE, prec, None, _lib.TG_MEM_DEVICE, vp(dest.data_ptr()),
                                    vp(stream)), "walk")
        kms = L.tg_tree_last_walk_kernel_ms(th)
        L.tg_tree_free(th)
        return {"kernel_ms": kms}

    ref_cfg = {}
    for label, prec, k in ((("fp32", _lib.TG_FP32, args.steps), ("fp64", _lib.TG_FP64, 3)) if ws == 1 else ()):
        sub = argparse.Namespace(warmup=1 if prec == _lib.TG_FP64 else args.warmup, steps=k)
        saved = args.warmup, args.steps
        args.warmup, args.steps = sub.warmup, sub.steps
        ms_b, st_b, _, _ = timed(lambda d, p=prec: blocks_step(d, p), out_plain)
        args.warmup, args.steps = saved
        ref_cfg[label] = {"value": round(n / (ms_b * 1e-3), 1), "ms_per_step": round(ms_b, 3),
                          "walk_kernel_ms": round(statistics.mean(s["kernel_ms"] for s in st_b), 3),
                          "steps": k, "accuracy": accuracy(out_plain)}
    ref_cfg["config"] = ("build + Accel walk with pytreegrav's grouping (group_size=8 consecutive Morton-ordered "
                         "targets), plain theta=0.7, quadrupole; the reference arm's configuration")

    # the build alone (device arrays, L2 flushed before each), against the HBM copy rate on its
    # algorithmic bytes (bench_configs.build_roofline)
    import bench_configs

    vp = ctypes.c_void_p
    bev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
    nodes = 0
    for k in range(13):
        flush.zero_()
        th_ = vp()
        if k >= 3:
            bev[k - 3][0].record()
        _lib.check(L.tg_tree_build(vp(dpos.data_ptr()), vp(dm.data_ptr()), vp(dh.data_ptr()), n, 1, 1,
                                   _lib.TG_MEM_DEVICE, vp(stream), ctypes.byref(th_)), "build")
        if k >= 3:
            bev[k - 3][1].record()
        info = _lib.TreeInfo()
        L.tg_tree_info_get(th_, ctypes.byref(info))
        nodes = int(info.node_hi) - n
        L.tg_tree_free(th_)
    torch.cuda.synchronize()
    build = bench_configs.build_roofline(n, nodes, statistics.mean(a_.elapsed_time(b_) for a_, b_ in bev))

    base = cpu_baseline(x, m, h, os.cpu_count() or 1)
    return {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Plummer sphere, a=1, r<50)",
        "config": {"workload": f"Accel, N={n} Plummer (m=1/N, h={SOFT}), theta={THETA}, quadrupole, FP32 walk with FP64 "
                               f"tree build and moments, tree grouping <= {GROUP} targets/warp",
                   "variant": "learned: each group's acceptance test from the packaged 16-64-64-1 network (a "
                              "mass-aware tolerance per group, angle cap 1.2) at the lambda that matches the plain "
                              "walk's RMS error (see learned.lambda_choice); the plain theta=0.7 walk is timed the "
                              "same way under 'plain'",
                   "step": "octree build + learned Accel walk (features, BF16 inference, walk), inputs resident "
                           "in HBM",
                   "l2": "flushed between timed steps (256 MiB write, outside the step events)",
                   "parallelism": f"replicas x{ws}", "region_s": round(t_region, 4)},
        "accuracy": acc_learned, "learned": learned, "plain": plain,
        "walk": {"interactions_per_target": st["interactions"] / n, "node_tests": st["node_tests"],
                 "groups": st["groups"], "quad_interactions": st["quad_interactions"]},
        "roofline": roofline, "build": build, "cpu_baseline": base, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
        "reference_config_on_gpu": ref_cfg,
    }


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    n = args.n
    x = plummer(n, SEED)
    m = np.full(n, 1.0 / n)
    h = np.full(n, SOFT)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_step(x, m, h, cores)
    t0 = time.perf_counter()
    steps = [cpu_step(x, m, h, cores) for _ in range(args.steps)]
    region = time.perf_counter() - t0
    ms = 1e3 * region / args.steps  # every step timed whole: build + walk of all N particles
    value = n / (ms * 1e-3)
    base = {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{args.steps} full steps timed back to back: oracle build of all N={n} particles + FP64 "
                      f"grouped walk of all of them (group_size=8, theta={THETA}, quadrupole); mean build "
                      f"{statistics.mean(s[0] for s in steps):.3f} s, walk {statistics.mean(s[1] for s in steps):.3f} s"}
    return {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Plummer sphere, a=1, r<50)",
            "impl": "reference",
            "config": {"workload": f"Accel, N={n} Plummer (m=1/N, h={SOFT}), theta={THETA}, quadrupole",
                       "implementation": "C restatement of pytreegrav's radix build and grouped walk (oracle/), "
                                         "all host threads; pytreegrav itself needs numba, absent on this machine"},
            "cpu_baseline": base, "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}


def batched_systems(n_sys, lo, hi, seed):
    """n_sys systems with N log-uniform in [lo, hi]: even ones uniform cubes, odd ones Plummer spheres,
    float32 positions, masses 1/N per system."""
    from pytreegrav_gb300 import synthetic

    rng = np.random.default_rng(seed)
    ns = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), n_sys))).astype(np.int64)
    parts = [(synthetic.uniform(int(k), seed + 7 * s) if s % 2 == 0 else synthetic.plummer(int(k), seed + 7 * s))
             .astype(np.float32).astype(np.float64) for s, k in enumerate(ns)]
    return np.vstack(parts), np.concatenate([np.full(k, 1.0 / k) for k in ns]), np.concatenate([[0], np.cumsum(ns)])


def run_batched(args):
    """4096 systems, N log-uniform in [256, 65536], h=0.01, theta=0.7, monopole: a step is one
    segmented build plus the walk captured in a CUDA graph (made for the new tree, then launched),
    inputs resident in HBM; the launch shape comes from the autotuner, tuned before timing."""
    import torch

    from pytreegrav_gb300 import _lib, autotune
    from pytreegrav_gb300.tree import Octree, WalkGraph

    L = _bind(_lib.load())
    n_sys = 4096
    x, m, off = batched_systems(n_sys, 256, 65536, SEED)
    n = len(x)
    h = np.full(n, 0.01)
    dpos, dm, dh = (torch.from_numpy(a).cuda() for a in (x, m, h))
    doff = off.astype(np.int64)
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    vp = ctypes.c_void_p
    st = vp(torch.cuda.current_stream().cuda_stream)

    def build():
        t = vp()
        _lib.check(L.tg_tree_build_batched(vp(dpos.data_ptr()), vp(dm.data_ptr()), vp(dh.data_ptr()), _lib.ptr(doff),
                                           n_sys, 0, _lib.TG_MEM_DEVICE, st, ctypes.byref(t)), "batched build")
        return Octree._from_handle(t, False)

    tree = build()
    tune = autotune.tune(tree, n_systems=n_sys, repeats=1, use_cache=False)
    del tree

    def step():
        t = build()
        t.set_walk_config(tune["warps"], tune["stack"])
        g = WalkGraph(t, out, False, True, False, False, tune["group_size"], THETA, 1.0, "tree")
        g.launch(st)
        return t, g

    for _ in range(args.warmup):
        t, g = step()
        g.status(st)
        g.close()
        del t
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    l0 = L.tg_launch_count()
    last = None
    for k in range(args.steps):
        ev[k][0].record()
        t, g = step()
        ev[k][1].record()
        if last is not None:
            last[1].close()
        last = (t, g)
    torch.cuda.synchronize()
    launches = L.tg_launch_count() - l0
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    t, g = last
    g.status(st)
    # the walk alone: replays of the graph on one tree
    rev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
    for a, b in rev:
        a.record()
        g.launch(st)
        b.record()
    torch.cuda.synchronize()
    g.status(st)
    walk_ms = statistics.mean(a.elapsed_time(b) for a, b in rev)
    acc = out.cpu().numpy()
    g.close()
    import pytreegrav_gb300 as tg

    errs = []
    for s in range(0, n_sys, 512):
        a, b = off[s], off[s + 1]
        ref = tg.bruteforce(x[a:b], h[a:b], x[a:b], m[a:b], h[a:b], accel=True, precision="fp64")["accel"]
        errs.append(round(float(np.sqrt(np.mean(np.sum((acc[a:b] - ref) ** 2, 1)) / np.mean(np.sum(ref ** 2, 1)))), 6))
    return {"metric": "Accel particles/s, 4096 independent systems (batched form)", "value": round(n / (ms * 1e-3), 1),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded: even systems uniform cubes, odd systems Plummer spheres, float32 positions)",
            "config": {"workload": f"{n_sys} systems, N log-uniform in [256, 65536] ({n} particles), m=1/N, h=0.01, "
                                   "theta=0.7, monopole, FP32 walk",
                       "step": "segmented build + walk graph made for the new tree and launched",
                       "autotuned": {k: tune[k] for k in ("group_size", "warps", "stack", "ms")}},
            "walk_graph_replay_ms": round(walk_ms, 3), "walk_particles_per_s": round(n / (walk_ms * 1e-3), 1),
            "accuracy_rms_rel_vs_fp64_bruteforce_sampled_systems": errs, "gpu_launches": int(launches)}


def run_column(args):
    """Ray-traced column density, 1e6 Plummer particles as uniform spheres of radius 0.01, the six axis
    rays from every particle: a step is the tree build plus the FP64 walk of all N x 6 (target, ray)
    pairs, inputs resident in HBM. e2e is the public ColumnDensity call from host arrays."""
    import torch

    import pytreegrav_gb300 as tg
    from oracle import oracle as O
    from pytreegrav_gb300 import _lib
    from pytreegrav_gb300.tree import Octree

    L = _bind(_lib.load())
    n = args.n
    x = plummer(n, SEED)
    m = np.full(n, 1.0 / n)
    h = np.full(n, 0.01)
    rays = np.vstack([np.eye(3), -np.eye(3)])
    dpos, dm, dh, dr = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (x, m, h, rays))
    out = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    vp = ctypes.c_void_p
    st = vp(torch.cuda.current_stream().cuda_stream)

    def step():
        t = vp()
        _lib.check(L.tg_tree_build(vp(dpos.data_ptr()), vp(dm.data_ptr()), vp(dh.data_ptr()), n, 0, 1,
                                   _lib.TG_MEM_DEVICE, st, ctypes.byref(t)), "build")
        tree = Octree._from_handle(t, False)
        info = _lib.TreeInfo()
        _lib.check(L.tg_tree_info_get(t, ctypes.byref(info)), "tree info")
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        # targets: the tree's own particles, which its first N coordinate rows hold in Morton order
        _lib.check(L.tg_tree_column_density(t, vp(info.coord), n, vp(dr.data_ptr()), 6, 0, 0, 0.0, 0,
                                            _lib.TG_MEM_DEVICE, vp(out.data_ptr()), st), "column density")
        return tree, e

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 10))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    walk = []
    l0 = L.tg_launch_count()
    for k in range(steps):
        ev[k][0].record()
        tree, e = step()
        ev[k][1].record()
        walk.append((e, ev[k][1]))
    torch.cuda.synchronize()
    launches = L.tg_launch_count() - l0
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    walk_ms = statistics.mean(a.elapsed_time(b) for a, b in walk)
    # parity on a sample of targets against the oracle (FP64, same order of operations: equal)
    got = out.cpu().numpy()
    ot = O.OracleTree(x, m, h)
    sample = np.arange(0, n, max(1, n // 500))
    ref = O.column_rays(ot, x[ot.TreewalkIndices][sample], rays)
    mismatches = int(np.count_nonzero(got[sample] != ref))
    # end to end through the public call
    tg.ColumnDensity(x, m, h, rays=6)
    e2e_t = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tg.ColumnDensity(x, m, h, rays=6)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    # CPU baseline: the oracle (the reference's walk in C, FP64, OpenMP on all host cores), full build
    # and every 64th target, extrapolated
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ot2 = O.OracleTree(x, m, h)
    t1 = time.perf_counter()
    sub = x[ot2.TreewalkIndices][::64]
    O.column_rays(ot2, sub, rays, nthreads=cores)
    t2 = time.perf_counter()
    cpu_s = (t1 - t0) + (t2 - t1) * 64
    return {"metric": "ColumnDensity rays/s, 1e6 Plummer, six axis rays per particle", "value": round(6 * n / (ms * 1e-3), 1),
            "unit": "rays/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded Plummer sphere, a=1, r<50)",
            "config": {"workload": f"ColumnDensity, N={n} Plummer, m=1/N, radii 0.01, rays=6 (the axis grid), "
                                   "ray-traced walk of every particle",
                       "step": "tree build + FP64 column walk of N x 6 (target, ray) pairs, inputs resident in HBM"},
            "walk_ms": round(walk_ms, 3), "walk_rays_per_s": round(6 * n / (walk_ms * 1e-3), 1),
            "parity": {"sample_targets": int(len(sample)), "mismatches_vs_oracle": mismatches},
            "e2e": {"value": round(6 * n / e2e_s, 1), "unit": "rays/s", "h2d_bytes_per_step": int(x.nbytes + m.nbytes + h.nbytes),
                    "d2h_bytes_per_step": int(8 * 6 * n), "api": "pytreegrav_gb300.ColumnDensity(pos, m, radii, rays=6)",
                    "ms_per_step": round(1e3 * e2e_s, 3)},
            "cpu_baseline": {"value": round(6 * n / cpu_s, 1), "unit": "rays/s", "cores": cores, "kind": "port",
                             "sample": "oracle build of all N + the ray-traced walk (C, FP64, OpenMP) of every 64th "
                                       f"target, extrapolated; {cpu_s:.2f} s per step"},
            "gpu_launches": int(launches)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--config", choices=["plummer", "batched", "column", "uniform", "precision", "clustered",
                                         "largest", "corr", "build"], default="plummer",
                    help="batched: the 4096-system configuration; column: ray-traced column density; uniform, "
                         "precision, clustered, largest, corr, build: see bench_configs.py (each its own JSON line)")
    ap.add_argument("--sources", type=int, default=32_000_000, help="source count of --config largest")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.config == "batched" and args.impl == "ours":
        res = run_batched(args)
    elif args.config == "column" and args.impl == "ours":
        res = run_column(args)
    elif args.config in ("uniform", "precision", "clustered", "largest", "corr", "build") and args.impl == "ours":
        import bench_configs

        res = getattr(bench_configs, "run_" + args.config)(args)
    else:
        res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
