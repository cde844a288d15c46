"""Learned opening angle for the grouped walk (C entries in include/pytreegrav_gb300_theta.h).

pytreegrav walks with one global theta (treewalk.py:22-25, grouped_treewalk.py:163-241). Here a small
network gives every group of targets its own angle: groups whose error would be small open fewer
nodes, groups whose error dominates the total open more, so the same RMS force error costs fewer
interactions. Nothing here has a counterpart in pytreegrav.

The pieces, all on the GPU through the library:

* features: per group, from the tree (``tg_theta_features``);
* training data (:func:`collect`): for every angle of a grid, the walk's per-group cost (from its
  per-group counters) and the per-group force error against an FP32 Kahan-compensated brute-force
  sum on a sample of groups -- errors the method itself produces;
* :func:`train`: a 16-64-64-1 SiLU network fitted with the library's own FP32 forward, backward,
  loss and Adam kernels. Per group it minimises cost(theta) + lambda * error(theta); lambda, the
  price of error, is one of the inputs, so one network covers a range of accuracies;
* :func:`calibrate`: the lambda at which the predicted angles reach a requested error relative to
  the plain walk at theta = 0.7, from the training systems' tables;
* inference: ``tg_theta_infer``, one fused BF16 tensor-core kernel, inside
  ``tg_tree_fields_learned``; the plain global-theta walk is the fallback (no model, or a
  non-finite angle).

Cost and error are normalised per system so that, at the plain angle, the sampled groups' costs
sum to 1 and their squared errors sum to 1; the error ratio sqrt(sum err) is then the RMS force
error relative to the plain walk's.

Train a model (GPU): ``python -m pytreegrav_gb300.theta --out model.npz``.
"""

import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

from . import _lib

GRID = np.round(np.arange(0.3, 1.0001, 0.1), 6)  # angles of the training walks (angle models)
THETA_MIN, THETA_MAX = float(GRID[0]), float(GRID[-1])
# log10 of the tolerance relative to the system's estimated RMS acceleration (tolerance models)
TOL_GRID = np.round(np.arange(-3.5, 1.0001, 0.5), 6)
THETA_CAP = 1.2  # angle cap of the mass-aware test
GROUP_SIZE = 32  # targets per group of the tree grouping the models are trained and used with
PLAIN_THETA = 0.7
I_PLAIN = int(np.argmin(np.abs(GRID - PLAIN_THETA)))
KINDS = {"angle": _lib.TG_THETA_KIND_ANGLE, "tolerance": _lib.TG_THETA_KIND_TOLERANCE}


def grid_of(kind):
    return GRID if kind == "angle" else TOL_GRID
# cost of a group in relative warp time: point-mass entries, quadrupole entries, node tests; the
# entries of a group of n targets take P/32 of a warp's time, P the power of two >= n that the walk
# gives each slice of lanes
COST_W = np.array([1.0, 1.7, 0.1])


def group_cost(stats, count):
    p = 2 ** np.ceil(np.log2(np.maximum(count, 1)))
    return (stats[:, 0] * COST_W[0] + stats[:, 1] * COST_W[1]) * (p / 32.0) + stats[:, 2] * COST_W[2]
LOG10_LAMBDA_RANGE = (-1.5, 2.5)
NF = _lib.TG_THETA_NFEAT
NP = _lib.TG_MLP_NPARAM
H = _lib.TG_MLP_H
OFF = dict(W1=0, b1=H * NF, W2=H * NF + H, b2=H * NF + H + H * H, W3=H * NF + 2 * H + H * H,
           b3=H * NF + 3 * H + H * H)
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "theta_mlp.npz")


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _check(rc, what):
    _lib.check(rc, what)


class ThetaModel:
    """Network parameters (FP32), feature normalisation, output kind and range, the angle cap of a
    tolerance model, and the calibrated lambda."""

    def __init__(self, params, mean, std, log10_lambda=0.0, meta=None, kind="angle", theta_max=THETA_CAP):
        self.params = np.ascontiguousarray(params, np.float32).reshape(NP)
        self.mean = np.ascontiguousarray(mean, np.float32).reshape(NF)
        self.std = np.ascontiguousarray(std, np.float32).reshape(NF)
        self.log10_lambda = float(log10_lambda)
        self.meta = dict(meta or {})
        self.kind = kind
        self.theta_max = float(theta_max)
        self._handle = None

    @property
    def error_budget(self):
        """Per-group relative error budget of a tolerance model (tg_theta_model_set_error_budget; 0:
        no rewalk), kept in the model file's metadata."""
        return float(self.meta.get("error_budget", 0.0))

    @error_budget.setter
    def error_budget(self, value):
        self.meta["error_budget"] = float(value)
        if self._handle is not None:
            _check(_lib.load().tg_theta_model_set_error_budget(self._handle, float(value)), "error budget")

    @property
    def out_range(self):
        g = grid_of(self.kind)
        return float(g[0]), float(g[-1])

    @staticmethod
    def init_params(seed=0):
        rng = np.random.default_rng(seed)
        p = np.zeros(NP, np.float32)
        p[OFF["W1"]:OFF["b1"]] = rng.normal(0, np.sqrt(2.0 / NF), H * NF)
        p[OFF["W2"]:OFF["b2"]] = rng.normal(0, np.sqrt(2.0 / H), H * H)
        p[OFF["W3"]:OFF["b3"]] = rng.normal(0, np.sqrt(1.0 / H), H)
        return p

    def save(self, path):
        np.savez(path, params=self.params, mean=self.mean, std=self.std,
                 log10_lambda=np.float64(self.log10_lambda), meta=json.dumps(self.meta), kind=self.kind,
                 theta_max=np.float64(self.theta_max))

    @classmethod
    def load(cls, path=None):
        z = np.load(path or DEFAULT_MODEL, allow_pickle=False)
        return cls(z["params"], z["mean"], z["std"], float(z["log10_lambda"]), json.loads(str(z["meta"])),
                   str(z["kind"]), float(z["theta_max"]))

    def handle(self):
        """The library's inference model (BF16 weights on the current device)."""
        if self._handle is None:
            L = _lib.load()
            h = ctypes.c_void_p()
            lo, hi = self.out_range
            _check(L.tg_theta_model_create(_lib.ptr(self.params), _lib.ptr(self.mean), _lib.ptr(self.std),
                                           KINDS[self.kind], lo, hi, self.theta_max, _lib.TG_MEM_HOST,
                                           ctypes.byref(h)), "theta model")
            self._handle = h
            if self.error_budget > 0:
                _check(L.tg_theta_model_set_error_budget(h, self.error_budget), "error budget")
        return self._handle

    def close(self):
        if self._handle is not None:
            _lib.load().tg_theta_model_free(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------------
# Training data


def _tree_device(torch, pos, m, h, quadrupole):
    L = _lib.load()
    dpos = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()
    dm = torch.from_numpy(np.ascontiguousarray(m, np.float64)).cuda()
    dh = torch.from_numpy(np.ascontiguousarray(h, np.float64)).cuda()
    tree = ctypes.c_void_p()
    st = torch.cuda.current_stream().cuda_stream
    _check(L.tg_tree_build(_vp(dpos), _vp(dm), _vp(dh), len(pos), int(quadrupole), 1, _lib.TG_MEM_DEVICE,
                           ctypes.c_void_p(st), ctypes.byref(tree)), "build")
    return tree, (dpos, dm, dh)


def groups_of(tree, group_size):
    """(first, count, node) of the tree grouping, host int32 arrays."""
    L = _lib.load()
    ng = ctypes.c_int64()
    _check(L.tg_tree_groups(tree, group_size, ctypes.byref(ng), None), "groups")
    first, count, node = (np.empty(ng.value, np.int32) for _ in range(3))
    _check(L.tg_tree_groups_copy(tree, group_size, _lib.ptr(first), _lib.ptr(count), _lib.ptr(node),
                                 _lib.TG_MEM_HOST, None), "groups copy")
    return first, count, node


def features(tree, group_size, quadrupole):
    """Per-group features (ngroups x 16 float32, host)."""
    import torch

    L = _lib.load()
    ng = ctypes.c_int64()
    _check(L.tg_tree_groups(tree, group_size, ctypes.byref(ng), None), "groups")
    f = torch.empty((max(ng.value, 1), NF), dtype=torch.float32, device="cuda")
    _check(L.tg_theta_features(tree, group_size, int(quadrupole), _vp(f),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "features")
    torch.cuda.synchronize()
    return f[:ng.value].cpu().numpy()


def collect(pos, m, h, quadrupole=True, group_size=GROUP_SIZE, sample=0.25, seed=0, G=1.0, label="", kind="tolerance",
            theta_max=THETA_CAP, targets=None):
    """Training tables of one particle system (see the module docstring): for every value of the
    kind's grid, each sampled group's cost and squared force error, both relative to the plain
    walk at theta = 0.7 (summed over the sampled groups, the plain walk's are 1).

    targets=None: the system's own particles are the targets, in the tree grouping. targets=(pos_t,
    h_t): external targets, grouped by their own octree (a TargetSet), judged against the same
    sources (tolerance models only)."""
    import torch

    L = _lib.load()
    n = len(pos)
    pos = np.ascontiguousarray(pos, np.float64)
    m = np.ascontiguousarray(m, np.float64)
    h = np.ascontiguousarray(h, np.float64)
    tree, keep = _tree_device(torch, pos, m, h, quadrupole)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    grid = grid_of(kind)
    tset = None
    try:
        if targets is None:
            first, count, node = groups_of(tree, group_size)
            walk_idx = np.empty(n, np.int64)
            _check(L.tg_tree_copy_out(tree, None, None, None, None, None, None, None, None, _lib.ptr(walk_idx),
                                      None), "copy out")
            feat = features(tree, group_size, quadrupole)
            tpos, th_ = pos, h
            nt = n
        else:
            if kind != "tolerance":
                raise ValueError("external-target tables are made for tolerance models")
            tpos = np.ascontiguousarray(targets[0], np.float64)
            th_ = np.ascontiguousarray(targets[1], np.float64)
            nt = len(tpos)
            tset = ctypes.c_void_p()
            _check(L.tg_targets_create(tree, _lib.ptr(tpos), _lib.ptr(th_), nt, group_size, _lib.TG_MEM_HOST, None,
                                       ctypes.byref(tset)), "target set")
            ngv = ctypes.c_int64()
            _check(L.tg_targets_info(tset, None, ctypes.byref(ngv)), "target set")
            first, count, node = (np.empty(ngv.value, np.int32) for _ in range(3))
            walk_idx = np.empty(nt, np.int64)
            _check(L.tg_targets_groups_copy(tset, _lib.ptr(first), _lib.ptr(count), _lib.ptr(node), _lib.ptr(walk_idx),
                                            _lib.TG_MEM_HOST, None), "target groups")
            fd = torch.empty((max(ngv.value, 1), NF), dtype=torch.float32, device="cuda")
            _check(L.tg_targets_features(tset, int(quadrupole), _vp(fd), st), "target features")
            torch.cuda.synchronize()
            feat = fd[:ngv.value].cpu().numpy()
        ng = len(first)
        rng = np.random.default_rng(seed)
        S = np.sort(rng.choice(ng, size=max(1, int(sample * ng)), replace=False))
        seg = np.concatenate([[0], np.cumsum(count[S])])
        sel = np.concatenate([np.arange(first[g], first[g] + count[g]) for g in S])
        idx = walk_idx[sel]
        # judge: FP32 Kahan-compensated direct sum over all sources (self pairs at r == 0 skipped)
        t0 = time.time()
        dpt = torch.from_numpy(np.ascontiguousarray(tpos[idx])).cuda()
        dht = torch.from_numpy(np.ascontiguousarray(th_[idx])).cuda()
        aref = torch.empty((len(idx), 3), dtype=torch.float64, device="cuda")
        _check(L.tg_bruteforce(_vp(dpt), _vp(dht), len(idx), _vp(keep[0]), _vp(keep[1]), _vp(keep[2]), n,
                               _lib.TG_FIELD_ACCEL, 0, G, _lib.TG_FP32, _lib.TG_MEM_DEVICE, _vp(aref), st),
               "brute force")
        torch.cuda.synchronize()
        t_bf = time.time() - t0
        aref_h = aref.cpu().numpy()
        rms2 = float(np.mean(np.sum(aref_h ** 2, axis=1)))
        out = torch.empty((nt, 3), dtype=torch.float64, device="cuda")
        didx = torch.from_numpy(idx).cuda()
        stats = np.empty((ng, 3), np.uint32)
        u = torch.empty(max(ng, 1), dtype=torch.float32, device="cuda")
        tol = torch.empty(max(ng, 1), dtype=torch.float32, device="cuda")
        _check(L.tg_tree_record_group_stats(tree, 1), "record")

        def measure(angle, tol_dev=None):
            tp = None if tol_dev is None else _vp(tol_dev)
            if tset is not None:
                _check(L.tg_targets_fields(tset, _lib.TG_FIELD_ACCEL, int(quadrupole), float(angle), G, _lib.TG_FP32,
                                           tp, _lib.TG_MEM_DEVICE, _vp(out), st), "target walk")
            elif tol_dev is None:
                _check(L.tg_tree_fields(tree, None, None, n, _lib.TG_FIELD_ACCEL, int(quadrupole), float(angle), G,
                                        group_size, _lib.TG_GROUP_TREE, _lib.TG_ORDER_TREE, _lib.TG_FP32, None,
                                        _lib.TG_MEM_DEVICE, _vp(out), st), "walk")
            else:
                _check(L.tg_tree_fields_grouped(tree, _lib.TG_FIELD_ACCEL, int(quadrupole), G, group_size,
                                                float(angle), None, tp, _lib.TG_MEM_DEVICE, _vp(out), st), "walk")
            _check(L.tg_tree_last_group_stats(tree, _lib.ptr(stats), _lib.TG_MEM_HOST, st), "group stats")
            a = out.index_select(0, didx).cpu().numpy()
            d2 = np.sum((a - aref_h) ** 2, axis=1) / rms2
            return group_cost(stats[S].astype(np.float64), count[S]), np.add.reduceat(d2, seg[:-1])

        c_plain, e_plain = measure(PLAIN_THETA)
        cost = np.empty((len(S), len(grid)))
        err = np.empty((len(S), len(grid)))
        for k, v in enumerate(grid):
            if kind == "angle":
                cost[:, k], err[:, k] = measure(v)
            else:
                u.fill_(float(v))
                if tset is not None:
                    _check(L.tg_targets_tolerances(tset, int(quadrupole), _vp(u), _vp(tol), st), "tolerances")
                else:
                    _check(L.tg_theta_tolerances(tree, group_size, int(quadrupole), _vp(u), _vp(tol), st),
                           "tolerances")
                cost[:, k], err[:, k] = measure(theta_max, tol)
        _check(L.tg_tree_record_group_stats(tree, 0), "record")
    finally:
        if tset is not None:
            L.tg_targets_free(tset)
        L.tg_tree_free(tree)
    c0, e0 = c_plain.sum(), e_plain.sum()
    floor = 1e-6 / len(S)
    return dict(label=label, kind=kind, n=n, ngroups=ng, sampled=len(S), features=feat[S],
                log_cost=np.log(cost / c0).astype(np.float32), log_err=np.log(err / e0 + floor).astype(np.float32),
                plain_rms_rel=float(np.sqrt(e0 / len(idx))), bf_seconds=t_bf, quadrupole=bool(quadrupole),
                targets=targets is not None)


# ---------------------------------------------------------------------------------------------
# Training with the library's kernels


def feature_stats(datasets):
    X = np.concatenate([d["features"] for d in datasets])
    mean = X.mean(axis=0)
    std = X.std(axis=0)
    lo, hi = LOG10_LAMBDA_RANGE
    mean[_lib.TG_THETA_FEAT_LAMBDA] = 0.5 * (lo + hi)
    std[_lib.TG_THETA_FEAT_LAMBDA] = (hi - lo) / np.sqrt(12.0)
    std = np.where(std > 1e-6, std, 1.0)
    return mean.astype(np.float32), std.astype(np.float32)


def train(datasets, steps=3000, batch=8192, lr=2e-3, seed=0, log_every=500, verbose=True, theta_max=THETA_CAP):
    """Fit the network to the datasets' tables; returns a ThetaModel (lambda not yet calibrated)."""
    import torch

    L = _lib.load()
    kind = datasets[0]["kind"]
    assert all(d["kind"] == kind for d in datasets)
    grid = grid_of(kind)
    mean, std = feature_stats(datasets)
    X = np.concatenate([d["features"] for d in datasets]).astype(np.float32)
    Xn = ((X - mean) / std).astype(np.float32)
    LC = np.concatenate([d["log_cost"] for d in datasets]).astype(np.float32)
    LE = np.concatenate([d["log_err"] for d in datasets]).astype(np.float32)
    # each system weighs the same, whatever its number of sampled groups
    w = np.concatenate([np.full(d["sampled"], 1.0 / d["sampled"]) for d in datasets])
    w = w / w.sum()
    dev = "cuda"
    Xd, LCd, LEd = (torch.from_numpy(a).to(dev) for a in (Xn, LC, LE))
    wd = torch.from_numpy(w).to(dev)
    params = torch.from_numpy(ThetaModel.init_params(seed)).to(dev)
    m1 = torch.zeros(NP, dtype=torch.float32, device=dev)
    v1 = torch.zeros(NP, dtype=torch.float32, device=dev)
    grad = torch.zeros(NP, dtype=torch.float32, device=dev)
    B = min(batch, len(X))
    y = torch.empty(B, dtype=torch.float32, device=dev)
    dy = torch.empty(B, dtype=torch.float32, device=dev)
    acts = torch.empty((B, 2 * H), dtype=torch.float32, device=dev)
    work = torch.empty((B, 2 * H), dtype=torch.float32, device=dev)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    lo, hi = LOG10_LAMBDA_RANGE
    li = _lib.TG_THETA_FEAT_LAMBDA
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    history = []
    t0 = time.time()
    for step in range(1, steps + 1):
        rows = torch.multinomial(wd, B, replacement=True, generator=gen)
        xb = Xd.index_select(0, rows).contiguous()
        l10 = lo + (hi - lo) * torch.rand(B, device=dev, generator=gen)
        xb[:, li] = (l10 - float(mean[li])) / float(std[li])
        lam = torch.pow(10.0, l10).float().contiguous()
        lcb = LCd.index_select(0, rows).contiguous()
        leb = LEd.index_select(0, rows).contiguous()
        loss.zero_()
        _check(L.tg_mlp_forward(_vp(params), _vp(xb), B, _vp(acts), _vp(y), st), "forward")
        _check(L.tg_theta_loss(_vp(y), _vp(lcb), _vp(leb), _vp(lam), B, len(grid), float(grid[0]),
                               float(grid[1] - grid[0]), float(grid[0]), float(grid[-1]), _vp(dy), _vp(loss), st),
               "loss")
        _check(L.tg_mlp_backward(_vp(params), _vp(xb), _vp(acts), _vp(dy), B, _vp(work), _vp(grad), st), "backward")
        rate = lr * (0.1 + 0.9 * 0.5 * (1 + np.cos(np.pi * step / steps)))  # cosine decay to lr/10
        _check(L.tg_adam_step(_vp(params), _vp(grad), _vp(m1), _vp(v1), NP, float(rate), 0.9, 0.999, 1e-8, step, st),
               "adam")
        if step % log_every == 0 or step == steps:
            history.append((step, float(loss.item())))
            if verbose:
                print(f"  step {step:5d}  loss {history[-1][1]:.5f}  ({time.time() - t0:.1f} s)", file=sys.stderr)
    model = ThetaModel(params.cpu().numpy(), mean, std, 0.0,
                       meta=dict(steps=steps, batch=B, lr=lr, history=history,
                                 systems=[d["label"] for d in datasets]), kind=kind, theta_max=theta_max)
    return model


def predict(model, feats, log10_lambda):
    """Network outputs (angles or log10 relative tolerances) from the BF16 inference kernel (host
    arrays in and out)."""
    import torch

    L = _lib.load()
    f = torch.from_numpy(np.ascontiguousarray(feats, np.float32)).cuda()
    out = torch.empty(len(feats), dtype=torch.float32, device="cuda")
    _check(L.tg_theta_infer(model.handle(), _vp(f), len(feats), float(log10_lambda), _vp(out),
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "infer")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def table_at(log_tab, theta, grid=GRID):
    """Per-row linear interpolation of a log table over `grid` at the values theta."""
    u = (np.clip(theta, grid[0], grid[-1]) - grid[0]) / (grid[1] - grid[0])
    k = np.clip(np.floor(u).astype(int), 0, len(grid) - 2)
    w = u - k
    r = np.arange(len(theta))
    return np.exp(log_tab[r, k] * (1 - w) + log_tab[r, k + 1] * w)


def predicted_ratios(model, d, log10_lambda):
    """(error ratio, cost ratio) against the plain walk that the model's angles give on dataset d."""
    th = predict(model, d["features"], log10_lambda)
    g = grid_of(model.kind)
    return float(np.sqrt(table_at(d["log_err"], th, g).sum())), float(table_at(d["log_cost"], th, g).sum())


MODES = ((True, False), (False, False), (True, True), (False, True))  # (quadrupole, external targets)


def _lambda_key(quadrupole, targets):
    return "log10_lambda" + ("_targets" if targets else "") + ("" if quadrupole else "_mono")


def calibrate(model, datasets, target_ratio=0.85, grid=None):
    """Error-ratio curves of the training systems over a lambda grid, stored in the model; the
    default lambda of each mode -- multipole order, and own particles or external targets as the
    targets -- is the smallest (cheapest) one at which the median error ratio of that mode's systems
    is within target_ratio. Returns the per-system (error, cost) ratios at the chosen lambdas."""
    grid = np.arange(LOG10_LAMBDA_RANGE[0], LOG10_LAMBDA_RANGE[1] + 1e-9, 0.05) if grid is None else grid
    curves = {d["label"]: dict(quadrupole=d["quadrupole"], targets=bool(d.get("targets", False)), error=[], cost=[])
              for d in datasets}
    for l10 in grid:
        for d in datasets:
            e, c = predicted_ratios(model, d, l10)
            curves[d["label"]]["error"].append(e)
            curves[d["label"]]["cost"].append(c)
    model.meta["calibration"] = dict(grid=[float(g) for g in grid], target_ratio=target_ratio, systems=curves)
    chosen = {}
    for quad, tgt in MODES:
        l10 = lambda_for_ratio(model, target_ratio, quad, tgt)
        if l10 is not None:
            chosen[(quad, tgt)] = l10
            model.meta[_lambda_key(quad, tgt)] = l10
    model.log10_lambda = chosen.get((True, False), 0.0)
    out = []
    for d in datasets:
        out.append(predicted_ratios(model, d, default_lambda(model, d["quadrupole"], d.get("targets", False))))
    return out


def lambda_for_ratio(model, ratio, quadrupole, targets=False):
    """log10 lambda at which the median training system of this mode (multipole order; own particles
    or external targets) is predicted to reach `ratio` times the plain walk's RMS force error (None
    without calibration curves). Systems of the other target kind stand in when a mode has none."""
    cal = model.meta.get("calibration")
    if not cal:
        return None
    allv = list(cal["systems"].values())
    sys_ = [v for v in allv if v["quadrupole"] == bool(quadrupole) and v.get("targets", False) == bool(targets)]
    sys_ = sys_ or [v for v in allv if v.get("targets", False) == bool(targets)]
    sys_ = sys_ or [v for v in allv if v["quadrupole"] == bool(quadrupole)] or allv
    med = np.median(np.array([v["error"] for v in sys_]), axis=0)
    grid = np.array(cal["grid"])
    ok = np.nonzero(med <= ratio)[0]
    return float(grid[ok[0]]) if len(ok) else float(grid[-1])


def default_lambda(model, quadrupole, targets=False):
    """The calibrated log10 lambda of a mode (see calibrate)."""
    if quadrupole and not targets:
        return model.log10_lambda
    v = model.meta.get(_lambda_key(quadrupole, targets))
    if v is None and targets:  # a model calibrated on own-particle systems only
        v = model.meta.get(_lambda_key(quadrupole, False))
    if v is None:
        v = model.log10_lambda
    return float(v)


# ---------------------------------------------------------------------------------------------
# Training run


def training_systems(scale=1.0):
    """(label, positions, softening, quadrupole) of the synthetic training systems whose own particles
    are the targets. The seeds are not the benchmark's, so the benchmark systems are held out."""
    from . import synthetic as S

    n4, n0, n1, n2, n3 = (int(v * scale) for v in (4_000_000, 2_000_000, 1_000_000, 500_000, 250_000))
    return [
        ("plummer_2e6_q", S.plummer(n0, 112), 0.005, True),
        ("plummer_1e6_q", S.plummer(n1, 101), 0.005, True),
        ("plummer_5e5_q", S.plummer(n2, 102), 0.005, True),
        ("plummer_2.5e5_q", S.plummer(n3, 109), 0.005, True),
        ("clustered_4e6_q", S.clustered(n4, 113), 0.002, True),
        ("clustered_1e6_q", S.clustered(n1, 103), 0.002, True),
        ("clustered_5e5_q", S.clustered(n2, 104), 0.002, True),
        ("clustered_2.5e5_q", S.clustered(n3, 110), 0.002, True),
        ("uniform_5e5_q", S.uniform(n2, 105), 0.01, True),
        ("plummer_1e6_m", S.plummer(n1, 106), 0.005, False),
        ("plummer_2.5e5_m", S.plummer(n3, 111), 0.005, False),
        ("clustered_1e6_m", S.clustered(n1, 107), 0.002, False),
        ("uniform_5e5_m", S.uniform(n2, 108), 0.01, False),
    ]


def target_systems(scale=1.0):
    """(label, source positions, source softenings, target positions, target softenings, quadrupole) of
    the synthetic training systems with external targets: Plummer sources with lognormal softenings
    and targets uniform in a ball of radius 5, or drawn from the sources' own distribution; clustered
    sources with targets uniform in their box; uniform sources with uniform targets."""
    from . import synthetic as S

    def ball(k, seed, radius=5.0):
        rng = np.random.default_rng(seed)
        d = rng.normal(size=(k, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        return d * (radius * rng.random(k) ** (1 / 3))[:, None]

    def lognormal_h(k, seed):
        return np.exp(np.random.default_rng(seed).normal(np.log(0.003), 0.7, k))

    n4, n1, n2 = (int(v * scale) for v in (4_000_000, 1_000_000, 500_000))
    t2, t1 = (int(v * scale) for v in (250_000, 100_000))
    return [
        ("plummer_4e6_ball_q", S.plummer(n4, 201), lognormal_h(n4, 202), ball(t2, 203), np.zeros(t2), True),
        ("plummer_1e6_ball_q", S.plummer(n1, 204), lognormal_h(n1, 205), ball(t2, 206), np.zeros(t2), True),
        ("plummer_5e5_self_dist_q", S.plummer(n2, 207), np.full(n2, 0.005), S.plummer(t1, 208), np.full(t1, 0.005),
         True),
        ("clustered_1e6_box_q", S.clustered(n1, 209), np.full(n1, 0.002),
         np.random.default_rng(210).uniform(-10, 10, (t2, 3)), np.zeros(t2), True),
        ("uniform_5e5_cube_q", S.uniform(n2, 211), np.full(n2, 0.01), S.uniform(t1, 212), np.zeros(t1), True),
        ("plummer_1e6_ball_m", S.plummer(n1, 213), lognormal_h(n1, 214), ball(t2, 215), np.zeros(t2), False),
    ]


def group_errors(model, pos, h, quadrupole, log10_lambda=None, G=1.0):
    """Per-group estimated relative truncation errors (tg_tree_last_group_error) of the learned walk of
    one system (m = 1/N, softening h), taken with the budget check off."""
    import torch

    n = len(pos)
    L = _lib.load()
    tree, keep = _tree_device(torch, pos, np.full(n, 1.0 / n), np.full(n, h), quadrupole)
    handle = model.handle()
    try:
        _check(L.tg_tree_record_group_stats(tree, 1), "group stats")
        _check(L.tg_theta_model_set_error_budget(handle, 0.0), "error budget")
        l10 = default_lambda(model, quadrupole) if log10_lambda is None else float(log10_lambda)
        out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _check(L.tg_tree_fields_learned(tree, _lib.TG_FIELD_ACCEL, int(quadrupole), float(G), GROUP_SIZE, handle,
                                        float(l10), 0.7, _lib.TG_MEM_DEVICE, _vp(out), st), "learned walk")
        first, _, _ = groups_of(tree, GROUP_SIZE)
        eta = np.empty(len(first), np.float32)
        _check(L.tg_tree_last_group_error(tree, _lib.ptr(eta), _lib.TG_MEM_HOST, st), "group error")
    finally:
        _check(L.tg_theta_model_set_error_budget(handle, model.error_budget), "error budget")
        L.tg_tree_free(tree)
    return eta


def target_group_errors(model, pos, h, pos_t, h_t, quadrupole, log10_lambda=None, G=1.0):
    """group_errors for external targets (a TargetSet of the sources' tree, m = 1/N)."""
    import torch

    n = len(pos)
    L = _lib.load()
    tree, keep = _tree_device(torch, pos, np.full(n, 1.0 / n), h, quadrupole)
    handle = model.handle()
    tset = ctypes.c_void_p()
    try:
        pt = np.ascontiguousarray(pos_t, np.float64)
        ht = np.ascontiguousarray(h_t, np.float64)
        _check(L.tg_targets_create(tree, _lib.ptr(pt), _lib.ptr(ht), len(pt), GROUP_SIZE, _lib.TG_MEM_HOST, None,
                                   ctypes.byref(tset)), "target set")
        _check(L.tg_tree_record_group_stats(tree, 1), "group stats")
        _check(L.tg_theta_model_set_error_budget(handle, 0.0), "error budget")
        l10 = default_lambda(model, quadrupole, True) if log10_lambda is None else float(log10_lambda)
        out = torch.empty((len(pt), 3), dtype=torch.float64, device="cuda")
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _check(L.tg_targets_fields_learned(tset, _lib.TG_FIELD_ACCEL, int(quadrupole), float(G), handle, float(l10),
                                           0.7, _lib.TG_MEM_DEVICE, _vp(out), st), "learned target walk")
        ng = ctypes.c_int64()
        _check(L.tg_targets_info(tset, None, ctypes.byref(ng)), "target set")
        eta = np.empty(ng.value, np.float32)
        _check(L.tg_tree_last_group_error(tree, _lib.ptr(eta), _lib.TG_MEM_HOST, st), "group error")
    finally:
        _check(L.tg_theta_model_set_error_budget(handle, model.error_budget), "error budget")
        if tset.value:
            L.tg_targets_free(tset)
        L.tg_tree_free(tree)
    return eta


def calibrate_error_budget(model, systems, factor=2.0, targets=()):
    """The error budget: `factor` times the largest per-group estimate seen on the training systems
    (own particles and external targets) at the model's calibrated lambdas, so that only groups
    outside anything met in training (a network asked about inputs unlike its data) are walked again
    at the global theta. Sets and returns it."""
    worst = 0.0
    for _, x, soft, quad in systems:
        eta = group_errors(model, x, soft, quad)
        worst = max(worst, float(np.max(eta)) if len(eta) else 0.0)
    for _, x, h, xt, ht, quad in targets:
        eta = target_group_errors(model, x, h, xt, ht, quad)
        worst = max(worst, float(np.max(eta)) if len(eta) else 0.0)
    model.error_budget = factor * worst
    return model.error_budget


def main(argv=None):
    ap = argparse.ArgumentParser(description="Train the learned opening-angle network on the GPU.")
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--scale", type=float, default=1.0, help="system size factor (smaller for a quick run)")
    ap.add_argument("--sample", type=float, default=0.25, help="fraction of groups judged by brute force")
    ap.add_argument("--target-ratio", type=float, default=0.85,
                    help="median training error relative to the plain walk at the default lambda")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--save-data", default=None, help="also save the training tables (.npz)")
    ap.add_argument("--kind", choices=sorted(KINDS), default="tolerance")
    ap.add_argument("--theta-max", type=float, default=THETA_CAP, help="angle cap of a tolerance model")
    ap.add_argument("--budget-only", action="store_true",
                    help="only calibrate the error budget of the model at --out (no training)")
    args = ap.parse_args(argv)
    if args.budget_only:
        model = ThetaModel.load(args.out)
        budget = calibrate_error_budget(model, training_systems(args.scale), targets=target_systems(args.scale))
        model.save(args.out)
        print(json.dumps(dict(out=args.out, error_budget=budget)))
        return model
    t0 = time.time()
    datasets = []
    for label, x, soft, quad in training_systems(args.scale):
        n = len(x)
        d = collect(x, np.full(n, 1.0 / n), np.full(n, soft), quadrupole=quad, sample=args.sample,
                    seed=args.seed + len(datasets), label=label, kind=args.kind, theta_max=args.theta_max)
        datasets.append(d)
        print(f"{label}: {d['ngroups']} groups, {d['sampled']} judged, plain RMS rel error {d['plain_rms_rel']:.3e}, "
              f"brute force {d['bf_seconds']:.2f} s", file=sys.stderr)
    if args.kind == "tolerance":
        for label, x, h, xt, ht, quad in target_systems(args.scale):
            n = len(x)
            d = collect(x, np.full(n, 1.0 / n), h, quadrupole=quad, sample=args.sample, seed=args.seed + len(datasets),
                        label=label, kind=args.kind, theta_max=args.theta_max, targets=(xt, ht))
            datasets.append(d)
            print(f"{label}: {d['ngroups']} target groups, {d['sampled']} judged, plain RMS rel error "
                  f"{d['plain_rms_rel']:.3e}, brute force {d['bf_seconds']:.2f} s", file=sys.stderr)
    t1 = time.time()
    if args.save_data:
        np.savez(args.save_data, **{f"{d['label']}/{k}": d[k] for d in datasets
                                    for k in ("features", "log_cost", "log_err")})
    model = train(datasets, steps=args.steps, batch=args.batch, lr=args.lr, seed=args.seed,
                  theta_max=args.theta_max)
    t2 = time.time()
    ratios = calibrate(model, datasets, target_ratio=args.target_ratio)
    budget = (calibrate_error_budget(model, training_systems(args.scale), targets=target_systems(args.scale))
              if model.kind == "tolerance" else 0.0)
    model.meta.update(collect_seconds=t1 - t0, train_seconds=t2 - t1, target_ratio=args.target_ratio)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    model.save(args.out)
    summary = dict(out=args.out, kind=model.kind, theta_max=model.theta_max, log10_lambda=model.log10_lambda,
                   error_budget=budget, lambdas={_lambda_key(q, t): model.meta.get(_lambda_key(q, t)) for q, t in MODES},
                   ratios={d["label"]: dict(error=e, cost=c, speedup=1.0 / c) for d, (e, c) in zip(datasets, ratios)},
                   collect_s=round(t1 - t0, 1), train_s=round(t2 - t1, 1))
    print(json.dumps(summary))
    return model


if __name__ == "__main__":
    main()
