"""Learned warm start for OSTR: a small 3D residual CNN on the tensor cores.

An early OSTR iterate (after 2 iterations) goes in; the network predicts the
converged volume (50 iterations) as x_warm = max(0, x + f(s x)/s); OSTR then
continues from x_warm.  Plain OSTR is both the fallback and the arbiter: the
warm start is kept only if, at equal total subset-iterations, its FP64
penalized-likelihood objective is no worse than plain OSTR's.

The network and its training run entirely in libnrgb300 (nr_cnn_*): BF16
implicit-GEMM convolutions on tcgen05 with FP32 accumulation in TMEM, the
backward pass and Adam.  Training pairs come from OSTR itself on seeded
phantoms; patches of the volumes are the training samples.
"""
from __future__ import annotations

import ctypes
import dataclasses
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import native
from .ostr import OSTR, _device, _stream

DEFAULT_SCALE = 20.0  # u = s x: attenuation of ~0.05 /mm becomes O(1)


class NrCnnDims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("nb", ctypes.c_int32)]


def param_count() -> int:
    n = ctypes.c_int64(0)
    native.call("nr_cnn_param_count", ctypes.byref(n))
    return int(n.value)


def init_params(seed: int, last_scale: float = 0.0) -> np.ndarray:
    """He-normal weights, zero biases; the last layer starts at last_scale x He
    (0: the network starts as the identity warm start x_warm = x)."""
    rng = np.random.default_rng(seed)
    layers = [(1, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 1)]
    out = []
    for l, (ni, no) in enumerate(layers):
        w = rng.normal(scale=np.sqrt(2.0 / (27 * ni)), size=27 * no * ni)
        if l == 5:
            w = w * last_scale
        out.append(w)
        out.append(np.zeros(no))
    p = np.concatenate(out).astype(np.float32)
    assert p.size == param_count()
    return p


def _p(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


class WarmStartCNN:
    """Parameters, Adam state and workspaces of the warm-start network."""

    def __init__(self, params: Optional[np.ndarray] = None, seed: int = 0,
                 scale: float = DEFAULT_SCALE):
        dev = _device()
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        self.params = torch.from_numpy(p.copy()).to(dev)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.scale = float(scale)
        self._ws: Dict[Tuple[int, int, int, int, int], torch.Tensor] = {}
        self._loss = torch.zeros(1, dtype=torch.float64, device=dev)

    def _workspace(self, dims: Tuple[int, int, int, int], training: bool):
        key = tuple(dims) + (int(training),)
        d = NrCnnDims(*dims)
        if key not in self._ws:
            n = ctypes.c_size_t(0)
            native.call("nr_cnn_workspace_size", ctypes.byref(d), int(training), ctypes.byref(n))
            self._ws[key] = torch.zeros(int(n.value), dtype=torch.uint8, device=self.params.device)
        ws = self._ws[key]
        return d, ws

    def forward(self, x: torch.Tensor, dims: Tuple[int, int, int, int],
                out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """x_warm for x ([nb][nz][ny][nx] float32 on the device)."""
        d, ws = self._workspace(dims, False)
        out = torch.empty_like(x) if out is None else out
        native.call("nr_cnn_forward", ctypes.byref(d), _p(self.params), _p(x),
                    ctypes.c_float(self.scale), _p(out), _p(ws), ctypes.c_size_t(ws.numel()),
                    _stream())
        return out

    def loss_grad(self, x: torch.Tensor, target: torch.Tensor,
                  dims: Tuple[int, int, int, int]) -> Tuple[float, torch.Tensor]:
        d, ws = self._workspace(dims, True)
        grad = torch.empty_like(self.params)
        native.call("nr_cnn_loss_grad", ctypes.byref(d), _p(self.params), _p(x), _p(target),
                    ctypes.c_float(self.scale), _p(grad), _p(self._loss), _p(ws),
                    ctypes.c_size_t(ws.numel()), _stream())
        return float(self._loss.item()), grad

    def train_step(self, x: torch.Tensor, target: torch.Tensor, dims: Tuple[int, int, int, int],
                   lr: float) -> torch.Tensor:
        """One Adam step on a batch; returns the (device) loss before the step."""
        d, ws = self._workspace(dims, True)
        self.step += 1
        native.call("nr_cnn_train_step", ctypes.byref(d), _p(self.params), _p(self.m), _p(self.v),
                    self.step, ctypes.c_float(lr), _p(x), _p(target), ctypes.c_float(self.scale),
                    _p(self._loss), _p(ws), ctypes.c_size_t(ws.numel()), _stream())
        return self._loss

    def adam(self, grad: torch.Tensor, lr: float) -> None:
        self.step += 1
        native.call("nr_cnn_adam", _p(self.params), _p(self.m), _p(self.v), _p(grad),
                    int(self.params.numel()), self.step, ctypes.c_float(lr), _stream())

    def check(self) -> None:
        flags = ctypes.c_int32(0)
        for ws in self._ws.values():
            native.call("nr_cnn_check", _p(ws), ctypes.byref(flags), _stream())

    def state(self) -> np.ndarray:
        return self.params.cpu().numpy()


# ---------------------------------------------------------------------------
# Training data, training, evaluation.

@dataclasses.dataclass
class TrainConfig:
    """Training / validation recipe (seeded end to end)."""

    n_train: int = 512               # training phantoms
    n_val: int = 64                  # held-out phantoms
    crop: Tuple[int, int] = (256, 128)   # in-plane voxels per case (0.14 mm), full thickness
    early_iters: int = 2             # the network's input: OSTR after this many iterations
    full_iters: int = 50             # the target: OSTR after this many iterations
    after_iters: int = 3             # OSTR iterations after the warm start
    patch: Tuple[int, int, int] = (126, 32, 16)  # training patch (nx, ny, nz): one 126-wide
                                                 # tile of the dx-stacked convolution per row
    batch: int = 8                   # patches per Adam step
    steps: int = 2000
    lr: float = 2e-3
    seed: int = 10_000               # training seeds seed .. seed+n_train-1, validation after
    workers: int = 8                 # processes generating phantoms
    last_scale: float = 0.1          # initial scale of the last layer (x He)
    workload: str = "batch"          # "batch": the batched workload's statistics (hyperbola,
                                     # delta 0.002, beta 50); "clinical": the clinical
                                     # workload's (25 views over +-25 deg, I0 5e3, 60 slices,
                                     # Huber delta 0.003, beta 100); "fullres": the
                                     # full-resolution workload's (0.085 mm, 70 slices, 15
                                     # views over +-7.5 deg, I0 4e3, hyperbola 0.002 / 200)


def case_configs(n: int, seed: int, crop: Tuple[int, int], workload: str = "batch"):
    """Cases on a cropped in-plane field with the detector fitted to the
    volume's shadow: the batched workload's statistics (uneven thickness /
    views / dose; hyperbola) or the clinical workload's (Huber)."""
    from .geometry import Geometry, ReconConfig, view_angles

    if workload not in ("batch", "clinical", "fullres"):
        raise ValueError(f"unknown workload {workload!r}")
    out = []
    for c in range(n):
        rng = np.random.default_rng(seed + c)
        if workload == "fullres":
            # the full-resolution workload: 0.085 mm, 70 slices, 15 views over
            # +-7.5 deg, I0 4e3, hyperbola delta 0.002, beta 200
            nx, ny = crop
            gland = float(rng.uniform(0.10, 0.50))
            g0 = Geometry.dbt(nx, ny, 70, 0.085, 1.0, 8, 8, 0.085, 15)
            angles = view_angles(15, 7.5)
            g = fit_detector(g0, angles)
            out.append(ReconConfig(f"case{seed + c}", g, angles, 4e3, 15, 50, "hyperbola", 200.0,
                                   0.002, int(round(100 * gland)), 10, 70.0, seed + c))
            continue
        if workload == "clinical":
            nx, ny = crop
            gland = float(rng.uniform(0.10, 0.50))
            g0 = Geometry.dbt(nx, ny, 60, 0.14, 1.0, 8, 8, 0.14, 25)
            angles = view_angles(25, 25.0)
            g = fit_detector(g0, angles)
            out.append(ReconConfig(f"case{seed + c}", g, angles, 5e3, 25, 50, "huber", 100.0,
                                   0.003, int(round(100 * gland)), 10, 60.0, seed + c))
            continue
        nz = int(round(rng.uniform(30, 80)))
        views = int(rng.choice([9, 15, 25]))
        span = float(rng.uniform(7.5, 25.0))
        I0 = float(rng.uniform(3e3, 2e4))
        gland = float(rng.uniform(0.10, 0.50))
        nx, ny = crop
        g0 = Geometry.dbt(nx, ny, nz, 0.14, 1.0, 8, 8, 0.14, views)
        angles = view_angles(views, span)
        g = fit_detector(g0, angles)
        out.append(ReconConfig(f"case{seed + c}", g, angles, I0, views, 50, "hyperbola", 50.0,
                               0.002, int(round(100 * gland)), 10, float(nz), seed + c))
    return out


def fit_detector(g, angles, margin: int = 4):
    """A detector on the 0.14 mm bin grid covering the volume's shadow in every view."""
    xs = [g.x_p0, g.x_p0 + g.nx * g.vx]
    ys = [g.y_p0, g.y_p0 + g.ny * g.vy]
    zs = [g.z_p0, g.z_p0 + g.nz * g.vz]
    lo = [np.inf, np.inf]
    hi = [-np.inf, -np.inf]
    for th in np.asarray(angles, np.float64):
        sx, sy, sz = g.sourceR * np.sin(th), g.sourceY, g.sourceR * np.cos(th)
        for x in xs:
            for y in ys:
                for z in zs:
                    t = (-g.detectorR - sz) / (z - sz)
                    px, py = sx + (x - sx) * t, sy + (y - sy) * t
                    lo = [min(lo[0], px), min(lo[1], py)]
                    hi = [max(hi[0], px), max(hi[1], py)]
    b = g.bx
    i0 = int(np.floor(lo[0] / b)) - margin
    i1 = int(np.ceil(hi[0] / b)) + margin
    j0 = int(np.floor(lo[1] / b)) - margin
    j1 = int(np.ceil(hi[1] / b)) + margin
    return dataclasses.replace(g, nbx=i1 - i0, nby=j1 - j0, x_d0=i0 * b, y_d0=j0 * b)


def _phantom_job(args):
    from .phantom import breast_phantom

    g, seed, gland, n_calc = args
    return breast_phantom(g, seed, 0, n_calc, glandular_fraction=gland).ravel()


def phantoms(cfgs, workers: int) -> List[np.ndarray]:
    """Seeded phantoms, generated in `workers` spawned processes."""
    jobs = [(c.geom, c.seed, c.n_glandular / 100.0, c.n_calc) for c in cfgs]
    if workers <= 1:
        return [_phantom_job(j) for j in jobs]
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_phantom_job, jobs)


@dataclasses.dataclass
class Pair:
    cfg: object
    x_early: torch.Tensor
    x_full: torch.Tensor
    y: np.ndarray
    b: np.ndarray
    x_true: Optional[np.ndarray] = None  # the phantom


def make_pairs(cfgs, phantom_vols, early: int, full: int) -> List[Pair]:
    """OSTR on each phantom's Poisson scan: the early iterate and the target."""
    from . import ostr
    from .phantom import poisson_counts

    out = []
    for c, xt in zip(cfgs, phantom_vols):
        g = c.geom
        ostr.set_geometry(g)
        idx = np.arange(g.n_angles, dtype=np.int32)
        line = torch.zeros(g.n_angles * g.n_bins, device="cuda")
        ostr.fprojectCB_1R_GPU_OSTR_cos(torch.from_numpy(xt).cuda(), line,
                                        torch.from_numpy(c.angles).cuda(),
                                        torch.from_numpy(idx).cuda(), 0, g.n_angles)
        y = poisson_counts(line.cpu().numpy(), c.I0, c.seed)
        b = np.full_like(y, c.I0)
        plan = OSTR(g, subset_num=c.subset_num, beta=c.beta, delta=c.delta,
                    potential=c.potential)
        plan.setup(c.angles, y, b)
        x = torch.zeros(g.n_voxels, device="cuda")
        plan.iterate(x, early)
        x_early = x.clone()
        plan.iterate(x, full - early)
        plan.check()
        out.append(Pair(c, x_early, x.clone(), y, b, xt))
    return out


def sample_batch(pairs: Sequence[Pair], patch, batch: int, rng: np.random.Generator):
    px, py, pz = patch
    xs, ts = [], []
    for _ in range(batch):
        p = pairs[int(rng.integers(len(pairs)))]
        g = p.cfg.geom
        x0 = int(rng.integers(0, g.nx - px + 1))
        y0 = int(rng.integers(0, g.ny - py + 1))
        z0 = int(rng.integers(0, g.nz - pz + 1))
        sl = (slice(z0, z0 + pz), slice(y0, y0 + py), slice(x0, x0 + px))
        xs.append(p.x_early.view(g.nz, g.ny, g.nx)[sl])
        ts.append(p.x_full.view(g.nz, g.ny, g.nx)[sl])
    return (torch.stack(xs).contiguous().view(-1), torch.stack(ts).contiguous().view(-1),
            (px, py, pz, batch))


def train(cnn: WarmStartCNN, pairs: Sequence[Pair], cfg: TrainConfig, log_every: int = 100):
    """Adam with a cosine-decayed learning rate; returns [(step, loss), ...]."""
    rng = np.random.default_rng(cfg.seed + 7)
    hist = []
    for s in range(cfg.steps):
        lr = cfg.lr * 0.5 * (1.0 + np.cos(np.pi * s / cfg.steps))
        xb, tb, dims = sample_batch(pairs, cfg.patch, cfg.batch, rng)
        loss = cnn.train_step(xb, tb, dims, max(lr, 1e-6))
        if s % log_every == 0 or s == cfg.steps - 1:
            hist.append((s, float(loss.item())))
    cnn.check()
    return hist


def _rmse(a: torch.Tensor, b: torch.Tensor) -> float:
    return float(torch.sqrt(torch.mean((a.double() - b.double()) ** 2)).item())


def warm_start_volume(cnn: WarmStartCNN, x_early: torch.Tensor, g) -> torch.Tensor:
    """x_warm for a whole volume (one patch of the full size)."""
    return cnn.forward(x_early, (g.nx, g.ny, g.nz, 1))


def evaluate(cnn: WarmStartCNN, pair: Pair, after: int, early: int = 2,
             rmse_tol: float = 1e-4, max_iters: int = 60) -> dict:
    """Warm start vs plain OSTR on one case, judged on the FP64 objective at
    equal total subset-iterations and on RMSE against the target x_full.

    Wall times are measured with the plan set up (scan resident on the GPU),
    from x = 0: plain OSTR counts iterations to reach RMSE <= rmse_tol; the
    warm start counts early iterations + inference + iterations after it.
    """
    c = pair.cfg
    g = c.geom
    plan = OSTR(g, subset_num=c.subset_num, beta=c.beta, delta=c.delta, potential=c.potential)
    plan.setup(c.angles, pair.y, pair.b)
    M = c.subset_num
    ref = pair.x_full
    # equal-work comparison
    xp = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(xp, early + after)
    xe = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(xe, early)
    xw = warm_start_volume(cnn, xe, g)
    plan.iterate(xw, after)
    plan.check()
    obj_plain = plan.total_objective(xp)
    obj_warm = plan.total_objective(xw)
    obj_ref = plan.total_objective(ref)
    accept = obj_warm <= obj_plain
    out = dict(case=c.name, subsets=M, early=early, after=after,
               objective_plain=obj_plain, objective_warm=obj_warm, objective_full=obj_ref,
               rmse_plain=_rmse(xp, ref), rmse_warm=_rmse(xw, ref),
               max_abs_plain=float((xp - ref).abs().max().item()),
               max_abs_warm=float((xw - ref).abs().max().item()), accepted=bool(accept))
    # time to RMSE <= tol: plain
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = torch.zeros(g.n_voxels, device="cuda")
    it_plain = None
    for k in range(1, max_iters + 1):
        plan.iterate(x, 1)
        if _rmse(x, ref) <= rmse_tol:
            it_plain = k
            break
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, early)
    x = warm_start_volume(cnn, x, g)
    it_warm = None
    for k in range(1, max_iters + 1):
        plan.iterate(x, 1)
        if _rmse(x, ref) <= rmse_tol:
            it_warm = k
            break
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    out.update(rmse_tol=rmse_tol, iters_to_tol_plain=it_plain, seconds_to_tol_plain=t_plain,
               iters_to_tol_warm=None if it_warm is None else early + it_warm,
               seconds_to_tol_warm=t_warm)
    if max_iters > 0 and pair.x_true is not None:
        out.update(criteria(cnn, plan, pair, early, full=max_iters))
    return out


def criteria(cnn: WarmStartCNN, plan, pair: Pair, early: int, full: int = 50,
             frac: float = 0.01) -> dict:
    """The warm start against plain OSTR on the two criteria of the target:
    (a) the FP64 objective within `frac` of plain OSTR's objective gap after
    `full` iterations: f(x) - f_full <= frac (f(0) - f_full); (b) RMSE
    against the phantom within `frac` of plain OSTR's after `full`
    iterations: rmse(x) <= (1 + frac) rmse_full.  Iterations to each (early
    iterations and the network counted for the warm start), and wall times:
    the measured time of one iteration times the iterations, plus the
    network's measured time for the warm start."""
    g = pair.cfg.geom
    truth = torch.from_numpy(np.asarray(pair.x_true, np.float32)).cuda()
    dims = (g.nx, g.ny, g.nz, 1)

    def track(x, n):
        fs, rs = [plan.total_objective(x)], [_rmse(x, truth)]
        for _ in range(n):
            plan.iterate(x, 1)
            fs.append(plan.total_objective(x))
            rs.append(_rmse(x, truth))
        return fs, rs

    fp, rp = track(torch.zeros(g.n_voxels, device="cuda"), full)
    f0, f_full, r_full = fp[0], fp[-1], rp[-1]
    xw = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(xw, early)
    xw = warm_start_volume(cnn, xw, g)
    fw, rw = track(xw, full - early)

    def first(vals, ok, offset):
        for k, v in enumerate(vals):
            if ok(v):
                return offset + k
        return None

    obj_ok = lambda f: f - f_full <= frac * (f0 - f_full)
    rmse_ok = lambda r: r <= (1.0 + frac) * r_full
    # timings: one plain iteration and one network pass, on this volume
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan.iterate(x, 2)
    torch.cuda.synchronize()
    t_it = (time.perf_counter() - t0) / 2
    t0 = time.perf_counter()
    cnn.forward(x, dims)
    torch.cuda.synchronize()
    t_cnn = time.perf_counter() - t0
    res = {"criteria_frac": frac, "objective_gap_full": f0 - f_full, "rmse_phantom_full": r_full,
           "seconds_per_iteration": t_it, "seconds_cnn": t_cnn}
    for name, ok, vp, vw in (("objective", obj_ok, fp, fw), ("rmse_phantom", rmse_ok, rp, rw)):
        kp = first(vp, ok, 0)
        kw = first(vw, ok, early)
        tp = None if kp is None else kp * t_it
        tw = None if kw is None else kw * t_it + t_cnn
        res[name] = {"iters_plain": kp, "iters_warm": kw, "seconds_plain": tp,
                     "seconds_warm": tw, "speedup": (tp / tw) if (tp and tw) else None}
    return res


def warm_reconstruct(cnn: WarmStartCNN, geom, prj, blank, *, angles, subset_num: int,
                     iter_num: int, beta: float, delta: float, potential: str = "hyperbola",
                     early: int = 2, scat=None) -> Tuple[torch.Tensor, dict]:
    """OSTR with the learned warm start and plain OSTR as fallback and judge.

    Runs `early` iterations, the network, then `iter_num - early` iterations;
    the same number of plain iterations is run from the early iterate, and the
    result with the lower FP64 objective is returned with a report."""
    plan = OSTR(geom, subset_num=subset_num, beta=beta, delta=delta, potential=potential,
                has_scatter=scat is not None)
    plan.setup(angles, prj, blank, scat)
    x = torch.zeros(geom.n_voxels, device=plan.ws.device)
    plan.iterate(x, early)
    xw = warm_start_volume(cnn, x, geom)
    rest = max(iter_num - early, 0)
    plan.iterate(xw, rest)
    plan.iterate(x, rest)
    plan.check()
    ow, op = plan.total_objective(xw), plan.total_objective(x)
    keep = ow <= op
    return (xw if keep else x), dict(objective_warm=ow, objective_plain=op, accepted=keep)


def run(cfg: TrainConfig, out_params: Optional[str] = None, n_time: int = 4,
        log=print) -> dict:
    """The whole recipe: data, training, held-out evaluation.  Returns a report."""
    t0 = time.perf_counter()
    tr_cfgs = case_configs(cfg.n_train, cfg.seed, cfg.crop, cfg.workload)
    va_cfgs = case_configs(cfg.n_val, cfg.seed + cfg.n_train, cfg.crop, cfg.workload)
    vols = phantoms(tr_cfgs + va_cfgs, cfg.workers)
    t1 = time.perf_counter()
    pairs = make_pairs(tr_cfgs, vols[:cfg.n_train], cfg.early_iters, cfg.full_iters)
    val = make_pairs(va_cfgs, vols[cfg.n_train:], cfg.early_iters, cfg.full_iters)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    log(f"data: {len(pairs)} train + {len(val)} held-out pairs; phantoms {t1 - t0:.1f} s, "
        f"OSTR pairs {t2 - t1:.1f} s")
    cnn = WarmStartCNN(init_params(cfg.seed, last_scale=cfg.last_scale))
    hist = train(cnn, pairs, cfg)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    log(f"train: {cfg.steps} steps in {t3 - t2:.1f} s, loss {hist[0][1]:.3e} -> {hist[-1][1]:.3e}")
    evals = []
    for k, p in enumerate(val):
        e = evaluate(cnn, p, cfg.after_iters, cfg.early_iters,
                     max_iters=cfg.full_iters if k < n_time else 0)
        evals.append(e)
    t4 = time.perf_counter()
    acc = [e["accepted"] for e in evals]
    rep = {
        "config": dataclasses.asdict(cfg),
        "params": int(cnn.params.numel()),
        "loss_history": hist,
        "seconds": {"phantoms": t1 - t0, "ostr_pairs": t2 - t1, "train": t3 - t2,
                    "eval": t4 - t3},
        "held_out": evals,
        "accept_rate": float(np.mean(acc)) if acc else None,
        "mean_objective_gain": float(np.mean([(e["objective_plain"] - e["objective_warm"])
                                              / abs(e["objective_plain"]) for e in evals])),
        "mean_rmse_plain": float(np.mean([e["rmse_plain"] for e in evals])),
        "mean_rmse_warm": float(np.mean([e["rmse_warm"] for e in evals])),
    }
    timed = [e for e in evals if "objective" in e]
    for name in ("objective", "rmse_phantom"):
        sp = [e[name]["speedup"] for e in timed if e[name]["speedup"] is not None]
        rep[f"speedup_{name}"] = {"cases": len(timed), "reached_by_both": len(sp),
                                  "mean": float(np.mean(sp)) if sp else None,
                                  "min": float(np.min(sp)) if sp else None,
                                  "max": float(np.max(sp)) if sp else None}
    if out_params:
        np.savez_compressed(out_params, params=cnn.state(), scale=cnn.scale,
                            early_iters=cfg.early_iters, workload=cfg.workload)
    return rep


def time_forward(dims: Tuple[int, int, int], reps: int = 5) -> dict:
    """Wall time of the network's forward pass on a seeded volume of dims =
    (nx, ny, nz) with seeded weights: 3 warm-up passes, then `reps` timed."""
    nx, ny, nz = dims
    n = nx * ny * nz
    gen = torch.Generator(device="cuda").manual_seed(1)
    x = torch.rand(n, device="cuda", generator=gen) * 0.1
    cnn = WarmStartCNN(init_params(3, last_scale=0.5), scale=20.0)
    shape = (nx, ny, nz, 1)
    for _ in range(3):
        cnn.forward(x, shape)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        cnn.forward(x, shape)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    cnn.check()
    flops = n * 2 * 27 * (32 + 4 * 32 * 32 + 32)
    return {"dims": list(dims), "ms": dt * 1e3, "tflops": flops / dt / 1e12}


def load(path: str) -> WarmStartCNN:
    z = np.load(path)
    return WarmStartCNN(z["params"], scale=float(z["scale"]))


def main(argv=None) -> int:
    import argparse
    import json

    ap = argparse.ArgumentParser(description="train and evaluate the OSTR warm-start CNN")
    ap.add_argument("--n-train", type=int, default=512)
    ap.add_argument("--n-val", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--n-time", type=int, default=4)
    ap.add_argument("--workload", default="batch", choices=["batch", "clinical", "fullres"])
    ap.add_argument("--time-forward", type=int, nargs=3, metavar=("NX", "NY", "NZ"),
                    default=None,
                    help="only time the network's forward pass on a seeded NX x NY x NZ "
                         "volume (3 warm-up and 5 timed passes) and exit")
    ap.add_argument("--crop", type=int, nargs=2, default=[256, 128])
    ap.add_argument("--out", default=None, help="write the trained parameters (.npz)")
    ap.add_argument("--report", default=None, help="write the JSON report")
    a = ap.parse_args(argv)
    from . import native as _n

    _n.load()
    if a.time_forward:
        print(json.dumps(time_forward(tuple(a.time_forward))))
        return 0
    cfg = TrainConfig(n_train=a.n_train, n_val=a.n_val, steps=a.steps, batch=a.batch, lr=a.lr,
                      workers=a.workers, workload=a.workload, crop=tuple(a.crop))
    rep = run(cfg, a.out, n_time=a.n_time)
    txt = json.dumps(rep, indent=1, default=float)
    if a.report:
        with open(a.report, "w") as f:
            f.write(txt)
    summary = {k: rep[k] for k in ("accept_rate", "mean_objective_gain", "mean_rmse_plain",
                                   "mean_rmse_warm", "seconds", "speedup_objective",
                                   "speedup_rmse_phantom")}
    print(json.dumps(summary, default=float))
    return 0


if __name__ == "__main__":
    import sys

    sys.exit(main())
