"""Generates the whole-run parity fixtures: the FP64 oracle's reconstruction of
a workload at its full iteration count, stored compactly so that the GPU test
does not have to run the oracle for minutes.

    python tests/golden/make_fullrun.py              # both fixtures
    python tests/golden/make_fullrun.py clinical     # one of them

Fixtures:

``fullrun_clinical.npz``  the clinical workload (1024x512x60 voxels of
                          0.14x0.14x1 mm, 1664x832 detector, 25 views over
                          +-25 deg, I0 5e3), 50 iterations x 25 subsets =
                          1250 sub-iterations, Huber delta 0.003, beta 100.
``fullrun_batch8.npz``    case 8 of the mixed batch (``batch_configs(16,
                          seed=7)``: 710x339x33 voxels, 9 views, I0 9451,
                          glandular fraction 38 %), 50 iterations x 9 subsets,
                          hyperbola delta 0.002, beta 50.

Inputs are rebuilt from seeds on any machine: the phantom (numpy), then the
counts y ~ Poisson(I0 exp(-FP(phantom))) with FP the FP64 oracle's forward
projector (built with -ffp-contract=off, so x86 and Arm give the same bits).
The fixture stores, besides the oracle's output, the per-view sums of the
counts so that a test can check it rebuilt the same inputs.

Output summary (float64 unless noted): per-slice sums of the volume, the
volume at every ``stride``-th voxel (float32), the FP64 objective (data term,
penalty) of the oracle volume, and the run's parameters.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from newrecon_gb300.geometry import batch_configs, config  # noqa: E402
from newrecon_gb300.phantom import breast_phantom, poisson_counts  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

SAMPLES = 1 << 18   # voxel samples stored per fixture


def workload(name: str):
    """(config, phantom, counts, blank) of a whole-run fixture, rebuilt from seeds."""
    if name == "clinical":
        cfg = config("clinical", seed=0)
        x = breast_phantom(cfg.geom, 0, cfg.n_glandular, cfg.n_calc,
                           thickness_mm=cfg.thickness_mm)
        seed = 0
    elif name == "batch8":
        cfg = batch_configs(16, seed=7)[8]
        x = breast_phantom(cfg.geom, cfg.seed, 0, cfg.n_calc, thickness_mm=cfg.thickness_mm,
                           glandular_fraction=cfg.n_glandular / 100.0)
        seed = cfg.seed
    else:
        raise KeyError(name)
    g = cfg.geom
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = Oracle(np.float64).fp_ostr(g, x.ravel(), cfg.angles, idx, 0, g.n_angles)
    y = poisson_counts(line, cfg.I0, seed)
    return cfg, x.ravel(), y, np.full_like(y, cfg.I0)


def count_sums(cfg, y) -> np.ndarray:
    return y.reshape(cfg.geom.n_angles, -1).astype(np.float64).sum(axis=1)


def stride_of(n_voxels: int) -> int:
    return max(1, n_voxels // SAMPLES)


def summary(cfg, vol) -> dict:
    g = cfg.geom
    v = np.asarray(vol, np.float64).reshape(g.nz, -1)
    st = stride_of(g.n_voxels)
    return dict(slice_sums=v.sum(axis=1), stride=np.int64(st),
                samples=np.asarray(vol).ravel()[::st].astype(np.float32))


def make(name: str) -> str:
    t0 = time.time()
    cfg, _, y, b = workload(name)
    t1 = time.time()
    kw = dict(subset_num=cfg.subset_num, iter_num=cfg.iter_num, beta=cfg.beta, delta=cfg.delta,
              potential=cfg.potential)
    O = Oracle(np.float64)
    xo = O.reconstruct(cfg.geom, cfg.angles, y, b, **kw)
    t2 = time.time()
    data, pen = O.objective(cfg.geom, cfg.angles, y, b, xo, potential=cfg.potential,
                            delta=cfg.delta)
    out = dict(count_sums=count_sums(cfg, y), objective=np.array([data, pen]),
               subset_num=np.int32(cfg.subset_num), iter_num=np.int32(cfg.iter_num),
               beta=np.float64(cfg.beta), delta=np.float64(cfg.delta),
               potential=np.array(cfg.potential), oracle_threads=np.int32(O.max_threads),
               oracle_seconds=np.float64(t2 - t1))
    out.update(summary(cfg, xo))
    path = os.path.join(HERE, f"fullrun_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: inputs {t1 - t0:.1f} s, oracle {cfg.iter_num} x {cfg.subset_num} "
          f"{t2 - t1:.1f} s on {O.max_threads} threads; objective {data + cfg.beta * pen:.12e}")
    return path


if __name__ == "__main__":
    names = sys.argv[1:] or ["batch8", "clinical"]
    for n in names:
        make(n)
