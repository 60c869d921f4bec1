"""Parity of whole reconstructions at their full iteration counts against the
FP64 oracle, from committed fixtures (``tests/golden/make_fullrun.py``):

* the clinical workload, 1024x512x60 voxels, 25 views, 50 iterations x 25
  subsets = 1250 sub-iterations, Huber, through ``ostr.reconstruct``;
* case 8 of the mixed batch (710x339x33 voxels, 9 views, hyperbola), 50
  iterations x 9 subsets, advanced inside a ``Batch`` next to another case of
  a different size and view count.

The fixtures hold the oracle's volume at every stride-th voxel, its per-slice
sums and its FP64 objective; running the oracle itself takes minutes.  The
inputs are rebuilt here from the same seeds (phantom, oracle FP64 forward
projection, Poisson counts), and their per-view count sums must equal the
fixture's before anything is compared.

Bars: relative RMSE over the sampled voxels <= 1e-4 (the bar of every OSTR
parity test here; the sample of 2^18 voxels estimates the full-volume figure
to well under 1 %), per-slice sums within 1e-4 relative, and the FP64
objective of the GPU volume (evaluated by the oracle) within 1e-9 of the
oracle volume's.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

REL_RMSE_BAR = 1e-4
OBJ_BAR = 1e-9


def _inputs(name):
    import make_fullrun

    fx = np.load(os.path.join(HERE, "golden", f"fullrun_{name}.npz"))
    cfg, _, y, b = make_fullrun.workload(name)
    # the inputs are the fixture's, bit for bit (integer counts summed in double)
    np.testing.assert_array_equal(make_fullrun.count_sums(cfg, y), fx["count_sums"])
    assert int(fx["iter_num"]) == cfg.iter_num and int(fx["subset_num"]) == cfg.subset_num
    return fx, cfg, y, b


def _compare(name, fx, cfg, y, b, vol):
    import make_fullrun
    from oracle.oracle import Oracle

    vol = np.asarray(vol, np.float32).ravel()
    s = make_fullrun.summary(cfg, vol)
    ref = fx["samples"].astype(np.float64)
    diff = s["samples"].astype(np.float64) - ref
    rmse = np.sqrt(np.mean(diff ** 2))
    rel = rmse / np.sqrt(np.mean(ref ** 2))
    sl = np.abs(s["slice_sums"] - fx["slice_sums"]) / np.maximum(np.abs(fx["slice_sums"]), 1e-30)
    data, pen = Oracle(np.float64).objective(cfg.geom, cfg.angles, y, b, vol,
                                             potential=cfg.potential, delta=cfg.delta)
    tg = data + cfg.beta * pen
    to = float(fx["objective"][0] + cfg.beta * fx["objective"][1])
    print(f"{name} {cfg.iter_num} x {cfg.subset_num}: rel RMSE {rel:.2e}  RMSE {rmse:.2e}/mm  "
          f"max-abs {np.abs(diff).max():.2e}/mm (over {ref.size} sampled voxels); "
          f"slice sums max rel {sl.max():.2e}; objective oracle {to:.12e} GPU {tg:.12e} "
          f"(rel {abs(tg - to) / abs(to):.2e})")
    assert np.isfinite(vol).all() and (vol >= 0).all()
    assert rel <= REL_RMSE_BAR
    assert sl.max() <= REL_RMSE_BAR
    assert abs(tg - to) <= OBJ_BAR * abs(to)


def test_clinical_fifty_iterations_match_fp64_oracle():
    from newrecon_gb300 import native, ostr

    native.load()
    fx, cfg, y, b = _inputs("clinical")
    vol = ostr.reconstruct(cfg.geom, y, b, angles=cfg.angles, subset_num=cfg.subset_num,
                           iter_num=cfg.iter_num, beta=cfg.beta, delta=cfg.delta,
                           potential=cfg.potential)
    _compare("clinical", fx, cfg, y, b, vol)


def test_mixed_batch_case_matches_fp64_oracle_at_full_iterations():
    import torch

    from newrecon_gb300 import native, ostr
    from newrecon_gb300.geometry import batch_configs
    from newrecon_gb300.phantom import breast_phantom, poisson_counts
    from oracle.oracle import Oracle

    native.load()
    fx, cfg, y, b = _inputs("batch8")
    # a neighbour case of another size, view count and iteration count in the same batch
    other = batch_configs(16, seed=7)[15]
    g2 = other.geom
    x2 = breast_phantom(g2, other.seed, 0, other.n_calc, thickness_mm=other.thickness_mm,
                        glandular_fraction=other.n_glandular / 100.0).ravel()
    y2 = poisson_counts(Oracle(np.float64).fp_ostr(g2, x2, other.angles,
                                                   np.arange(g2.n_angles, dtype=np.int32), 0,
                                                   g2.n_angles), other.I0, other.seed)
    cases = [dict(geom=cfg.geom, angles=cfg.angles, prj=y, blank=b, subset_num=cfg.subset_num,
                  iter_num=cfg.iter_num, beta=cfg.beta, delta=cfg.delta,
                  potential=cfg.potential),
             dict(geom=g2, angles=other.angles, prj=y2, blank=np.full_like(y2, other.I0),
                  subset_num=other.subset_num, iter_num=20, beta=other.beta, delta=other.delta,
                  potential=other.potential)]
    bt = ostr.Batch(cases)
    vols = bt.run()
    torch.cuda.synchronize()
    _compare("batch8", fx, cfg, y, b, vols[0].cpu().numpy())
