"""Parity at the full workload sizes: the clinical workload (1024x512x60
voxels, 1664x832 detector, 25 views, Huber) and the full-resolution workload
(2048x1024x70 voxels, 3328x1664 detector, 15 views, hyperbola).  One OSTR
iteration (every subset once, from x = 0, with the gamma/d set-up) runs on the
GPU and in the FP64 oracle (OpenMP over the host cores) on the same seeded
counts.  Bar: relative RMSE of the volume <= 1e-4, the same bar as the small
cases; RMSE and max-abs (1/mm) are printed.

The whole 50-iteration clinical reconstruction is checked against the oracle
in test_gpu_fullrun.py, from a committed fixture.

Besides the volume, two size-independent properties are checked on the GPU at
full size: the forward projector is linear (FP(a x1 + x2) = a FP(x1) + FP(x2)
to float rounding) and the update keeps the volume non-negative and finite.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

REL_RMSE_BAR = 1e-4


@pytest.fixture(scope="module")
def mod():
    from newrecon_gb300 import native, ostr

    native.load()
    return ostr


def scan(mod, name):
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts

    cfg = config(name, seed=0)
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc, thickness_mm=cfg.thickness_mm)
    mod.set_geometry(g)
    idx = torch.arange(g.n_angles, dtype=torch.int32, device="cuda")
    line = torch.zeros(g.n_angles * g.n_bins, device="cuda")
    mod.fprojectCB_1R_GPU_OSTR_cos(torch.from_numpy(x.ravel()).cuda(), line,
                                   torch.from_numpy(cfg.angles).cuda(), idx, 0, g.n_angles)
    y = poisson_counts(line.cpu().numpy(), cfg.I0, 0)
    return cfg, x.ravel(), y, np.full_like(y, cfg.I0)


@pytest.mark.parametrize("name", ["clinical", "fullres"])
def test_one_iteration_matches_fp64_oracle(mod, name):
    from oracle.oracle import Oracle

    cfg, _, y, b = scan(mod, name)
    kw = dict(subset_num=cfg.subset_num, iter_num=1, beta=cfg.beta, delta=cfg.delta,
              potential=cfg.potential)
    xg = mod.reconstruct(cfg.geom, y, b, angles=cfg.angles, **kw)
    xg = xg.cpu().numpy() if isinstance(xg, torch.Tensor) else np.asarray(xg)
    xo = Oracle(np.float64).reconstruct(cfg.geom, cfg.angles, y, b, **kw)
    diff = xg.astype(np.float64) - xo
    rmse = np.sqrt(np.mean(diff ** 2))
    rel = rmse / np.sqrt(np.mean(xo ** 2))
    print(f"{name} 1 x {cfg.subset_num}: rel RMSE {rel:.2e}  RMSE {rmse:.2e}/mm  "
          f"max-abs {np.abs(diff).max():.2e}/mm")
    assert np.isfinite(xg).all() and (xg >= 0).all()
    assert rel <= REL_RMSE_BAR


@pytest.mark.parametrize("name", ["clinical", "fullres"])
def test_projector_is_linear_at_full_size(mod, name):
    from newrecon_gb300.geometry import config

    cfg = config(name, seed=0)
    g = cfg.geom
    mod.set_geometry(g)
    gen = torch.Generator(device="cuda").manual_seed(3)
    x1 = torch.rand(g.n_voxels, device="cuda", generator=gen) * 0.05
    x2 = torch.rand(g.n_voxels, device="cuda", generator=gen) * 0.05
    ang = torch.from_numpy(cfg.angles).cuda()
    idx = torch.arange(g.n_angles, dtype=torch.int32, device="cuda")
    a0, a1 = 0, min(3, g.n_angles)

    def fp(x):
        out = torch.zeros(g.n_angles * g.n_bins, device="cuda")
        mod.fprojectCB_1R_GPU_OSTR_cos(x, out, ang, idx, a0, a1)
        return out.double()

    lhs = fp(2.5 * x1 + x2)
    rhs = 2.5 * fp(x1) + fp(x2)
    rel = (lhs - rhs).norm() / rhs.norm()
    assert rel < 1e-6, float(rel)
