"""The alternative update tiles against the one-voxel tile: the two-voxel tile
(upd_tile = 1) and the TMA-fed ring (upd_tile = 2, a producer warp streaming
the planes into shared memory, consumer warps synchronised by mbarriers).

Each voxel's sums are formed in the same order and grouping by every tile, so
the bar is bit-identical volumes after whole OSTR iterations, for every
potential, on shapes that leave partly filled tiles, odd column counts (a
thread whose second voxel is outside the volume; a row the TMA form cannot
describe, where it falls back to the one-voxel tile), a single column, and
slab chunks cut short in z.  The oracle parity of the one-voxel tile is
covered by test_gpu_recon.py.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [(203, 77, 13), (65, 9, 5), (1, 1, 3), (2, 3, 4), (64, 8, 16), (130, 17, 33),
          (127, 40, 7), (128, 40, 7), (36, 9, 5), (4, 3, 4), (100, 17, 33)]


@pytest.fixture(scope="module")
def mod():
    from newrecon_gb300 import native, ostr

    native.load()
    return ostr


def scan(mod, g, angles, seed, I0=1e4):
    from newrecon_gb300.phantom import poisson_counts

    rng = np.random.default_rng(seed)
    x = (rng.random(g.n_voxels, dtype=np.float32) * 0.05).astype(np.float32)
    mod.set_geometry(g)
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = torch.zeros(g.n_angles * g.n_bins, device="cuda")
    mod.fprojectCB_1R_GPU_OSTR_cos(torch.from_numpy(x).cuda(), line,
                                   torch.from_numpy(angles).cuda(),
                                   torch.from_numpy(idx).cuda(), 0, g.n_angles)
    y = poisson_counts(line.cpu().numpy(), I0, seed)
    return torch.from_numpy(y).cuda(), torch.full((y.size,), I0, device="cuda")


def run(mod, g, angles, y, b, iters, pot, beta, delta, tile, planes=0):
    plan = mod.OSTR(g, subset_num=g.n_angles, beta=beta, delta=delta, potential=pot,
                    upd_tile=tile)
    plan.params.upd_planes = planes
    plan.setup(angles, y, b)
    x = torch.zeros(g.n_voxels, dtype=torch.float32, device="cuda")
    plan.iterate(x, iters)
    assert plan.check() == 0
    return x


@pytest.mark.parametrize("tile", [1, 2])
@pytest.mark.parametrize("shape", SHAPES)
def test_alternative_tile_is_bit_identical(mod, shape, tile):
    from newrecon_gb300.geometry import Geometry, view_angles

    nx, ny, nz = shape
    g = Geometry.dbt(nx, ny, nz, 0.5, 1.0, max(8, nx + 10), max(8, ny + 6), 0.5, 6)
    angles = view_angles(6, 15.0)
    y, b = scan(mod, g, angles, nx * 7 + ny)
    for pot in ("q2", "lange", "hyperbola", "huber"):
        for planes in (8, 16, 32):
            a = run(mod, g, angles, y, b, 2, pot, 20.0, 0.01, 0, planes)
            c = run(mod, g, angles, y, b, 2, pot, 20.0, 0.01, tile, planes)
            assert torch.isfinite(a).all()
            assert torch.equal(a, c), (shape, pot, planes, float((a - c).abs().max()))


@pytest.mark.parametrize("tile", [1, 2])
def test_alternative_tile_clinical(mod, tile):
    """One iteration (25 sub-iterations) of the clinical workload, both tiles."""
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts

    cfg = config("clinical")
    g = cfg.geom
    x = breast_phantom(g, 1, cfg.n_glandular, cfg.n_calc, thickness_mm=cfg.thickness_mm)
    mod.set_geometry(g)
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = torch.zeros(g.n_angles * g.n_bins, device="cuda")
    mod.fprojectCB_1R_GPU_OSTR_cos(torch.from_numpy(x.ravel()).cuda(), line,
                                   torch.from_numpy(cfg.angles).cuda(),
                                   torch.from_numpy(idx).cuda(), 0, g.n_angles)
    y = torch.from_numpy(poisson_counts(line.cpu().numpy(), cfg.I0, 1)).cuda()
    b = torch.full_like(y, cfg.I0)
    a = run(mod, g, cfg.angles, y, b, 1, cfg.potential, cfg.beta, cfg.delta, 0)
    c = run(mod, g, cfg.angles, y, b, 1, cfg.potential, cfg.beta, cfg.delta, tile)
    assert torch.equal(a, c)
    assert float(a.abs().max()) > 0


@pytest.mark.parametrize("nx", [70, 72])
def test_many_view_subsets(mod, nx):
    """With several views per subset the two-voxel tile falls back to the
    one-voxel tile, and the TMA-fed ring runs its view loop (nx = 72) or
    falls back too (nx = 70: rows of 280 bytes cannot be described)."""
    from newrecon_gb300.geometry import Geometry, view_angles

    g = Geometry.dbt(nx, 20, 9, 0.5, 1.0, 80, 26, 0.5, 6)
    angles = view_angles(6, 15.0)
    y, b = scan(mod, g, angles, 5)
    out = []
    for tile in (0, 1, 2):
        plan = mod.OSTR(g, subset_num=3, beta=20.0, delta=0.01, potential="huber", upd_tile=tile)
        plan.setup(angles, y, b)
        x = torch.zeros(g.n_voxels, dtype=torch.float32, device="cuda")
        plan.iterate(x, 2)
        out.append(x)
    assert torch.equal(out[0], out[1]) and torch.equal(out[0], out[2])


def test_reconstruct_applies_the_cached_choice(mod, tmp_path, monkeypatch):
    """reconstruct(tune="cached") runs the autotuner's cached variants for the
    geometry; the result is the defaults' result bit for bit."""
    import json

    from newrecon_gb300 import autotune
    from newrecon_gb300.geometry import Geometry, view_angles

    cache = tmp_path / "tune.json"
    monkeypatch.setenv("NR_TUNE_CACHE", str(cache))
    g = Geometry.dbt(130, 17, 33, 0.5, 1.0, 140, 23, 0.5, 6)
    angles = view_angles(6, 15.0)
    y, b = scan(mod, g, angles, 11)
    kw = dict(angles=angles, subset_num=6, iter_num=2, beta=20.0, delta=0.01, potential="huber")
    plain = mod.reconstruct(g, y, b, tune=False, **kw)
    plan = mod.OSTR(g, subset_num=6, beta=20.0, delta=0.01, potential="huber")
    assert autotune.apply_cached(plan) is None            # nothing cached yet
    tuned = mod.reconstruct(g, y, b, tune=True, **kw)     # tunes and caches
    rec = autotune.apply_cached(plan)
    assert rec is not None
    assert (plan.params.upd_tile, plan.params.upd_planes) == (rec["upd_tile"], rec["upd_planes"])
    cached = mod.reconstruct(g, y, b, **kw)
    assert torch.equal(plain, tuned) and torch.equal(plain, cached)
    # a cached entry that names no variant is ignored
    cache.write_text(json.dumps({autotune.signature(plan): {"fp_batch": 3, "upd_planes": 16}}))
    assert autotune.apply_cached(mod.OSTR(g, subset_num=6, beta=20.0, delta=0.01,
                                          potential="huber")) is None
    with pytest.raises(ValueError):
        mod.reconstruct(g, y, b, tune="always", **kw)


@pytest.mark.parametrize("tile", [0, 1, 2])
def test_nonfinite_input_is_reported_by_every_tile(mod, tile):
    """A NaN count reaches the update through h; every tile flags the
    non-finite voxels it produces (one-view subsets, so the tile applies;
    the tiny volume's 40 columns allow the TMA form)."""
    from conftest import golden
    from test_oracle_golden import geom_of

    from newrecon_gb300.native import NrError

    z = golden("tiny")
    g = geom_of(z)
    y = z["y"].copy()
    y[(g.nbx // 2) * g.nby + g.nby // 2] = np.nan
    plan = mod.OSTR(g, subset_num=g.n_angles, beta=1.0, delta=0.01, potential="huber",
                    upd_tile=tile)
    plan.setup(z["angles"], y, z["b"])
    xt = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(xt, 1)
    with pytest.raises(NrError) as e:
        plan.check()
    assert e.value.code == 4
    assert plan.check() == 0
