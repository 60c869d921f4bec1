"""CUDA-graph replay of the subset loop and the batched persistent path, against
the single-reconstruction path (same tile code, so results agree to float
rounding of possibly different instruction scheduling; in practice exactly)."""
import numpy as np
import pytest
import torch

from conftest import golden
from test_oracle_golden import geom_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mod():
    from newrecon_gb300 import native, ostr

    native.load()
    return ostr


def close(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) <= 1e-6 * max(np.linalg.norm(b), 1e-30) and \
        np.abs(a - b).max() <= 1e-5 * max(np.abs(b).max(), 1e-30)


def small_scan():
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts
    from oracle.oracle import Oracle

    cfg = config("small")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    idx = np.arange(g.n_angles, dtype=np.int32)
    y = poisson_counts(Oracle(np.float64).fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles),
                       cfg.I0, 0)
    return cfg, y, np.full_like(y, cfg.I0)


def test_graph_replay_matches_iterate(mod):
    cfg, y, b = small_scan()
    plan = mod.OSTR(cfg.geom, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                    potential=cfg.potential)
    plan.setup(cfg.angles, y, b)
    x1 = torch.zeros(cfg.geom.n_voxels, device="cuda")
    x2 = torch.zeros(cfg.geom.n_voxels, device="cuda")
    gr = plan.graph(x2, 2)
    plan.iterate(x1, 2)
    gr.launch()
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)
    plan.iterate(x1, 2)
    gr.launch()  # replays continue from the current x
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)
    gr.close()


def test_graph_with_odd_subiteration_count(mod):
    z = golden("tiny")
    g = geom_of(z)
    plan = mod.OSTR(g, subset_num=3, beta=float(z["beta"]), delta=float(z["delta"]),
                    potential="lange")
    plan.setup(z["angles"], z["y"], z["b"])
    x1 = torch.zeros(g.n_voxels, device="cuda")
    x2 = torch.zeros(g.n_voxels, device="cuda")
    gr = plan.graph(x2, 1)  # 3 sub-iterations: ends in the ping-pong buffer, copied back
    plan.iterate(x1, 1)
    gr.launch()
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)
    gr.close()


def batch_cases():
    cfg, y, b = small_scan()
    zt, zr = golden("tiny"), golden("ragged")
    return [
        dict(geom=cfg.geom, angles=cfg.angles, prj=y, blank=b, subset_num=cfg.subset_num,
             iter_num=2, beta=cfg.beta, delta=cfg.delta, potential="hyperbola"),
        dict(geom=geom_of(zt), angles=zt["angles"], prj=zt["y"], blank=zt["b"], subset_num=3,
             iter_num=1, beta=float(zt["beta"]), delta=float(zt["delta"]), potential="lange"),
        dict(geom=geom_of(zr), angles=zr["angles"], prj=zr["y"], blank=zr["b"], scat=zr["s"],
             subset_num=2, iter_num=3, beta=float(zr["beta"]), delta=float(zr["delta"]),
             potential="huber"),
        dict(geom=geom_of(zt), angles=zt["angles"], prj=zt["y"], blank=zt["b"], subset_num=6,
             iter_num=2, beta=float(zt["beta"]), delta=float(zt["delta"]), potential="q2"),
    ]


def single(mod, c):
    return mod.reconstruct(c["geom"], c["prj"], c["blank"], c.get("scat"), angles=c["angles"],
                           subset_num=c["subset_num"], iter_num=c["iter_num"], beta=c["beta"],
                           delta=c["delta"], potential=c["potential"])


def test_batch_matches_single_reconstructions(mod):
    cases = batch_cases()
    bt = mod.Batch(cases)
    assert bt.n_steps == max(c["iter_num"] * c["subset_num"] for c in cases)
    out = [x.cpu().numpy() for x in bt.run()]
    for c, xb in zip(cases, out):
        xs = single(mod, c)
        assert close(xb, xs), c["potential"]


def test_batch_slab_depths_match_single(mod):
    """Cases walked with different slab depths share the launches (one update
    class per depth) and compute what the single-case path does."""
    cases = batch_cases()
    for c, zc in zip(cases, (8, 32, 16, 32)):
        c["upd_planes"] = zc
    out = [x.cpu().numpy() for x in mod.Batch(cases).run()]
    for c, xb in zip(cases, out):
        assert close(xb, single(mod, c)), (c["potential"], c["upd_planes"])


def test_batch_two_voxel_tile_is_bit_identical(mod):
    """One-view cases on the two-voxel update tile (their own update class)
    give the one-voxel tile's volumes bit for bit; many-view cases keep the
    one-voxel tile."""
    cases = batch_cases()
    for c in cases:
        c["subset_num"] = c["geom"].n_angles  # one view per subset
    cases[3]["subset_num"] = 3                 # except one case
    ref = [x.clone() for x in mod.Batch(cases).run()]
    for k, c in enumerate(cases):
        c["upd_tile"] = 1
        c["upd_planes"] = (8, 16, 32)[k % 3]
    out = mod.Batch(cases).run()
    for a, b in zip(ref, out):
        assert torch.equal(a, b)


def test_batch_graph_matches_run(mod):
    cases = batch_cases()
    b1 = mod.Batch(cases)
    r1 = [x.clone() for x in b1.run()]
    b2 = mod.Batch(cases)
    gr = b2.graph()
    gr.launch()
    torch.cuda.synchronize()
    b2.check()
    for x1, x2 in zip(r1, b2.x):
        assert torch.equal(x1, x2)
    gr.close()


def test_partial_batch_graph_matches_steps(mod):
    """A graph of the first k steps (and the finish) runs what k step calls
    and the finish run, from the same volumes."""
    import ctypes

    from newrecon_gb300 import native

    cases = batch_cases()
    k = 5
    b1 = mod.Batch(cases)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for step in range(k):
        native.call("nr_batch_step", b1._table_ptr(), step, stream)
    native.call("nr_batch_finish", b1._table_ptr(), stream)
    b2 = mod.Batch(cases)
    gr = b2.graph(k)
    gr.launch()
    torch.cuda.synchronize()
    for x1, x2 in zip(b1.x, b2.x):
        assert torch.equal(x1, x2)
    gr.close()


def test_autotune_variants_agree_and_cache(mod, tmp_path, monkeypatch):
    """Every kernel variant computes the same sub-iteration; the tuner caches."""
    import json

    from newrecon_gb300 import autotune

    monkeypatch.setenv("NR_TUNE_CACHE", str(tmp_path / "tune.json"))
    cfg, y, b = small_scan()
    plan = mod.OSTR(cfg.geom, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                    potential=cfg.potential)
    plan.setup(cfg.angles, y, b)
    x = torch.zeros(cfg.geom.n_voxels, device="cuda")
    plan.iterate(x, 1)
    outs = []
    for k, st in autotune.FP_VARIANTS:
        for zc in autotune.UPD_PLANES:
            for t in autotune.UPD_TILES:
                plan.params.fp_batch, plan.params.fp_stage = k, st
                plan.params.upd_planes, plan.params.upd_tile = zc, t
                xo = torch.empty_like(x)
                plan.project(x, 3)
                plan.update(x, xo, 3)
                outs.append(xo)
    torch.cuda.synchronize()
    for o in outs[1:]:
        assert torch.equal(o, outs[0])
    rec = plan.autotune(x)
    assert plan.params.fp_batch in autotune.FP_BATCHES
    assert plan.params.upd_planes in autotune.UPD_PLANES
    data = json.load(open(tmp_path / "tune.json"))
    assert autotune.signature(plan) in data
    plan.params.fp_batch = plan.params.upd_planes = 0
    rec2 = plan.autotune(x)  # served from the cache
    assert (plan.params.fp_batch, plan.params.upd_planes) == (rec["fp_batch"], rec["upd_planes"])
    assert plan.params.fp_stage == rec["fp_stage"]
    assert plan.params.upd_tile == rec["upd_tile"] in autotune.UPD_TILES
    assert len(rec["update_ms"]) == len(autotune.UPD_PLANES) * len(autotune.UPD_TILES)


def test_sequential_mode_matches_shared_launches(mod):
    """mode="sequential" (each case through its own loop, and its whole-run
    graph: each case's loop as its own graph) gives the shared launches'
    volumes bit for bit."""
    cases = batch_cases()
    ref = [x.clone() for x in mod.Batch(cases, mode="shared").run()]
    bs = mod.Batch(cases, mode="sequential")
    assert bs.mode == "sequential"
    out = bs.run()
    for a, b in zip(ref, out):
        assert torch.equal(a, b)
    for x in bs.x:
        x.zero_()
    gr = bs.graph()
    gr.launch()
    torch.cuda.synchronize()
    bs.check()
    gr.close()
    for a, b in zip(ref, bs.x):
        assert torch.equal(a, b)
