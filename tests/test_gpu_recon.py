"""The device-resident OSTR path (fused kernels) against the FP64 oracle.

Bar: the plain GPU path matches the FP64 oracle (the reference's gold
algorithm run in double on the same inputs) within 1e-4 relative RMSE of the
volume after the same iterations; RMSE and max-abs (1/mm) are printed.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from test_oracle_golden import geom_of

pytestmark = pytest.mark.gpu

REL_RMSE_BAR = 1e-4


def stats(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    rmse = np.sqrt(np.mean((a - b) ** 2))
    return rmse / np.sqrt(np.mean(b ** 2)), rmse, np.abs(a - b).max()


@pytest.fixture(scope="module")
def mod():
    from newrecon_gb300 import native, ostr

    native.load()
    return ostr


@pytest.mark.parametrize("pot", ["lange", "q2", "hyperbola", "huber"])
@pytest.mark.parametrize("name", ["tiny", "ragged"])
def test_fused_vs_oracle(mod, name, pot):
    from oracle.oracle import Oracle

    z = golden(name)
    g = geom_of(z)
    kw = dict(subset_num=int(z["subset_num"]), iter_num=int(z["iters"]) + 1,
              beta=float(z["beta"]), delta=float(z["delta"]), potential=pot)
    scat = z["s"] if name == "ragged" else None
    xg = mod.reconstruct(g, z["y"], z["b"], scat, angles=z["angles"], **kw)
    xo = Oracle(np.float64).reconstruct(g, z["angles"], z["y"], z["b"], scat, **kw)
    rel, rmse, mx = stats(xg, xo)
    print(f"{name}/{pot}: rel RMSE {rel:.2e}  RMSE {rmse:.2e}/mm  max-abs {mx:.2e}/mm")
    assert rel < REL_RMSE_BAR
    assert (xg >= 0).all()


def test_fused_matches_gold_driver_fixture(mod):
    """Lange/Q2 reconstructions against the reference's own gold driver output."""
    for name in ("tiny", "ragged"):
        z = golden(name)
        g = geom_of(z)
        scat = z["s"] if name == "ragged" else None
        for pot, key in (("lange", "recon_lange"), ("q2", "recon_q2")):
            xg = mod.reconstruct(g, z["y"], z["b"], scat, angles=z["angles"],
                                 subset_num=int(z["subset_num"]), iter_num=int(z["iters"]),
                                 beta=float(z["beta"]), delta=float(z["delta"]), potential=pot)
            rel, rmse, mx = stats(xg, z[key])
            print(f"{name}/{pot} vs gold driver: rel RMSE {rel:.2e}")
            assert rel < REL_RMSE_BAR


@pytest.fixture(scope="module")
def small_case():
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts
    from oracle.oracle import Oracle

    cfg = config("small")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    idx = np.arange(g.n_angles, dtype=np.int32)
    y = poisson_counts(Oracle(np.float64).fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles),
                       cfg.I0, 0)
    b = np.full_like(y, cfg.I0)
    return cfg, x, y, b


def test_small_workload_full_run(mod, small_case):
    """256x128x24, 9 views, 10 iterations x 9 subsets, hyperbola: the whole run."""
    from oracle.oracle import Oracle

    cfg, x, y, b = small_case
    kw = dict(subset_num=cfg.subset_num, iter_num=cfg.iter_num, beta=cfg.beta, delta=cfg.delta,
              potential=cfg.potential)
    xg = mod.reconstruct(cfg.geom, y, b, angles=cfg.angles, **kw)
    xo = Oracle(np.float64).reconstruct(cfg.geom, cfg.angles, y, b, **kw)
    rel, rmse, mx = stats(xg, xo)
    print(f"small/hyperbola 10x9: rel RMSE {rel:.2e}  RMSE {rmse:.2e}/mm  max-abs {mx:.2e}/mm")
    assert rel < REL_RMSE_BAR


def test_objective_fp64_matches_oracle(mod, small_case):
    from oracle.oracle import Oracle

    cfg, x, y, b = small_case
    for pot in ("hyperbola", "lange", "huber", "q2"):
        plan = mod.OSTR(cfg.geom, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                        potential=pot)
        plan.setup(cfg.angles, y, b)
        xt = torch.from_numpy(x).cuda()
        d, p = plan.objective(xt)
        do, po = Oracle(np.float64).objective(cfg.geom, cfg.angles, y, b, x, potential=pot,
                                              delta=cfg.delta)
        print(f"{pot}: data rel {abs(d - do) / abs(do):.2e}, penalty rel {abs(p - po) / abs(po):.2e}")
        # the data term's line integrals come from the FP32 projector; the
        # penalty is evaluated in double throughout
        assert abs(d - do) <= 1e-7 * abs(do), (pot, d, do)
        assert abs(p - po) <= 1e-10 * abs(po), (pot, p, po)


def test_objective_decreases(mod, small_case):
    cfg, x, y, b = small_case
    plan = mod.OSTR(cfg.geom, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                    potential=cfg.potential)
    plan.setup(cfg.angles, y, b)
    xt = torch.zeros(cfg.geom.n_voxels, device="cuda")
    vals = [plan.total_objective(xt)]
    for _ in range(4):
        plan.iterate(xt, 1)
        vals.append(plan.total_objective(xt))
    assert all(v1 < v0 for v0, v1 in zip(vals, vals[1:])), vals


def test_deterministic_and_subiter_consistent(mod, small_case):
    cfg, x, y, b = small_case
    plan = mod.OSTR(cfg.geom, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                    potential=cfg.potential)
    plan.setup(cfg.angles, y, b)
    x1 = torch.zeros(cfg.geom.n_voxels, device="cuda")
    x2 = torch.zeros(cfg.geom.n_voxels, device="cuda")
    x3 = torch.zeros(cfg.geom.n_voxels, device="cuda")
    plan.iterate(x1, 2)
    plan.iterate(x2, 2)
    for _ in range(2):
        for a in range(cfg.subset_num):
            plan.subiter(x3, a)
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)
    assert torch.equal(x1, x3)


def test_nonfinite_input_is_reported(mod):
    from newrecon_gb300.native import NrError

    z = golden("tiny")
    g = geom_of(z)
    y = z["y"].copy()
    # a bin in the middle of view 0, seen by the volume's central voxels
    y[(g.nbx // 2) * g.nby + g.nby // 2] = np.nan
    plan = mod.OSTR(g, subset_num=3, beta=1.0, delta=0.01, potential="lange")
    plan.setup(z["angles"], y, z["b"])
    xt = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(xt, 1)
    with pytest.raises(NrError) as e:
        plan.check()
    assert e.value.code == 4
    assert plan.check() == 0  # cleared


def test_workspace_too_small_is_rejected(mod):
    import ctypes

    from newrecon_gb300 import native
    from newrecon_gb300.geometry import NrOstrParams

    z = golden("tiny")
    g = geom_of(z)
    p = NrOstrParams(3, 1, 0, 0, 1.0, 0.01)
    gc = g.to_c()
    buf = torch.empty(1024, dtype=torch.uint8, device="cuda")
    rc = native.load().nr_ostr_iterate(ctypes.byref(gc), ctypes.byref(p),
                                       ctypes.c_void_p(buf.data_ptr()), 1,
                                       ctypes.c_void_p(buf.data_ptr()), ctypes.c_size_t(1024),
                                       ctypes.c_void_p(0))
    assert rc == 6


@pytest.mark.parametrize("cfgname", ["tiny", "small"])
def test_staged_projection_is_bit_identical(mod, cfgname):
    """The projection that stages the volume slab by slab in shared memory (TMA)
    gives the same bits as the one that gathers from global memory, for every
    subset, and so do whole reconstructions."""
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts

    cfg = config(cfgname)
    g = cfg.geom
    assert g.nx % 4 == 0  # the staged path applies
    x = breast_phantom(g, 1, cfg.n_glandular, cfg.n_calc).ravel()
    line = np.zeros(g.n_angles * g.n_bins, np.float32)
    mod.set_geometry(g)
    idx = np.arange(g.n_angles, dtype=np.int32)
    mod.fprojectCB_1R_GPU_OSTR_cos(x, line, cfg.angles, idx, 0, g.n_angles)
    y = poisson_counts(line, cfg.I0, 1)
    b = np.full_like(y, cfg.I0)
    xd = torch.from_numpy(x).cuda()
    hs = []
    for stage in (True, False):
        plan = mod.OSTR(g, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                        potential=cfg.potential, stage=stage)
        plan.setup(cfg.angles, y, b)
        outs = []
        for a in range(cfg.subset_num):
            plan.project(xd, a)
            outs.append(plan.section("h").clone())
        x0 = torch.zeros(g.n_voxels, device="cuda")
        plan.iterate(x0, 2)
        assert plan.check() == 0
        hs.append((torch.stack(outs), x0))
    assert torch.equal(hs[0][0], hs[1][0])
    assert torch.equal(hs[0][1], hs[1][1])


def test_monotone_iterations_accept_only_decreases(mod):
    """monotone=True keeps the FP64 objective non-increasing; while no
    iteration is rejected it computes exactly what plain iterations do."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(subset_num=3, beta=float(z["beta"]), delta=float(z["delta"]), potential="lange")
    plan = mod.OSTR(g, **kw)
    plan.setup(z["angles"], z["y"], z["b"])
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 4, monotone=True)
    h = plan.history
    assert all(b <= a for a, b in zip(h, h[1:]))
    n_ok = len(h) - 1
    ref = mod.OSTR(g, **kw)
    ref.setup(z["angles"], z["y"], z["b"])
    xr = torch.zeros(g.n_voxels, device="cuda")
    ref.iterate(xr, n_ok)
    torch.cuda.synchronize()
    assert torch.equal(x, xr)
    assert plan.rejected_at is None or plan.rejected_at == n_ok


def test_monotone_undoes_a_rising_iteration(mod, monkeypatch):
    """An iteration whose objective rises (planted on the host) is undone and
    the loop stops: x is the iterate before it."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(subset_num=3, beta=float(z["beta"]), delta=float(z["delta"]), potential="lange")
    plan = mod.OSTR(g, **kw)
    plan.setup(z["angles"], z["y"], z["b"])
    values = iter([10.0, 5.0, 7.0, 1.0])
    monkeypatch.setattr(plan, "total_objective", lambda x: next(values))
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 3, monotone=True)
    assert plan.history == [10.0, 5.0] and plan.rejected_at == 1
    ref = mod.OSTR(g, **kw)
    ref.setup(z["angles"], z["y"], z["b"])
    xr = torch.zeros(g.n_voxels, device="cuda")
    ref.iterate(xr, 1)
    torch.cuda.synchronize()
    assert torch.equal(x, xr)


def test_monotone_checkpoints_undo_a_rising_block(mod, monkeypatch):
    """check_every=2: the objective is checked after every second iteration;
    a checkpoint whose objective rises (planted on the host) is undone back to
    the previous checkpoint and the loop stops."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(subset_num=3, beta=float(z["beta"]), delta=float(z["delta"]), potential="lange")
    plan = mod.OSTR(g, **kw)
    plan.setup(z["angles"], z["y"], z["b"])
    values = iter([10.0, 5.0, 7.0, 1.0])
    monkeypatch.setattr(plan, "total_objective", lambda x: next(values))
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 6, monotone=True, check_every=2)
    assert plan.history == [10.0, 5.0] and plan.rejected_at == 2
    ref = mod.OSTR(g, **kw)
    ref.setup(z["angles"], z["y"], z["b"])
    xr = torch.zeros(g.n_voxels, device="cuda")
    ref.iterate(xr, 2)
    torch.cuda.synchronize()
    assert torch.equal(x, xr)
    with pytest.raises(ValueError):
        plan.iterate(x, 1, monotone=True, check_every=0)


def test_subset_data_terms_add_up_to_the_objective(mod, small_case):
    """nr_ostr_project_fp64: the same h as nr_ostr_project, and its per-subset
    FP64 data terms add up to the objective's data term (the same per-bin
    terms, summed in another order); nr_ostr_penalty is the objective's
    penalty bit for bit."""
    cfg, x, y, b = small_case
    plan = mod.OSTR(cfg.geom, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                    potential=cfg.potential)
    plan.setup(cfg.angles, y, b)
    xt = torch.from_numpy(x).cuda()
    total = 0.0
    for a in range(cfg.subset_num):
        plan.project(xt, a)
        h1 = plan.section("h").clone()
        total += float(plan.project_fp64(xt, a).item())
        assert torch.equal(h1, plan.section("h"))
    d, p = plan.objective(xt)
    assert abs(total - d) <= 1e-12 * abs(d), (total, d)
    assert float(plan.penalty(xt).item()) == p


def test_monotone_subset_keeps_only_non_rising_steps(mod):
    """monotone="subset": every kept step lowers (or keeps) the FP64 subset
    objective, every dropped one would have raised it; with nothing dropped
    the volume is the plain iterations' bit for bit."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(subset_num=3, beta=float(z["beta"]), delta=float(z["delta"]), potential="lange")
    plan = mod.OSTR(g, **kw)
    plan.setup(z["angles"], z["y"], z["b"])
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 3, monotone="subset")
    log = plan.subset_history
    assert len(log) == 3 * 3
    assert all((after <= before) == kept for _, _, before, after, kept in log)
    if plan.rejected_steps == 0:
        ref = mod.OSTR(g, **kw)
        ref.setup(z["angles"], z["y"], z["b"])
        xr = torch.zeros(g.n_voxels, device="cuda")
        ref.iterate(xr, 3)
        torch.cuda.synchronize()
        assert torch.equal(x, xr)


def test_monotone_subset_drops_a_rising_step(mod, monkeypatch):
    """A sub-iteration step whose subset objective rises (planted on the
    host) is dropped: x stays, and the loop goes on with the next subset."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(subset_num=3, beta=float(z["beta"]), delta=float(z["delta"]), potential="lange")
    plan = mod.OSTR(g, **kw)
    plan.setup(z["angles"], z["y"], z["b"])
    calls = []

    def planted(before, after):
        calls.append(0)
        return (1.0, 2.0) if len(calls) == 2 else (2.0, 1.0)   # step 2 of 6 rises

    monkeypatch.setattr(plan, "_subset_values", planted)
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 2, monotone="subset")
    assert [e[4] for e in plan.subset_history] == [True, False, True, True, True, True]
    assert plan.rejected_steps == 1
    ref = mod.OSTR(g, **kw)
    ref.setup(z["angles"], z["y"], z["b"])
    xr = torch.zeros(g.n_voxels, device="cuda")
    for k, a in [(0, 0), (0, 2), (1, 0), (1, 1), (1, 2)]:   # subset 1 of iteration 0 dropped
        ref.subiter(xr, a)
    torch.cuda.synchronize()
    assert torch.equal(x, xr)
    with pytest.raises(ValueError):
        plan.iterate(x, 1, monotone="always")


def test_pinned_inputs_return_a_pinned_volume(mod):
    """Host tensors in pinned memory give the volume back in pinned memory (the
    download skips the pageable bounce), equal to the device result."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(angles=z["angles"], subset_num=3, iter_num=2, beta=float(z["beta"]),
              delta=float(z["delta"]), potential="lange")
    y = torch.from_numpy(z["y"]).pin_memory()
    b = torch.from_numpy(z["b"]).pin_memory()
    vol = mod.reconstruct(g, y, b, **kw)
    assert vol.device.type == "cpu" and vol.is_pinned()
    ref = mod.reconstruct(g, y.cuda(), b.cuda(), **kw)
    assert torch.equal(vol, ref.cpu())
    pageable = mod.reconstruct(g, torch.from_numpy(z["y"]), torch.from_numpy(z["b"]), **kw)
    assert not pageable.is_pinned() and torch.equal(pageable, vol)


def test_reconstruct_on_a_side_stream(mod):
    """reconstruct(stream=s) runs on s and gives the current stream's result
    bit for bit, for host and for device inputs."""
    z = golden("tiny")
    g = geom_of(z)
    kw = dict(angles=z["angles"], subset_num=3, iter_num=2, beta=1.0, delta=0.01,
              potential="lange")
    ref = mod.reconstruct(g, z["y"], z["b"], **kw)
    s = torch.cuda.Stream()
    got = mod.reconstruct(g, z["y"], z["b"], stream=s, **kw)
    assert isinstance(got, np.ndarray) and np.array_equal(ref, got)
    yd = torch.from_numpy(z["y"]).cuda()
    bd = torch.from_numpy(z["b"]).cuda()
    torch.cuda.synchronize()  # the inputs are written on the current stream
    dev = mod.reconstruct(g, yd, bd, stream=s, **kw)
    assert dev.is_cuda and np.array_equal(ref, dev.cpu().numpy())
    with pytest.raises(TypeError):
        mod.reconstruct(g, z["y"], z["b"], stream=1, **kw)
