"""The SART / OS-SART family on the GPU against the FP64 oracle and the
fixtures made by the reference's own SART kernels.

Operators through the drop-in names (newrecon_gb300.sart), with the
projector / back projector tolerances of the OSTR operators (the same walk
and the same interpolation; see test_gpu_ops): relative RMSE 5e-6 / 5e-5 and
max 1e-4 / 2e-4 of scale; the projection difference is bit-exact.  The fused
OS-SART loop is held to the OSTR loop's bar, relative RMSE 1e-4.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden
from test_gpu_ops import CASES, RMSE_BP, RMSE_FP, TOL, dev, maxrel, relrmse
from test_oracle_golden import geom_of

pytestmark = pytest.mark.gpu

LOOP_BAR = 1e-4


@pytest.fixture(scope="module")
def sart():
    from newrecon_gb300 import native, sart as mod

    native.load()
    return mod


def _subsets(name, A):
    return A if name == "small" else 2 if name == "ragged" else 3


@pytest.mark.parametrize("use_cos", [False, True], ids=["plain", "cos"])
@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_fp_sart(sart, name, g, angles, x, use_cos):
    from newrecon_gb300 import ostr
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    A = g.n_angles
    M = _subsets(name, A)
    ridx = Oracle(np.float64).reorder_index(A, M)
    Vs = A // M
    fn = sart.fprojectCB_1R_GPU_SART_cos if use_cos else sart.fprojectCB_1R_GPU_SART
    for idx, a0, a1 in ((np.arange(A, dtype=np.int32), 0, A), (ridx, Vs, 2 * Vs)):
        s = -7.0
        n = (a1 - a0) * g.n_bins
        re, rn = Oracle(np.float64).fp_sart(g, x, angles, idx, a0, a1, use_cos,
                                            est=np.full(n, s), norm=np.full(n, s))
        est = torch.full((n,), s, device="cuda")
        norm = torch.full((n,), s, device="cuda")
        fn(dev(x), est, norm, dev(angles), dev(idx, torch.int32), a0, a1)
        ge, gn = est.cpu().numpy(), norm.cpu().numpy()
        miss = rn == s
        assert np.array_equal(gn == s, miss) and np.array_equal(ge == s, miss)
        print(f"{name} fp_sart cos={use_cos}: est {relrmse(ge[~miss], re[~miss]):.2e} "
              f"norm {relrmse(gn[~miss], rn[~miss]):.2e}")
        assert relrmse(ge[~miss], re[~miss]) < RMSE_FP
        assert maxrel(ge[~miss], re[~miss]) < TOL
        assert relrmse(gn[~miss], rn[~miss]) < RMSE_FP
        assert maxrel(gn[~miss], rn[~miss]) < TOL


@pytest.mark.parametrize("cos,layout", [(False, "ji"), (True, "ij")])
@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_fp_4r(sart, name, g, angles, x, cos, layout):
    from newrecon_gb300 import ostr
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    A = g.n_angles
    M = _subsets(name, A)
    ridx = Oracle(np.float64).reorder_index(A, M)
    Vs = A // M
    for idx, a0, a1 in ((np.arange(A, dtype=np.int32), 0, A), (ridx, Vs, 2 * Vs)):
        s = -7.0
        rsub = np.full(4 * (a1 - a0) * g.n_bins, s)
        ref = Oracle(np.float64).fp_4r(g, x, angles, idx, a0, a1, cos, layout, sub=rsub)
        out = torch.full(((a1 - a0) * g.n_bins,), s, device="cuda")
        if not cos and layout == "ji":
            sub = torch.full((4 * (a1 - a0) * g.n_bins,), s, device="cuda")
            sart.fprojectCB1_4R_GPU_SART(dev(x), out, sub, dev(angles), dev(idx, torch.int32),
                                         a0, a1)
            gs = sub.cpu().numpy()
            miss = rsub == s
            assert np.array_equal(gs == s, miss)
            assert relrmse(gs[~miss], rsub[~miss]) < RMSE_FP
            assert maxrel(gs[~miss], rsub[~miss]) < TOL
        else:
            sart.fproject_4R(dev(x), out, dev(angles), dev(idx, torch.int32), a0, a1, cos, layout)
        got = out.cpu().numpy()
        assert not (got == s).any()  # every bin is written
        print(f"{name} fp_4r cos={cos} {layout}: rel RMSE {relrmse(got, ref):.2e} "
              f"max {maxrel(got, ref):.2e}")
        assert relrmse(got, ref) < RMSE_FP
        assert maxrel(got, ref) < TOL


def test_fp_4r_matches_reference_fixture(sart):
    from newrecon_gb300 import ostr

    for name in ("tiny", "ragged"):
        z = golden(f"sart_{name}")
        g = geom_of(z)
        ostr.set_geometry(g)
        A = g.n_angles
        idx = dev(np.arange(A, dtype=np.int32), torch.int32)
        out = torch.zeros(A * g.n_bins, device="cuda")
        sub = torch.zeros(4 * A * g.n_bins, device="cuda")
        sart.fprojectCB1_4R_GPU_SART(dev(z["x"]), out, sub, dev(z["angles"]), idx, 0, A)
        assert maxrel(sub.cpu().numpy(), z["fp4r_sub"]) < TOL
        assert maxrel(out.cpu().numpy(), z["fp4r_merged_ji"]) < TOL


@pytest.mark.parametrize("name", ["tiny", "ragged"])
def test_prj_diff_bitexact(sart, name):
    from newrecon_gb300 import ostr

    z = golden(f"sart_{name}")
    g = geom_of(z)
    ostr.set_geometry(g)
    A, M = g.n_angles, int(z["subset_num"])
    Vs = A // M
    from oracle.oracle import Oracle

    ridx = Oracle().reorder_index(A, M)
    p = z["line"].reshape(A, -1)[ridx[Vs:2 * Vs]].ravel()
    out = torch.full((Vs * g.n_bins,), 5.0, device="cuda")
    sart.SART_prj_diff(out, dev(p), dev(z["fpc_sub1_est"]), dev(z["fpc_sub1_norm"]),
                       dev(ridx, torch.int32), Vs, 2 * Vs)
    assert np.array_equal(out.cpu().numpy(), z["diff_sub1"])


@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_prior_sart_accumulates(sart, name, g, angles, x):
    from newrecon_gb300 import ostr
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    rng = np.random.default_rng(8)
    xn = (x + rng.normal(scale=0.004, size=x.size)).astype(np.float32)
    base = rng.normal(size=g.n_voxels)
    ref = Oracle(np.float64).prior_sart(g, xn, 0.003, prior=base.copy())
    pr = dev(base)
    sart.prior_GPU_SART(pr, dev(xn), 0.003)
    got = pr.cpu().numpy() - base.astype(np.float32)
    assert relrmse(got, ref - base) < 1e-5
    assert maxrel(got, ref - base) < 1e-4
    with pytest.raises(ValueError):
        sart.prior_GPU_SART(pr, dev(xn), 0.0)


def test_prior_sart_matches_reference_fixture(sart):
    from newrecon_gb300 import ostr

    for name in ("tiny", "ragged"):
        z = golden(f"sart_{name}")
        g = geom_of(z)
        ostr.set_geometry(g)
        pr = torch.zeros(g.n_voxels, device="cuda")
        sart.prior_GPU_SART(pr, dev(z["x"]), float(z["delta"]))
        assert maxrel(pr.cpu().numpy(), z["prior"]) < TOL


@pytest.mark.parametrize("reg", [False, True], ids=["plain", "reg"])
@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_bp_ossart(sart, name, g, angles, x, reg):
    from newrecon_gb300 import ostr
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    A = g.n_angles
    M = _subsets(name, A)
    Vs = A // M
    ridx = Oracle(np.float64).reorder_index(A, M)
    rng = np.random.default_rng(9)
    diff = (rng.normal(size=Vs * g.n_bins) * 0.01).astype(np.float32)
    prior = Oracle(np.float32).prior_sart(g, x, 0.01) if reg else None
    ref = Oracle(np.float64).bp_ossart(g, x, diff, ridx, angles, Vs, 2 * Vs, 0.7, prior, -0.3)
    xd = dev(x)
    if reg:
        sart.bprojectCB_4B_GPU_SART_R(xd, dev(diff), dev(prior), dev(ridx, torch.int32),
                                      dev(angles), Vs, 2 * Vs, 0.7, -0.3)
    else:
        sart.bprojectCB_4B_GPU_SART(xd, dev(diff), dev(ridx, torch.int32), dev(angles), Vs,
                                    2 * Vs, 0.7)
    got = xd.cpu().numpy()
    print(f"{name} bp_ossart reg={reg}: rel RMSE {relrmse(got, ref):.2e} "
          f"max {maxrel(got, ref):.2e}")
    assert relrmse(got, ref) < RMSE_BP
    assert maxrel(got, ref) < 2 * TOL
    assert (got >= 0).all()


def test_bp_ossart_matches_reference_fixture(sart):
    from newrecon_gb300 import ostr
    from oracle.oracle import Oracle

    for name in ("tiny", "ragged"):
        z = golden(f"sart_{name}")
        g = geom_of(z)
        ostr.set_geometry(g)
        A, M = g.n_angles, int(z["subset_num"])
        Vs = A // M
        ridx = dev(Oracle().reorder_index(A, M), torch.int32)
        for key, prior in (("bp_plain", None), ("bp_reg", z["prior"])):
            xd = dev(z["x"])
            if prior is None:
                sart.bprojectCB_4B_GPU_SART(xd, dev(z["bp_in"]), ridx, dev(z["angles"]), Vs,
                                            2 * Vs, float(z["lam"]))
            else:
                sart.bprojectCB_4B_GPU_SART_R(xd, dev(z["bp_in"]), dev(prior), ridx,
                                              dev(z["angles"]), Vs, 2 * Vs, float(z["lam"]),
                                              float(z["beta"]))
            assert maxrel(xd.cpu().numpy(), z[key]) < 2 * TOL, (name, key)


def test_line_integrals(sart):
    from oracle.oracle import Oracle

    z = golden("ragged")
    got = sart.line_integrals(z["y"], z["b"], z["s"])
    ref = Oracle(np.float64).line_integrals(z["y"], z["b"], z["s"])
    assert np.array_equal(got == 0, ref == 0)
    assert maxrel(got, ref) < 1e-6


def _small_line():
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts
    from oracle.oracle import Oracle

    cfg = config("small")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    idx = np.arange(g.n_angles, dtype=np.int32)
    y = poisson_counts(Oracle(np.float64).fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles), cfg.I0, 0)
    b = np.full_like(y, cfg.I0)
    line = Oracle(np.float64).line_integrals(y, b).astype(np.float32)
    return g, cfg.angles, line, 3


VARIANTS = {
    "cos": dict(use_cos=True),
    "plain": dict(use_cos=False),
    "reg": dict(use_cos=True, regularized=True, beta=-0.2, delta=0.01),
    "4r": dict(use_cos=True, supersample=True),
}


@pytest.mark.parametrize("variant", list(VARIANTS))
@pytest.mark.parametrize("name", ["tiny", "ragged", "small"])
def test_fused_ossart_matches_oracle(sart, name, variant):
    from oracle.oracle import Oracle

    if name == "small":
        g, angles, line, M = _small_line()
        iters, lam = 2, 0.8
    else:
        z = golden(f"sart_{name}")
        g, angles, line, M = geom_of(z), z["angles"], z["line"], int(z["subset_num"])
        iters, lam = int(z["iters"]), float(z["lam"])
    kw = dict(subset_num=M, iter_num=iters, lam=lam, **VARIANTS[variant])
    xg = sart.ossart_reconstruct(g, line, angles=angles, **kw)
    xo = Oracle(np.float64).ossart(g, angles, line, **kw)
    r = relrmse(xg, xo)
    print(f"{name}/{variant}: fused OS-SART vs FP64 oracle rel RMSE {r:.2e}")
    assert r < LOOP_BAR
    assert (xg >= 0).all()


@pytest.mark.parametrize("name", ["tiny", "ragged"])
def test_fused_ossart_matches_reference_fixture(sart, name):
    z = golden(f"sart_{name}")
    g = geom_of(z)
    base = dict(subset_num=int(z["subset_num"]), iter_num=int(z["iters"]), lam=float(z["lam"]))
    for key, kw in (("ossart", dict(use_cos=True)), ("ossart_nocos", dict(use_cos=False)),
                    ("ossart_reg", dict(use_cos=True, regularized=True, beta=float(z["beta"]),
                                        delta=float(z["delta"])))):
        xg = sart.ossart_reconstruct(g, z["line"], angles=z["angles"], **base, **kw)
        r = relrmse(xg, z[key])
        print(f"{name}/{key}: fused vs reference kernels rel RMSE {r:.2e}")
        assert r < LOOP_BAR


def test_workspace_sections(sart):
    from oracle.oracle import Oracle

    z = golden("sart_ragged")
    g = geom_of(z)
    M = int(z["subset_num"])
    plan = sart.OSSART(g, subset_num=M, lam=0.5)
    plan.setup(z["angles"], z["line"])
    A = g.n_angles
    ridx = Oracle().reorder_index(A, M)
    assert np.array_equal(plan.section("index").cpu().numpy(), ridx)
    # line: [view][j][i] in subset order
    want = z["line"].reshape(A, g.nbx, g.nby)[ridx].transpose(0, 2, 1).ravel()
    assert np.array_equal(plan.section("line").cpu().numpy(), want)
    chord = Oracle(np.float64).fp_gamma(g, z["angles"], ridx, 0, A, "chord")
    chord = np.where(chord > 0, chord, 0).reshape(A, g.nbx, g.nby).transpose(0, 2, 1).ravel()
    got = plan.section("norm").cpu().numpy()
    assert np.array_equal(got == 0, chord == 0)
    assert maxrel(got, chord) < TOL


def test_graph_and_subiter_match_iterate(sart):
    z = golden("sart_tiny")
    g = geom_of(z)
    M = int(z["subset_num"])
    plan = sart.OSSART(g, subset_num=M, lam=0.8, regularized=True, beta=-0.2, delta=0.01)
    plan.setup(z["angles"], z["line"])
    x1 = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x1, 2)
    x2 = torch.zeros(g.n_voxels, device="cuda")
    for _ in range(2):
        for a in range(M):
            plan.subiter(x2, a)
    x3 = torch.zeros(g.n_voxels, device="cuda")
    gr = plan.graph(x3, 1)
    gr.launch()
    gr.launch()
    torch.cuda.synchronize()
    gr.close()
    x4 = torch.zeros(g.n_voxels, device="cuda")
    x5 = torch.empty_like(x4)
    for _ in range(2):
        for a in range(M):
            plan.project(x4, a)
            plan.update(x4, x5, a)
            x4, x5 = x5, x4
    assert plan.check() == 0
    assert torch.equal(x1, x2)
    assert torch.equal(x1, x3)
    assert torch.equal(x1, x4)


def test_bad_parameters_and_nonfinite(sart):
    from newrecon_gb300 import native
    from newrecon_gb300.geometry import NrSartParams
    from newrecon_gb300.native import NrError

    z = golden("sart_tiny")
    g = geom_of(z)
    gc = g.to_c()
    size = ctypes.c_size_t(0)
    bad = [NrSartParams(3, 1, 1, 0, 0, 0.8, -0.2, 0.0),     # regularised, delta 0
           NrSartParams(3, 1, 0, 3, 0, 0.8, 0.0, 1.0),      # fp_batch 3
           NrSartParams(3, 1, 0, 0, 12, 0.8, 0.0, 1.0),     # upd_planes 12
           NrSartParams(3, 1, 0, 0, 0, float("nan"), 0.0, 1.0)]
    for p in bad:
        with pytest.raises(NrError) as e:
            native.call("nr_sart_workspace_size", ctypes.byref(gc), ctypes.byref(p),
                        ctypes.byref(size))
        assert e.value.code == 2
    with pytest.raises(NrError) as e:
        native.call("nr_sart_workspace_size", ctypes.byref(gc),
                    ctypes.byref(NrSartParams(4, 1, 0, 0, 0, 0.8, 0.0, 1.0)), ctypes.byref(size))
    assert e.value.code == 1  # 4 subsets of 6 views
    # a NaN in a measured bin reaches the volume and trips the status word
    line = z["line"].copy().reshape(g.n_angles, g.nbx, g.nby)
    line[0, g.nbx // 2, g.nby // 2] = np.nan
    plan = sart.OSSART(g, subset_num=3, lam=0.8)
    plan.setup(z["angles"], line.ravel())
    x = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x, 1)
    with pytest.raises(NrError) as e:
        plan.check()
    assert e.value.code == 4
    assert plan.check() == 0  # cleared
