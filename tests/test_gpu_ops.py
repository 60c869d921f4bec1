"""Parity of every C-ABI operator (through the drop-in ostr module) with the
FP64 oracle, on the fixtures' geometries and the 256x128x24 workload.

Tolerances: the kernels compute in float32 (the reference's precision); the
oracle in float64.  Per-operator results must agree to a relative RMSE of
5e-6 (projections) / 5e-5 (back projection), and to a max-abs error of 1e-4
(2e-4 for the back projection) of the output's scale.  The bounds are set by
geometry, not by arithmetic, and the inputs here are the worst case for it
(white-noise volumes and detector data):
* a ray nearly parallel to a voxel plane crosses it a distance L/|d| further
  along per unit of transverse offset, so the ~2e-6 mm rounding of its float
  entry point moves that crossing by up to ~1e-4 mm, ~1e-4 of the line
  integral where the two voxels differ by a calcification's 2/mm;
* the back projection samples the detector at a float position (~3e-5 mm
  rounding, ~1e-4 bin), and white-noise data change by O(1) per bin.
The FP32 reference algorithm has the same sensitivities (its own distance to
the FP64 oracle on these inputs is of the same order).  Integer and
permutation work is bit-exact.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from test_oracle_golden import geom_of

pytestmark = pytest.mark.gpu

TOL = 1e-4
RMSE_FP = 5e-6
RMSE_BP = 5e-5


@pytest.fixture(scope="module")
def ostr():
    from newrecon_gb300 import native, ostr as mod

    native.load()
    return mod


def maxrel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def relrmse(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def dev(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to("cuda", dtype)


def cases():
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom

    out = []
    for name in ("tiny", "ragged"):
        z = golden(name)
        out.append((name, geom_of(z), z["angles"], z["x"]))
    cfg = config("small")
    out.append(("small", cfg.geom, cfg.angles,
                breast_phantom(cfg.geom, 0, cfg.n_glandular, cfg.n_calc).ravel()))
    return out


CASES = cases()


@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_fp_ostr(ostr, name, g, angles, x):
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    A = g.n_angles
    M = A if name == "small" else 2 if name == "ragged" else 3
    ridx = Oracle(np.float64).reorder_index(A, M)
    Vs = A // M
    for idx, a0, a1 in ((np.arange(A, dtype=np.int32), 0, A), (ridx, Vs, 2 * Vs)):
        sentinel = -7.0
        ref = np.full((a1 - a0) * g.n_bins, sentinel)
        Oracle(np.float64).fp_ostr(g, x, angles, idx, a0, a1, out=ref)
        line = torch.full(((a1 - a0) * g.n_bins,), sentinel, device="cuda")
        ostr.fprojectCB_1R_GPU_OSTR_cos(dev(x), line, dev(angles), dev(idx, torch.int32), a0, a1)
        got = line.cpu().numpy()
        miss = ref == sentinel
        assert np.array_equal(got == sentinel, miss), "missed rays must stay untouched"
        print(f"{name} fp: rel RMSE {relrmse(got[~miss], ref[~miss]):.2e} "
              f"max {maxrel(got[~miss], ref[~miss]):.2e}")
        assert relrmse(got[~miss], ref[~miss]) < RMSE_FP
        assert maxrel(got[~miss], ref[~miss]) < TOL


@pytest.mark.parametrize("mode", ["length", "chord"])
@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_fp_gamma(ostr, name, g, angles, x, mode):
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    ostr.gamma_mode = mode
    try:
        A = g.n_angles
        idx = np.arange(A, dtype=np.int32)
        ref = np.full(A * g.n_bins, -1.0)
        Oracle(np.float64).fp_gamma(g, angles, idx, 0, A, mode, out=ref)
        gam = torch.full((A * g.n_bins,), -1.0, device="cuda")
        ostr.fprojectCB_1R_GPU_OSTR_normprj(gam, dev(angles), dev(idx, torch.int32), 0, A)
        got = gam.cpu().numpy()
        assert np.array_equal(got == -1.0, ref == -1.0)
        assert relrmse(got, ref) < RMSE_FP
        assert maxrel(got, ref) < TOL
    finally:
        ostr.gamma_mode = "length"


@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_bp_sbp_accumulates(ostr, name, g, angles, x):
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    A = g.n_angles
    rng = np.random.default_rng(5)
    h = rng.normal(size=A * g.n_bins).astype(np.float32)
    base = rng.normal(size=g.n_voxels).astype(np.float32)
    idx = np.arange(A, dtype=np.int32)
    ref = Oracle(np.float64).bp_sbp(g, h, idx, angles, 0, A, vol=base.astype(np.float64))
    vol = dev(base)
    ostr.bprojectCB_GPU_SBP(vol, dev(h), dev(idx, torch.int32), dev(angles), 0, A)
    got = vol.cpu().numpy() - base
    print(f"{name} bp: rel RMSE {relrmse(got, ref - base):.2e} max {maxrel(got, ref - base):.2e}")
    assert relrmse(got, ref - base) < RMSE_BP
    assert maxrel(got, ref - base) < 2 * TOL


@pytest.mark.parametrize("pot", ["q2", "lange", "hyperbola", "huber"])
@pytest.mark.parametrize("name,g,angles,x", CASES, ids=[c[0] for c in CASES])
def test_prior_accumulates(ostr, name, g, angles, x, pot):
    from oracle.oracle import Oracle

    ostr.set_geometry(g)
    rng = np.random.default_rng(6)
    xn = (x + rng.normal(scale=0.004, size=x.size)).astype(np.float32)
    delta = 0.003
    b1 = rng.normal(size=g.n_voxels)
    b2 = rng.normal(size=g.n_voxels)
    rdd_ref, rd_ref = Oracle(np.float64).prior(g, xn, pot, delta, RDD=b1.copy(), RD=b2.copy())
    rdd = dev(b1)
    rd = dev(b2)
    ostr.prior_GPU_OSTR_potential(rdd, rd, dev(xn), pot, delta, g.z_xy_ratio)
    assert maxrel(rdd.cpu().numpy(), rdd_ref) < 1e-5
    assert relrmse(rd.cpu().numpy() - b2.astype(np.float32), rd_ref - b2) < 1e-5
    assert maxrel(rd.cpu().numpy() - b2.astype(np.float32), rd_ref - b2) < 1e-4


def test_prior_wrappers_match_reference_names(ostr):
    z = golden("tiny")
    g = geom_of(z)
    ostr.set_geometry(g)
    rdd = torch.zeros(g.n_voxels, device="cuda")
    rd = torch.zeros(g.n_voxels, device="cuda")
    ostr.prior_GPU_OSTR(rdd, rd, dev(z["x"]), float(z["delta"]), g.z_xy_ratio)
    assert maxrel(rdd.cpu().numpy(), z["lange_RDD"]) < TOL
    assert maxrel(rd.cpu().numpy(), z["lange_RD"]) < 1e-4
    rdd.zero_()
    rd.zero_()
    ostr.prior_GPU_OSTR_Q2(rdd, rd, dev(z["x"]), g.z_xy_ratio)
    assert maxrel(rdd.cpu().numpy(), z["q2_RDD"]) < TOL
    with pytest.raises(ValueError):
        ostr.prior_GPU_OSTR(rdd, rd, dev(z["x"]), 0.0, g.z_xy_ratio)


@pytest.mark.parametrize("name", ["tiny", "ragged"])
def test_elementwise_helpers(ostr, name):
    z = golden(name)
    g = geom_of(z)
    ostr.set_geometry(g)
    M = int(z["subset_num"])
    ostr.subset_num = M
    ostr.beta = float(z["beta"])
    assert maxrel(ostr.compute_yry(z["y"], z["s"]), z["yry"]) < 1e-6
    n = (g.n_angles // M) * g.n_bins
    h = ostr.compute_h(z["y"][:n], z["b"][:n], z["fp_cos"][:n], z["s"][:n])
    # h = y - ybar cancels; float expf may differ by an ulp: a few ulps of ybar
    assert np.abs(h - z["h"][:n]).max() <= 5e-7 * z["b"].max()
    upd = ostr.update_est(z["x"], z["upd_capL"], z["lange_RD"], z["upd_d"], z["lange_RDD"])
    assert maxrel(upd, z["upd"]) < 1e-6
    assert np.array_equal(ostr.regroup_prj(z["y"]), z["regroup_y"])
    assert np.array_equal(ostr.x_y_flip(z["flip_in"]), z["flip"])
    gy = ostr.compute_gamma_yry(z["yry"], z["gamma_length"])
    assert maxrel(gy, z["yry"] * z["gamma_length"]) < 1e-7
    sc = ostr.temp_fun2(M, g.n_voxels, z["upd_capL"])
    assert np.array_equal(sc, (np.float32(M) * z["upd_capL"]).astype(np.float32))


def test_numba_style_float64_buffers(ostr):
    """Float64 device/host buffers (the Numba notebook's np.zeros) work in place."""
    z = golden("tiny")
    g = geom_of(z)
    ostr.set_geometry(g)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    vol64 = torch.zeros(g.n_voxels, dtype=torch.float64, device="cuda")
    ostr.bprojectCB_GPU_SBP(vol64, dev(z["bp_in"], torch.float64), dev(idx, torch.int32),
                            dev(z["angles"]), 0, A)
    assert vol64.dtype == torch.float64
    assert maxrel(vol64.cpu().numpy(), z["bp"]) < TOL
    host = np.zeros(A * g.n_bins)
    ostr.fprojectCB_1R_GPU_OSTR_cos(z["x"], host, z["angles"], idx, 0, A)
    from oracle.oracle import Oracle

    ref = Oracle(np.float64).fp_ostr(g, z["x"], z["angles"], idx, 0, A)
    assert relrmse(host, ref) < RMSE_FP
    assert maxrel(host, ref) < TOL


class DevArray:
    """A device array known only through ``__cuda_array_interface__`` (what a
    Numba device array exposes; numba itself is not needed)."""

    def __init__(self, t: torch.Tensor):
        self._t = t.contiguous()  # owns the memory; never handed to the wrapper
        self.__cuda_array_interface__ = {
            "shape": tuple(self._t.shape), "strides": None, "version": 3,
            "typestr": {torch.float32: "<f4", torch.float64: "<f8",
                        torch.int32: "<i4"}[self._t.dtype],
            "data": (self._t.data_ptr(), False)}


def test_cuda_array_interface_objects(ostr):
    """Interface-only device arrays go in and come out in place, with results
    identical to the same calls on torch tensors (accumulating operators add
    to what the caller's buffer held)."""
    z = golden("tiny")
    g = geom_of(z)
    ostr.set_geometry(g)
    A = g.n_angles
    idx = dev(np.arange(A), torch.int32)
    ang = dev(z["angles"])
    x = dev(z["x"])
    line = torch.zeros(A * g.n_bins, device="cuda")
    ostr.fprojectCB_1R_GPU_OSTR_cos(x, line, ang, idx, 0, A)
    line_da = DevArray(torch.zeros(A * g.n_bins, device="cuda"))
    ostr.fprojectCB_1R_GPU_OSTR_cos(DevArray(x), line_da, DevArray(ang), DevArray(idx), 0, A)
    assert torch.equal(line_da._t, line)

    h = dev(z["bp_in"])
    vol = torch.ones(g.n_voxels, device="cuda")
    ostr.bprojectCB_GPU_SBP(vol, h, idx, ang, 0, A)
    vol_da = DevArray(torch.ones(g.n_voxels, dtype=torch.float64, device="cuda"))
    ostr.bprojectCB_GPU_SBP(vol_da, DevArray(h), DevArray(idx), DevArray(ang), 0, A)
    assert torch.equal(vol_da._t.float(), vol)

    rdd, rd = torch.zeros_like(x), torch.full_like(x, 0.5)
    ostr.prior_GPU_OSTR(rdd, rd, x, float(z["delta"]), g.z_xy_ratio)
    rdd_da = DevArray(torch.zeros_like(x))
    rd_da = DevArray(torch.full_like(x, 0.5))
    ostr.prior_GPU_OSTR(rdd_da, rd_da, DevArray(x), float(z["delta"]), g.z_xy_ratio)
    assert torch.equal(rdd_da._t, rdd) and torch.equal(rd_da._t, rd)


def test_bad_arguments_raise(ostr):
    from newrecon_gb300.native import NrError

    z = golden("tiny")
    g = geom_of(z)
    ostr.set_geometry(g)
    ostr.IMGSIZx = 0
    try:
        with pytest.raises(NrError) as e:
            ostr.fprojectCB_1R_GPU_OSTR_cos(dev(z["x"]), torch.zeros(10, device="cuda"),
                                            dev(z["angles"]), dev(np.arange(6), torch.int32), 0, 1)
        assert e.value.code == 1
    finally:
        ostr.set_geometry(g)
    with pytest.raises(NrError):
        ostr.fprojectCB_1R_GPU_OSTR_cos(dev(z["x"]), torch.zeros(10, device="cuda"),
                                        dev(z["angles"]), dev(np.arange(6), torch.int32), 3, 1)
