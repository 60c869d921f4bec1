"""The oracle against the golden fixtures made by the reference's own code.

tests/golden/*.npz hold outputs of the reference's kernel bodies and gold
driver compiled for the CPU (tests/golden/make_golden.py).  The float32
oracle restates the reference's arithmetic operation for operation and must
match to within a few float ulps (bit-exact on x86-64; a last-ulp difference
of libm between platforms is allowed); the float64 oracle must match to
float32 rounding accuracy.
"""
import numpy as np
import pytest

from conftest import golden
from newrecon_gb300.geometry import Geometry, NrGeom
from oracle.oracle import Oracle

CASES = ["tiny", "ragged"]


def geom_of(z) -> Geometry:
    vals = z["geom"]
    kw = {}
    for (name, ctype), v in zip(NrGeom._fields_, vals):
        kw[name] = int(v) if ctype.__name__.startswith("c_int") else float(np.float32(v))
    return Geometry(**kw)


def close32(a, b, rtol=2e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() <= rtol * scale


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.fixture(params=CASES)
def case(request):
    z = golden(request.param)
    return request.param, z, geom_of(z)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_forward_projection(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    fp = O.fp_ostr(g, z["x"], z["angles"], idx, 0, A)
    Vs = A // int(z["subset_num"])
    fp1 = O.fp_ostr(g, z["x"], z["angles"], z["ridx"], Vs, 2 * Vs)
    tol = 2e-6 if dtype == np.float32 else 5e-5
    assert close32(fp, z["fp_cos"], tol), name
    assert close32(fp1, z["fp_cos_sub1"], tol), name


def test_forward_projection_bitexact_float32(case):
    """Same operation order as the reference: identical on this platform."""
    import platform

    if platform.machine() != "x86_64":
        pytest.skip("fixtures were generated on x86-64")
    name, z, g = case
    O = Oracle(np.float32)
    A = g.n_angles
    fp = O.fp_ostr(g, z["x"], z["angles"], np.arange(A, dtype=np.int32), 0, A)
    assert np.array_equal(fp, z["fp_cos"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gamma_length(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    A = g.n_angles
    gam = O.fp_gamma(g, z["angles"], np.arange(A, dtype=np.int32), 0, A, "length")
    assert close32(gam, z["gamma_length"], 2e-6 if dtype == np.float32 else 1e-6)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_back_projection(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    A = g.n_angles
    Vs = A // int(z["subset_num"])
    bp = O.bp_sbp(g, z["bp_in"], np.arange(A, dtype=np.int32), z["angles"], 0, A)
    bp1 = O.bp_sbp(g, z["bp_in"][: Vs * g.n_bins], z["ridx"], z["angles"], Vs, 2 * Vs)
    tol = 2e-6 if dtype == np.float32 else 5e-5
    assert close32(bp, z["bp"], tol)
    assert close32(bp1, z["bp_sub1"], tol)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_priors(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    d = float(z["delta"])
    rdd, rd = O.prior(g, z["x"], "lange", d)
    assert close32(rdd, z["lange_RDD"], 2e-6 if dtype == np.float32 else 1e-5)
    assert close32(rd, z["lange_RD"], 2e-6 if dtype == np.float32 else 1e-4)
    rdd, rd = O.prior(g, z["x"], "q2", d)
    assert close32(rdd, z["q2_RDD"], 2e-6)
    assert close32(rd, z["q2_RD"], 2e-6 if dtype == np.float32 else 1e-4)
    # G_Huber_prior (Tomo_OSTR.cu:258-325) is the hyperbola gradient with
    # unscaled z distances; the hyperbola potential with z_xy_ratio = 1 is it.
    _, rdh = O.prior(g, z["x"], "hyperbola", d, zxy=1.0)
    assert close32(rdh, z["hyp_grad"], 2e-6 if dtype == np.float32 else 1e-4)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_host_helpers(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    s = z["s"]
    assert close32(O.compute_yry(z["y"], s), z["yry"], 1e-6)
    # the reference's compute_h covers one subset's bins (Tomo_OSTR_gold.cpp:251)
    n = (g.n_angles // int(z["subset_num"])) * g.n_bins
    h = O.compute_h(z["y"][:n], z["b"][:n], z["fp_cos"][:n], s[:n])
    # h = y - ybar cancels: the float reference carries ulp(ybar) absolute error
    assert close32(h, z["h"][:n], 2e-6 if dtype == np.float32 else 1e-4)
    upd = O.update_est(z["x"], z["upd_capL"], z["lange_RD"], z["upd_d"], z["lange_RDD"],
                       float(z["beta"]))
    assert close32(upd, z["upd"], 2e-6 if dtype == np.float32 else 1e-5)
    rg = O.regroup(z["y"], g.n_angles, int(z["subset_num"]))
    assert np.array_equal(rg.astype(np.float32), z["regroup_y"])


def test_x_y_flip_layout(case):
    name, z, g = case
    flipped = z["flip_in"].reshape(g.nby, g.nbx).T.ravel()
    assert np.array_equal(flipped, z["flip"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("pot,key", [("lange", "recon_lange"), ("q2", "recon_q2")])
def test_reconstruction(case, dtype, pot, key):
    name, z, g = case
    O = Oracle(dtype)
    x = O.reconstruct(g, z["angles"], z["y"], z["b"], z["s"], subset_num=int(z["subset_num"]),
                      iter_num=int(z["iters"]), beta=float(z["beta"]), delta=float(z["delta"]),
                      potential=pot)
    if dtype == np.float32:
        assert close32(x, z[key], 5e-6)
    else:
        assert rel_rmse(x, z[key]) < 1e-5


def test_small_workload_pin():
    """Gold-driver reconstruction of the 256x128x24 workload, sampled."""
    from newrecon_gb300.geometry import config
    from newrecon_gb300.phantom import breast_phantom, poisson_counts

    z = golden("small")
    cfg = config("small")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    assert np.isclose(x.astype(np.float64).sum(), float(z["phantom_sum"]), rtol=1e-9)
    O = Oracle(np.float64)
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = O.fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles)
    y = poisson_counts(line, cfg.I0, 0)
    assert np.isclose(y.astype(np.float64).sum(), float(z["counts_sum"]), rtol=1e-9)
    O32 = Oracle(np.float32)
    fp0 = O32.fp_ostr(g, x, cfg.angles, idx, 0, 1)
    assert close32(fp0[z["fp0_idx"]], z["fp0_val"], 2e-6)
    b = np.full_like(y, cfg.I0)
    xr = O.reconstruct(g, cfg.angles, y, b, subset_num=cfg.subset_num, iter_num=cfg.iter_num,
                       beta=cfg.beta, delta=cfg.delta, potential="lange")
    samp = xr[z["recon_lange_idx"]]
    assert rel_rmse(samp, z["recon_lange_val"]) < 1e-4
    sums = xr.reshape(g.nz, -1).sum(axis=1)
    assert rel_rmse(sums, z["recon_lange_slice_sums"]) < 1e-5
