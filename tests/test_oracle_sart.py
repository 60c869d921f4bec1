"""The SART part of the oracle against fixtures made by the reference's own
SART kernels (tests/golden/sart_*.npz, tests/golden/make_golden.py --sart).

The float32 oracle follows the reference's operation order and must match to
a few float ulps (bit-exact on x86-64, where the fixtures were made); the
float64 oracle to float32 rounding accuracy.  The OS-SART loops in the
fixtures are composed from the reference's launch wrappers (the reference has
no OS-SART driver); the oracle's loop must reproduce them.
"""
import platform

import numpy as np
import pytest

from conftest import golden
from oracle.oracle import Oracle
from test_oracle_golden import close32, geom_of, rel_rmse


@pytest.fixture(params=["tiny", "ragged"])
def case(request):
    z = golden(f"sart_{request.param}")
    return request.param, z, geom_of(z)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sart_projector(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    tol = 2e-6 if dtype == np.float32 else 5e-5
    for cos, key in ((False, "fp"), (True, "fpc")):
        est, norm = O.fp_sart(g, z["x"], z["angles"], idx, 0, A, cos)
        assert close32(est, z[f"{key}_est"], tol), (name, key)
        assert close32(norm, z[f"{key}_norm"], 2e-6 if dtype == np.float32 else 1e-5), (name, key)
    ridx = O.reorder_index(A, int(z["subset_num"]))
    Vs = A // int(z["subset_num"])
    est, norm = O.fp_sart(g, z["x"], z["angles"], ridx, Vs, 2 * Vs, True)
    assert close32(est, z["fpc_sub1_est"], tol)
    assert close32(norm, z["fpc_sub1_norm"], 2e-6 if dtype == np.float32 else 1e-5)


def test_sart_projector_bitexact_float32(case):
    if platform.machine() != "x86_64":
        pytest.skip("fixtures were generated on x86-64")
    name, z, g = case
    A = g.n_angles
    est, norm = Oracle(np.float32).fp_sart(g, z["x"], z["angles"], np.arange(A, dtype=np.int32),
                                          0, A, True)
    assert np.array_equal(est, z["fpc_est"]) and np.array_equal(norm, z["fpc_norm"])


def test_sart_chord_is_gamma_chord(case):
    """normprj of the SART walk is the in-volume chord (the OSTR chord gamma)."""
    name, z, g = case
    O = Oracle(np.float64)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    _, norm = O.fp_sart(g, z["x"], z["angles"], idx, 0, A, False)
    chord = O.fp_gamma(g, z["angles"], idx, 0, A, "chord")
    assert np.array_equal(norm, chord)


def test_prj_diff(case):
    name, z, g = case
    Vs = g.n_angles // int(z["subset_num"])
    ridx = Oracle().reorder_index(g.n_angles, int(z["subset_num"]))
    p = z["line"].reshape(g.n_angles, -1)[ridx[Vs:2 * Vs]].ravel()
    d = Oracle(np.float32).sart_prj_diff(p, z["fpc_sub1_est"], z["fpc_sub1_norm"])
    assert np.array_equal(d, z["diff_sub1"])
    # rays that miss the volume (chord 0) give 0
    miss = z["fpc_sub1_norm"] == 0
    assert (z["diff_sub1"][miss] == 0).all()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sart_prior(case, dtype):
    name, z, g = case
    pr = Oracle(dtype).prior_sart(g, z["x"], float(z["delta"]))
    assert close32(pr, z["prior"], 2e-6 if dtype == np.float32 else 1e-4)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ossart_back_projection(case, dtype):
    name, z, g = case
    O = Oracle(dtype)
    A, M = g.n_angles, int(z["subset_num"])
    Vs = A // M
    ridx = O.reorder_index(A, M)
    lam, beta = float(z["lam"]), float(z["beta"])
    tol = 2e-6 if dtype == np.float32 else 2e-5
    x1 = O.bp_ossart(g, z["x"], z["bp_in"], ridx, z["angles"], Vs, 2 * Vs, lam)
    assert close32(x1, z["bp_plain"], tol)
    x2 = O.bp_ossart(g, z["x"], z["bp_in"], ridx, z["angles"], Vs, 2 * Vs, lam, z["prior"], beta)
    assert close32(x2, z["bp_reg"], tol)
    assert (x1 >= 0).all() and (x2 >= 0).all()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("key", ["ossart", "ossart_nocos", "ossart_reg"])
def test_ossart_loop(case, dtype, key):
    name, z, g = case
    kw = dict(subset_num=int(z["subset_num"]), iter_num=int(z["iters"]), lam=float(z["lam"]),
              use_cos=key != "ossart_nocos")
    if key == "ossart_reg":
        kw.update(regularized=True, beta=float(z["beta"]), delta=float(z["delta"]))
    x = Oracle(dtype).ossart(g, z["angles"], z["line"], **kw)
    r = rel_rmse(x, z[key])
    assert r < (1e-6 if dtype == np.float32 else 2e-5), (name, key, r)


def test_line_integrals():
    O = Oracle(np.float64)
    y = np.array([100.0, 50.0, 0.0, 10.0, 5.0], np.float64)
    b = np.array([200.0, 50.0, 10.0, 0.0, 10.0], np.float64)
    s = np.array([0.0, 10.0, 0.0, 1.0, 5.0], np.float64)
    out = O.line_integrals(y, b, s)
    ref = np.array([np.log(2.0), np.log(50.0 / 40.0), 0.0, 0.0, 0.0])
    np.testing.assert_allclose(out, ref, rtol=1e-15)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_4r_projector(case, dtype):
    """Sub-rays against the reference's 4R kernel; the merge as the reference intends it."""
    name, z, g = case
    O = Oracle(dtype)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    sub = np.zeros(4 * A * g.n_bins, dtype)
    merged = O.fp_4r(g, z["x"], z["angles"], idx, 0, A, use_cos=False, layout="ji", sub=sub)
    tol = 2e-6 if dtype == np.float32 else 5e-5
    assert close32(sub, z["fp4r_sub"], tol)
    assert close32(merged, z["fp4r_merged_ji"], tol)
    if dtype == np.float32 and platform.machine() == "x86_64":
        assert np.array_equal(sub, z["fp4r_sub"])
        assert np.array_equal(merged, z["fp4r_merged_ji"])
    # the [i][j] layout is the transpose; cos scales the merged value
    ij = O.fp_4r(g, z["x"], z["angles"], idx, 0, A, use_cos=True, layout="ij")
    ct = np.cos(z["angles"].astype(dtype))[:, None, None]
    want = merged.reshape(A, g.nby, g.nbx).transpose(0, 2, 1) * ct
    assert close32(ij, want.ravel(), 1e-6)


def test_4r_matches_centre_ray_where_linear(case):
    """Where a bin's chord through a uniform volume is linear in the detector
    position (rays entering the top face and leaving the bottom face), the mean
    of the 2 x 2 symmetric sub-rays equals the centre ray; at the shadow's
    edges they differ (that is what super-sampling is for)."""
    name, z, g = case
    O = Oracle(np.float64)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    ones = np.ones(g.n_voxels)
    r4 = O.fp_4r(g, ones, z["angles"], idx, 0, A, layout="ij").reshape(A, g.nbx, g.nby)
    est, norm = O.fp_sart(g, ones, z["angles"], idx, 0, A, False)
    est = est.reshape(A, g.nbx, g.nby)
    full = norm.reshape(A, g.nbx, g.nby) >= 0.9 * norm.max()
    inner = full.copy()   # bins whose 8 neighbours are fully inside the shadow too
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            inner &= np.roll(np.roll(full, di, axis=1), dj, axis=2)
    inner[:, [0, -1], :] = False
    inner[:, :, [0, -1]] = False
    assert inner.sum() > 0.2 * full.sum()
    assert np.abs(r4[inner] - est[inner]).max() < 1e-6 * est.max()
    assert np.abs(r4 - est).max() > 1e-3 * est.max()


def test_ossart_supersampled_fits_supersampled_data(case):
    """On data made by the 4R projector, OS-SART with the 4R projector fits the
    data better (and lands nearer the truth) than with one ray per bin."""
    name, z, g = case
    O = Oracle(np.float64)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    line4 = O.fp_4r(g, z["x"], z["angles"], idx, 0, A, layout="ij")
    kw = dict(subset_num=int(z["subset_num"]), iter_num=4, lam=float(z["lam"]), use_cos=False)
    x1 = O.ossart(g, z["angles"], line4, **kw)
    x4 = O.ossart(g, z["angles"], line4, supersample=True, **kw)
    res = lambda x: rel_rmse(O.fp_4r(g, x, z["angles"], idx, 0, A, layout="ij"), line4)
    assert res(x4) < 0.8 * res(x1)
    assert rel_rmse(x4, z["x"]) < rel_rmse(x1, z["x"])
    assert (x4 >= 0).all()
