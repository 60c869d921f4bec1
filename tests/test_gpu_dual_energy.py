"""Dual-energy subtraction on the GPU against the NumPy restatement of
syncrecon.m (oracle/dual_energy_oracle.py): the subtraction and the 8-bit
histograms are exact (bit-identical floats, identical counts), the entropies
and Otsu levels equal to 1e-12."""
import ctypes
import os

import numpy as np
import pytest
import torch

from conftest import golden
from oracle import dual_energy_oracle as de
from test_oracle_golden import geom_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mod():
    from newrecon_gb300 import dual_energy, native

    native.load()
    return dual_energy


def volumes(shape, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    he = rng.gamma(2.0, 0.02, size=nx * ny * nz).astype(np.float32)
    le = (he * rng.uniform(1.1, 1.6, size=he.size) + rng.normal(0, 0.003, he.size)).astype(np.float32)
    return he, le


@pytest.mark.parametrize("shape", [(40, 24, 8), (33, 17, 5)], ids=["even", "tail"])
def test_subtract_and_entropy_exact(mod, shape):
    he, le = volumes(shape, 1)
    w = list(mod.DEFAULT_WEIGHTS)
    z = shape[2] // 2
    d, ent = mod.subtract(torch.from_numpy(he).cuda(), torch.from_numpy(le).cuda(), w,
                          slice_shape=shape[:2], entropy_slice=z)
    ref, ref64 = de.subtract(he, le, w)
    assert np.array_equal(d.cpu().numpy(), ref)
    n2 = shape[0] * shape[1]
    for k in range(len(w)):
        assert ent[k] == pytest.approx(de.entropy(ref64[k, z * n2:(z + 1) * n2]), abs=1e-12)


def test_mask_and_otsu(mod):
    he, le = volumes((40, 24, 8), 2)
    he[: he.size // 3] *= 6.0   # a second mode
    t = mod.otsu_level(he)
    assert t == de.otsu_level(de.hist8(he))
    assert 0.0 < t < 1.0
    d, _ = mod.subtract(he, le, [0.3, 0.6], mask_level=t)
    ref, _ = de.subtract(he, le, [0.3, 0.6], mask_level=t)
    assert np.array_equal(d.cpu().numpy(), ref)
    assert (d.cpu().numpy()[:, he <= t] == 0).all()


def test_syncrecon_files(mod, tmp_path):
    shape = (33, 17, 5)
    he, le = volumes(shape, 3)
    he.tofile(tmp_path / "he.raw")
    le.tofile(tmp_path / "le.raw")
    got = mod.syncrecon(str(tmp_path / "he.raw"), str(tmp_path / "le.raw"), shape,
                        str(tmp_path), entropy_slice=2, log=lambda *_: None)
    ref, ref64 = de.subtract(he, le, mod.DEFAULT_WEIGHTS)
    n2 = shape[0] * shape[1]
    for k, w in enumerate(mod.DEFAULT_WEIGHTS):
        f = tmp_path / f"d_{w:g}.raw"
        assert f.exists(), f
        assert np.array_equal(np.fromfile(f, np.float32), ref[k])
        assert got[k][0] == w
        assert got[k][1] == pytest.approx(de.entropy(ref64[k, 2 * n2:3 * n2]), abs=1e-12)


def test_reconstruct_pair(mod):
    """Two OSTR reconstructions and their subtraction without leaving the GPU."""
    z = golden("tiny")
    g = geom_of(z)
    he_scan = dict(prj=z["y"], blank=z["b"])
    le_scan = dict(prj=(z["y"] * 0.8).astype(np.float32), blank=(z["b"] * 0.8).astype(np.float32))
    xh, xl, d, ent = mod.reconstruct_pair(g, he_scan, le_scan, [0.5, 1.0], angles=z["angles"],
                                          subset_num=int(z["subset_num"]), iter_num=2,
                                          beta=float(z["beta"]), delta=float(z["delta"]),
                                          entropy_slice=3)
    ref, _ = de.subtract(xh.cpu().numpy(), xl.cpu().numpy(), [0.5, 1.0])
    assert np.array_equal(d.cpu().numpy(), ref)
    assert len(ent) == 2 and all(e >= 0 for e in ent)


def test_bad_arguments(mod):
    from newrecon_gb300 import native
    from newrecon_gb300.native import NrError

    he = torch.zeros(64, device="cuda")
    w = np.array([0.5])
    out = torch.empty(64, device="cuda")
    with pytest.raises(NrError) as e:  # misaligned output
        native.call("nr_de_subtract", ctypes.c_void_p(he.data_ptr()),
                    ctypes.c_void_p(he.data_ptr()), w.ctypes.data_as(ctypes.c_void_p), 1, 32,
                    -1.0, ctypes.c_void_p(out.data_ptr() + 4), 0, 0, None, None)
    assert e.value.code == 2
    with pytest.raises(ValueError):
        mod.subtract(he, he, list(np.linspace(0, 1, 17)))


def _hard_cases(weights, n_each, seed):
    """he, le pairs that put b - a w near float rounding boundaries, in heavy
    cancellation, and on special values, for the weights given."""
    rng = np.random.default_rng(seed)
    he, le = [], []
    for w in weights:
        if w == 0.0 or not np.isfinite(w):
            continue
        # near-ties: a w = ulp(b)/2 (1 + delta), delta log-uniform 2^-30 .. 2^-8, either sign
        b = rng.uniform(0.5, 4.0, n_each).astype(np.float32) * np.float32(2.0) ** rng.integers(-20, 20, n_each).astype(np.float32)
        ulp = np.spacing(b).astype(np.float64)
        delta = 2.0 ** rng.uniform(-30, -8, n_each) * rng.choice([-1.0, 1.0], n_each)
        k = rng.integers(1, 8, n_each) * 2 - 1          # odd multiples of half an ulp
        a = (k * ulp / 2 * (1 + delta) / w).astype(np.float32)
        he.append(b); le.append(a)
        # cancellation: b = a w (1 + delta), delta log-uniform 2^-24 .. 2^-2
        a = rng.gamma(2.0, 0.02, n_each).astype(np.float32)
        delta = 2.0 ** rng.uniform(-24, -2, n_each) * rng.choice([-1.0, 1.0], n_each)
        he.append((a.astype(np.float64) * w * (1 + delta)).astype(np.float32)); le.append(a)
    # special values and magnitudes
    sp = np.array([0.0, -0.0, 1e-45, -1e-45, 1e-38, 3.4e38, -3.4e38, np.inf, -np.inf, np.nan,
                   1.0, -1.0, 2.0 ** -100, 2.0 ** 100, 0.0501, 0.08], np.float32)
    hh, ll = np.meshgrid(sp, sp)
    he.append(hh.ravel()); le.append(ll.ravel())
    he = np.concatenate(he).astype(np.float32)
    le = np.concatenate(le).astype(np.float32)
    pad = (-he.size) % 4
    return np.concatenate([he, np.ones(pad, np.float32)]), np.concatenate([le, np.ones(pad, np.float32)])


def _same_bits(got, ref):
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    return np.array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))


@pytest.mark.parametrize("weights", [
    [0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9],
    [1 / 3, np.pi / 10, -0.45, 1e-30, 3e25, 1.0, 0.0, 2.0 ** -40, 1.2345678901234567],
], ids=["syncrecon", "awkward"])
def test_fp32_path_is_bit_exact_on_hard_cases(mod, weights):
    """The FP32 evaluation (with its FP64 fallback) reproduces
    float(double(he) - double(le) * w) bit for bit, signed zeros included,
    near float rounding boundaries, in heavy cancellation and on special values."""
    he, le = _hard_cases(weights, 200_000, 5)
    d, _ = mod.subtract(torch.from_numpy(he).cuda(), torch.from_numpy(le).cuda(), weights)
    ref, _ = de.subtract(he, le, weights)
    got = d.cpu().numpy()
    for k in range(len(weights)):
        assert _same_bits(got[k], ref[k]), weights[k]
    # the unaligned (scalar) path too, and the mask
    n = he.size - 3
    d, _ = mod.subtract(torch.from_numpy(he[:n]).cuda(), torch.from_numpy(le[:n]).cuda(), weights,
                        mask_level=0.05)
    ref, _ = de.subtract(he[:n], le[:n], weights, mask_level=0.05)
    got = d.cpu().numpy()
    for k in range(len(weights)):
        assert _same_bits(got[k], ref[k]), weights[k]


def test_slice_histograms_exact_near_bin_edges(mod):
    """The per-weight 8-bit histograms of the double values, counted exactly,
    with values placed near the bin edges 255 v = k + 1/2 (the float
    evaluation must leave the undecidable ones to FP64)."""
    from newrecon_gb300 import native

    rng = np.random.default_rng(11)
    weights = [0.1, 0.3, 0.5, 0.7, 0.9, 1 / 3]
    n = 1 << 18
    le = rng.uniform(0.0, 0.3, n).astype(np.float32)
    k = rng.integers(-2, 258, n)
    off = 2.0 ** rng.uniform(-30, -17, n) * rng.choice([-1.0, 1.0], n)
    w = np.array(weights)[rng.integers(0, len(weights), n)]
    he = ((k + 0.5) / 255.0 + off + le.astype(np.float64) * w).astype(np.float32)
    he[:64] = np.float32(np.nan)
    he[64:128] = 0.0
    le[64:96] = 0.0
    h_d, l_d = torch.from_numpy(he).cuda(), torch.from_numpy(le).cuda()
    wd = np.asarray(weights, np.float64)
    d = torch.empty((len(weights), n), device="cuda")
    hist = torch.zeros((len(weights), 256), dtype=torch.int32, device="cuda")
    native.call("nr_de_subtract", ctypes.c_void_p(h_d.data_ptr()), ctypes.c_void_p(l_d.data_ptr()),
                wd.ctypes.data_as(ctypes.c_void_p), len(weights), n, -1.0,
                ctypes.c_void_p(d.data_ptr()), 0, n, ctypes.c_void_p(hist.data_ptr()), None)
    torch.cuda.synchronize()
    _, ref64 = de.subtract(he, le, weights)
    got = hist.cpu().numpy()
    for j in range(len(weights)):
        assert np.array_equal(got[j], de.hist8(ref64[j])), weights[j]
