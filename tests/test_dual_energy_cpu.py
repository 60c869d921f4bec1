"""The dual-energy oracle's known answers, and the library's host-side
histogram statistics (nr_hist_entropy, nr_otsu_level: plain C, no GPU) against
it."""
import ctypes

import numpy as np
import pytest

from oracle import dual_energy_oracle as de


def test_subtraction_is_double_then_float():
    he = np.array([0.3, 1e-8, 0.1], np.float32)
    le = np.array([0.2, 3e-8, 0.7], np.float32)
    d, d64 = de.subtract(he, le, [0.1, 0.5])
    want = (np.float64(he[0]) - np.float64(le[0]) * 0.1)
    assert d64[0, 0] == want and d[0, 0] == np.float32(want)
    assert d.dtype == np.float32 and d.shape == (2, 3)


def test_im8_rounding_and_saturation():
    v = np.array([-1.0, 0.0, 0.5 / 255, 1.5 / 255, 2.4999 / 255, 0.999, 1.0, 7.0, np.nan])
    assert list(de.im8(v)) == [0, 0, 1, 2, 2, 255, 255, 255, 0]


def test_entropy_known_answers():
    assert de.entropy(np.zeros(100)) == 0.0
    assert de.entropy(np.arange(256) / 255.0) == pytest.approx(8.0)
    assert de.entropy(np.array([0.0, 1.0] * 50)) == pytest.approx(1.0)


def test_otsu_splits_two_modes():
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.normal(0.2, 0.02, 5000), rng.normal(0.7, 0.02, 5000)])
    t = de.otsu_level(de.hist8(v))
    assert 0.3 < t < 0.6
    assert de.otsu_level(de.hist8(np.full(10, 0.5))) == 0.0   # one occupied bin


@pytest.fixture(scope="module")
def lib():
    from newrecon_gb300 import native

    return native.load()


def test_host_statistics_match_oracle(lib):
    rng = np.random.default_rng(1)
    for v in (rng.uniform(0, 1, 4000), rng.normal(0.05, 0.02, 4000),
              np.concatenate([rng.normal(0.2, 0.05, 3000), rng.normal(0.8, 0.05, 1000)]),
              np.full(50, 0.25)):
        h = de.hist8(v).astype(np.int32)
        e = ctypes.c_double()
        assert lib.nr_hist_entropy(h.ctypes.data_as(ctypes.c_void_p), v.size, ctypes.byref(e)) == 0
        assert e.value == pytest.approx(de.entropy(v), rel=1e-12, abs=1e-12)
        t = ctypes.c_double()
        assert lib.nr_otsu_level(h.ctypes.data_as(ctypes.c_void_p), ctypes.byref(t)) == 0
        assert t.value == de.otsu_level(h)
    z = np.zeros(256, np.int32)
    assert lib.nr_otsu_level(z.ctypes.data_as(ctypes.c_void_p), ctypes.byref(t)) == 2
