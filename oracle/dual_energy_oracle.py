"""TEST INFRASTRUCTURE ONLY: NumPy restatement of syncrecon.m (the reference's
dual-energy post-processing), the checker of newrecon_gb300.dual_energy.

MATLAB is absent, so parity with MATLAB's own outputs is unpinned; the
restatement follows the script and the documented behaviour of the MATLAB
functions it calls:

* ``d = he - le*weight`` (syncrecon.m:28) on volumes fread as double from
  float32 files, written back with fwrite 'float': float(double(he) -
  double(le) * w), two double roundings;
* ``entropy(d(:,:,24))`` (:34): the 8-bit image (round(255 v), half away
  from zero, saturated), its 256-bin histogram, -sum p log2 p over non-empty
  bins;
* ``graythresh(he)`` / ``imbinarize(he, t)`` (:7-8): Otsu's method (Otsu
  1979) on the same 8-bit histogram, level = (mean index of the maxima of the
  between-class variance - 1) / 255, 0 when the maximum is not finite; the
  mask he > t.
"""
from __future__ import annotations

import numpy as np


def subtract(he, le, weights, mask_level=None):
    h = np.asarray(he, np.float32).astype(np.float64)
    l = np.asarray(le, np.float32).astype(np.float64)
    if mask_level is not None:
        keep = h > mask_level
        h = np.where(keep, h, 0.0)
        l = np.where(keep, l, 0.0)
    d64 = np.stack([h - l * float(w) for w in weights])
    return d64.astype(np.float32), d64


def im8(v):
    v = np.asarray(v, np.float64)
    r = np.sign(255.0 * v) * np.floor(np.abs(255.0 * v) + 0.5)   # half away from zero
    r = np.where(np.isnan(r), 0.0, r)
    return np.clip(r, 0, 255).astype(np.int64)


def hist8(v):
    return np.bincount(im8(v).ravel(), minlength=256).astype(np.int64)


def entropy(v):
    h = hist8(v).astype(np.float64)
    p = h[h > 0] / h.sum()
    return float(-np.sum(p * np.log2(p)))


def otsu_level(counts):
    c = np.asarray(counts, np.float64)
    p = c / c.sum()
    omega = np.cumsum(p)
    mu = np.cumsum(p * np.arange(1, 257))
    mu_t = mu[-1]
    with np.errstate(divide="ignore", invalid="ignore"):
        sb = (mu_t * omega - mu) ** 2 / (omega * (1 - omega))
    finite = sb[~np.isnan(sb)]
    if finite.size == 0:
        return 0.0
    mx = finite.max()
    if not np.isfinite(mx):
        return 0.0
    idx = np.mean(np.nonzero(sb == mx)[0] + 1)
    return float((idx - 1) / 255.0)
