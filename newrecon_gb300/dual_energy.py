"""Dual-energy weighted subtraction on the device (the reference's syncrecon.m).

syncrecon.m reads a high-energy (HE) and a low-energy (LE) OSTR volume
(``reshape(.., 2000, 1000, 48)``: x fastest, the [z][y][x] layout here), and
for each weight w of a list writes ``d = he - le*w`` as float32 to
``d_<w>.raw`` and prints the entropy of slice 24 (1-based) of d; it also
computes an Otsu mask of he whose use is commented out.

``subtract`` does all weights in one streaming kernel (d computed in double
and rounded once to float, as MATLAB does on the float volumes it reads) and
the slice histograms for the entropies in a second, small one; ``syncrecon``
is the script's file-level workflow; ``reconstruct_pair`` runs the two OSTR
reconstructions and the subtraction without leaving the GPU.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import native
from .geometry import Geometry
from .ostr import _in, _p, _stream

MAX_WEIGHTS = 16
# syncrecon.m:24: the weight list it sweeps
DEFAULT_WEIGHTS = (0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9)


def _entropy(hist: np.ndarray, count: int) -> float:
    h = np.ascontiguousarray(hist, np.int32)
    e = ctypes.c_double(0.0)
    native.call("nr_hist_entropy", h.ctypes.data_as(ctypes.c_void_p), int(count), ctypes.byref(e))
    return float(e.value)


def otsu_level(x) -> float:
    """graythresh(x): Otsu's threshold of the 8-bit histogram of x, in [0, 1]."""
    t = _in(x)
    hist = torch.zeros(256, dtype=torch.int32, device=t.device)
    native.call("nr_hist8", _p(t), int(t.numel()), _p(hist), _stream())
    h = hist.cpu().numpy()
    lvl = ctypes.c_double(0.0)
    native.call("nr_otsu_level", h.ctypes.data_as(ctypes.c_void_p), ctypes.byref(lvl))
    return float(lvl.value)


def subtract(he, le, weights: Sequence[float] = DEFAULT_WEIGHTS, *,
             slice_shape: Optional[Tuple[int, int]] = None, entropy_slice: Optional[int] = None,
             mask_level: Optional[float] = None, out: Optional[torch.Tensor] = None):
    """d[k] = he - le * weights[k] for every weight, on the device.

    he, le: volumes of the same size (any layout; flat [z][y][x] for the slice
    entropies).  slice_shape = (nx, ny) and entropy_slice = z (0-based) select
    the slice whose entropy is returned per weight (MATLAB's d(:,:,z+1));
    mask_level zeroes he and le where he <= mask_level first.  Returns
    (d as a [K, N] float32 CUDA tensor, list of entropies or None).
    """
    h = _in(he)
    l = _in(le)
    if h.numel() != l.numel():
        raise ValueError("he and le differ in size")
    w = np.ascontiguousarray(weights, np.float64)
    if not 1 <= w.size <= MAX_WEIGHTS:
        raise ValueError(f"1 to {MAX_WEIGHTS} weights")
    n = h.numel()
    d = torch.empty((w.size, n), dtype=torch.float32, device=h.device) if out is None else out
    if d.numel() != w.size * n or not d.is_contiguous() or d.dtype != torch.float32:
        raise ValueError("out must be a contiguous float32 [K, N] tensor")
    hist = None
    begin = length = 0
    if entropy_slice is not None:
        if slice_shape is None:
            raise ValueError("slice_shape (nx, ny) is needed for the slice entropy")
        length = int(slice_shape[0]) * int(slice_shape[1])
        begin = int(entropy_slice) * length
        if begin < 0 or begin + length > n:
            raise ValueError("entropy_slice outside the volume")
        hist = torch.empty((w.size, 256), dtype=torch.int32, device=h.device)
    native.call("nr_de_subtract", _p(h), _p(l), w.ctypes.data_as(ctypes.c_void_p), int(w.size),
                int(n), float(-1.0 if mask_level is None else mask_level), _p(d), int(begin),
                int(length), _p(hist), _stream())
    ent = None
    if hist is not None:
        hh = hist.cpu().numpy()
        ent = [_entropy(hh[k], length) for k in range(w.size)]
    return d, ent


def weight_name(w: float) -> str:
    """The file-name form of a weight, as MATLAB's num2str (0.1 -> "0.1")."""
    return f"{w:.5g}"


def syncrecon(he_path: str, le_path: str, shape: Tuple[int, int, int], out_dir: str,
              weights: Sequence[float] = DEFAULT_WEIGHTS, entropy_slice: int = 23,
              mask: bool = False, log=print) -> List[Tuple[float, float]]:
    """syncrecon.m's workflow: read two raw float32 volumes (nx, ny, nz), write
    d_<w>.raw for each weight to out_dir, and return [(weight, entropy of
    slice entropy_slice)].  mask=True applies the Otsu mask of he first."""
    nx, ny, nz = shape
    n = nx * ny * nz
    vols = []
    for path in (he_path, le_path):
        a = np.fromfile(path, dtype=np.float32, count=n)
        if a.size != n:
            raise ValueError(f"{path}: fewer than {n} floats")
        vols.append(torch.from_numpy(a).cuda())
    level = otsu_level(vols[0]) if mask else None
    d, ent = subtract(vols[0], vols[1], weights, slice_shape=(nx, ny),
                      entropy_slice=entropy_slice, mask_level=level)
    out = []
    host = d.cpu().numpy()
    for k, w in enumerate(weights):
        host[k].tofile(os.path.join(out_dir, f"d_{weight_name(w)}.raw"))
        log(w)
        log(ent[k])
        out.append((float(w), ent[k]))
    return out


def reconstruct_pair(geom: Geometry, he_scan: dict, le_scan: dict, weights=DEFAULT_WEIGHTS, *,
                     angles, subset_num: int, iter_num: int, beta: float, delta: float,
                     potential: str = "lange", entropy_slice: Optional[int] = None):
    """Two OSTR reconstructions (he_scan / le_scan: dicts with prj, blank and
    optional scat, [view][i][j]) and the weighted subtraction, all on the GPU.
    Returns (he volume, le volume, d [K, N], entropies)."""
    from . import ostr

    vols = []
    for scan in (he_scan, le_scan):
        plan = ostr.OSTR(geom, subset_num=subset_num, beta=beta, delta=delta,
                         potential=potential, has_scatter=scan.get("scat") is not None)
        plan.setup(angles, scan["prj"], scan["blank"], scan.get("scat"))
        x = torch.zeros(geom.n_voxels, dtype=torch.float32, device="cuda")
        plan.iterate(x, iter_num)
        plan.check()
        vols.append(x)
    d, ent = subtract(vols[0], vols[1], weights, slice_shape=(geom.nx, geom.ny),
                      entropy_slice=entropy_slice)
    return vols[0], vols[1], d, ent
