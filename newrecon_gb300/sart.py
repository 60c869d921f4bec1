"""The SART / OS-SART family on the GB300 projectors.

Reference-shaped launch wrappers (``Tomo_OSTR.cu:2249-2332, 2460-2558``), same
names and arguments, reading the geometry from the module-level names of
``newrecon_gb300.ostr`` like the OSTR wrappers:

* ``fprojectCB_1R_GPU_SART`` / ``fprojectCB_1R_GPU_SART_cos``: line integral
  (times cos theta) and the ray's in-volume chord; missed rays untouched;
* ``fprojectCB1_4R_GPU_SART``: the 2 x 2 super-sampled projector, fixed
  (the reference's does not compile and never sets its fourth sub-ray index);
* ``SART_prj_diff``: (prj - est) / normprj, 0 where normprj is 0;
* ``bprojectCB_4B_GPU_SART`` / ``bprojectCB_4B_GPU_SART_R``: the in-place
  OS-SART update x = max(0, x + lambda (u [+ beta prior]) / sensitivity);
* ``prior_GPU_SART``: prior += the hyperbola gradient with plain neighbour
  distances (accumulates; the caller zeroes).  The reference ADDS
  beta * prior in the _R update, so a smoothing prior takes beta < 0.

``OSSART`` / ``ossart_reconstruct`` are the device-resident loop the
reference leaves empty (``Recon_Method`` 3, ``Tomo_OSTR_gold.cpp:1523``):
two fused kernels per sub-iteration over a caller-owned workspace.
"""
from __future__ import annotations

import ctypes

import torch

from . import native
from .geometry import Geometry, NrSartParams
from .ostr import _Out, _device, _geom_c, _in, _like_input, _p, _stream


def _fp_sart(estbuf, prj_est, d_normprj, d_angles, d_index, angleStart, angleEnd, use_cos):
    gp, g = _geom_c()
    x = _in(estbuf)
    est = _Out(prj_est)
    norm = _Out(d_normprj)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_fp_sart", gp, _p(x), est.ptr(), norm.ptr(), _p(ang), _p(idx),
                int(angleStart), int(angleEnd), int(use_cos), _stream())
    est.done()
    norm.done()


def fprojectCB_1R_GPU_SART(estbuf, prj_est, d_normprj, d_angles, d_index, angleStart, angleEnd):
    """prj_est = line integral, d_normprj = chord, views [angleStart, angleEnd) (Tomo_OSTR.cu:2278)."""
    _fp_sart(estbuf, prj_est, d_normprj, d_angles, d_index, angleStart, angleEnd, 0)


def fprojectCB_1R_GPU_SART_cos(estbuf, prj_est, d_normprj, d_angles, d_index, angleStart,
                               angleEnd):
    """As fprojectCB_1R_GPU_SART with prj_est times cos(theta) (Tomo_OSTR.cu:2306)."""
    _fp_sart(estbuf, prj_est, d_normprj, d_angles, d_index, angleStart, angleEnd, 1)


def fprojectCB1_4R_GPU_SART(d_objbuf, d_prjbuf, d_4R_prjbuf, d_angles, d_index, angleStart,
                            angleEnd):
    """d_prjbuf = mean of the 2 x 2 sub-ray line integrals per bin, [view][j][i] as the
    reference's merge writes it; d_4R_prjbuf (may be None) gets the sub-ray sums
    [view][2 BINSy][2 BINSx].  The fixed Tomo_OSTR.cu:2398 (see nr_fp_4r)."""
    gp, g = _geom_c()
    x = _in(d_objbuf)
    out = _Out(d_prjbuf)
    sub = None if d_4R_prjbuf is None else _Out(d_4R_prjbuf)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_fp_4r", gp, _p(x), out.ptr(), None if sub is None else sub.ptr(), _p(ang),
                _p(idx), int(angleStart), int(angleEnd), 0, 1, _stream())
    out.done()
    if sub is not None:
        sub.done()


def fproject_4R(estbuf, prj_est, d_angles, d_index, angleStart, angleEnd, use_cos=False,
                layout="ij"):
    """The 4R projector in either layout ("ij": [view][i][j] like the 1R projectors,
    "ji": [view][j][i]) and optionally times cos(theta)."""
    gp, g = _geom_c()
    x = _in(estbuf)
    out = _Out(prj_est)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_fp_4r", gp, _p(x), out.ptr(), None, _p(ang), _p(idx), int(angleStart),
                int(angleEnd), int(bool(use_cos)), {"ij": 0, "ji": 1}[layout], _stream())
    out.done()


def SART_prj_diff(diff_line, prjbuf, prj_est, normprj, d_index, angleStart, angleEnd):
    """diff_line = (prjbuf - prj_est) / normprj over the view range (Tomo_OSTR.cu:2537)."""
    from .ostr import BINSx, BINSy
    n = (int(angleEnd) - int(angleStart)) * int(BINSx) * int(BINSy)
    out = _Out(diff_line)
    prj, est, norm = _in(prjbuf), _in(prj_est), _in(normprj)
    if min(prj.numel(), est.numel(), norm.numel(), out.t.numel()) < n:
        raise ValueError("SART_prj_diff: buffers shorter than the view range")
    native.call("nr_sart_prj_diff", out.ptr(), _p(prj), _p(est), _p(norm), n, _stream())
    out.done()


def _bp_ossart(d_objbuf, d_prjbuf, d_prior, d_index, d_angles, angleStart, angleEnd, lam, beta):
    gp, g = _geom_c()
    x = _Out(d_objbuf)
    prj = _in(d_prjbuf)
    prior = None if d_prior is None else _in(d_prior)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_bp_ossart", gp, x.ptr(), _p(prj), _p(prior), _p(idx), _p(ang),
                int(angleStart), int(angleEnd), float(lam), float(beta), _stream())
    x.done()


def bprojectCB_4B_GPU_SART(d_objbuf, d_prjbuf, d_index, d_angles, angleStart, angleEnd, lambda_):
    """In-place OS-SART update from the difference d_prjbuf (Tomo_OSTR.cu:2460)."""
    _bp_ossart(d_objbuf, d_prjbuf, None, d_index, d_angles, angleStart, angleEnd, lambda_, 0.0)


def bprojectCB_4B_GPU_SART_R(d_objbuf, d_prjbuf, d_prior, d_index, d_angles, angleStart,
                             angleEnd, lambda_, beta):
    """As bprojectCB_4B_GPU_SART plus lambda beta prior / sensitivity (Tomo_OSTR.cu:2497)."""
    _bp_ossart(d_objbuf, d_prjbuf, d_prior, d_index, d_angles, angleStart, angleEnd, lambda_,
               beta)


def prior_GPU_SART(d_prior, d_est, delta):
    """d_prior += hyperbola gradient of d_est (Tomo_OSTR.cu:2249).  delta == 0 raises."""
    if delta == 0:
        raise ValueError("delta cannot be ZERO")  # Tomo_OSTR.cu:2260-2263
    gp, g = _geom_c()
    out = _Out(d_prior)
    x = _in(d_est)
    native.call("nr_prior_sart", gp, out.ptr(), _p(x), float(delta), _stream())
    out.done()


def line_integrals(prj, blank, scat=None):
    """log(blank / (prj - scat)) where both are positive, else 0 (SART input from counts)."""
    y = _in(prj)
    b = _in(blank)
    s = None if scat is None else _in(scat)
    out = torch.empty_like(y)
    native.call("nr_sart_line_integrals", _p(out), _p(y), _p(b), _p(s), int(y.numel()),
                _stream())
    return _like_input(prj, out)


SECTIONS = {"line": 0, "norm": 1, "diff": 2, "index": 3}


class OSSART:
    """The OS-SART loop on the GPU, over a caller-owned workspace.

    >>> plan = OSSART(geom, subset_num=5, lam=0.8)
    >>> plan.setup(angles, line)        # line integrals [view][i][j], original order
    >>> plan.iterate(x, 10)             # x [z][y][x] in place on the device
    """

    def __init__(self, geom: Geometry, *, subset_num: int, lam: float, use_cos: bool = True,
                 regularized: bool = False, beta: float = 0.0, delta: float = 1.0,
                 fp_batch: int = 0, upd_planes: int = 0, supersample: bool = False):
        geom.validate(subset_num)
        self.geom = geom
        self.params = NrSartParams(int(subset_num), int(bool(use_cos)), int(bool(regularized)),
                                   int(fp_batch), int(upd_planes), float(lam), float(beta),
                                   float(delta), int(bool(supersample)))
        self.gc = geom.to_c()
        size = ctypes.c_size_t(0)
        native.call("nr_sart_workspace_size", ctypes.byref(self.gc), ctypes.byref(self.params),
                    ctypes.byref(size))
        self.ws_bytes = int(size.value)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=_device())

    def _ws(self):
        return ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_size_t(self.ws_bytes)

    def setup(self, angles, line) -> None:
        ang = _in(angles)
        ln = _in(line)
        if ln.numel() != self.geom.n_angles * self.geom.n_bins:
            raise ValueError("line must hold n_angles x BINSx x BINSy values")
        ws, n = self._ws()
        native.call("nr_sart_setup", ctypes.byref(self.gc), ctypes.byref(self.params), _p(ang),
                    _p(ln), ws, n, _stream())
        self._keep = (ang, ln)

    def iterate(self, x: torch.Tensor, n_iters: int) -> torch.Tensor:
        ws, n = self._ws()
        native.call("nr_sart_iterate", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    int(n_iters), ws, n, _stream())
        return x

    def project(self, x: torch.Tensor, subset: int) -> None:
        """First half of a sub-iteration: the subset's normalised difference."""
        ws, n = self._ws()
        native.call("nr_sart_project", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    int(subset), ws, n, _stream())

    def update(self, x: torch.Tensor, x_out: torch.Tensor, subset: int) -> None:
        """Second half: x_out = the OS-SART update of x (x_out is not x)."""
        ws, n = self._ws()
        native.call("nr_sart_update", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    _p(x_out), int(subset), ws, n, _stream())

    def subiter(self, x: torch.Tensor, subset: int) -> torch.Tensor:
        ws, n = self._ws()
        native.call("nr_sart_subiter", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    int(subset), ws, n, _stream())
        return x

    def section(self, name: str) -> torch.Tensor:
        ws, n = self._ws()
        ptr = ctypes.c_void_p(0)
        size = ctypes.c_size_t(0)
        native.call("nr_sart_workspace_section", ctypes.byref(self.gc), ctypes.byref(self.params),
                    SECTIONS[name], ws, n, ctypes.byref(ptr), ctypes.byref(size))
        off = int(ptr.value) - self.ws.data_ptr()
        dt = torch.int32 if name == "index" else torch.float32
        return self.ws[off:off + int(size.value)].view(dt)

    def graph(self, x: torch.Tensor, n_iters: int) -> "SartGraph":
        return SartGraph(self, x, n_iters)

    def check(self) -> int:
        """Raises NrError if a kernel flagged NaN/Inf; returns the flags."""
        ws, n = self._ws()
        flags = ctypes.c_int32(0)
        native.call("nr_ostr_check", ws, n, ctypes.byref(flags), _stream())
        return int(flags.value)


class SartGraph:
    """A captured OS-SART loop: x and the plan's workspace are fixed; each
    launch() runs the iterations again on the current x."""

    def __init__(self, plan: OSSART, x: torch.Tensor, n_iters: int):
        self.plan = plan
        self.x = x
        self.n_iters = int(n_iters)
        self.handle = ctypes.c_void_p(0)
        self._stream = torch.cuda.Stream()
        self._stream.wait_stream(torch.cuda.current_stream())
        ws, n = plan._ws()
        native.call("nr_sart_graph_create", ctypes.byref(plan.gc), ctypes.byref(plan.params),
                    _p(x), self.n_iters, ws, n, ctypes.c_void_p(self._stream.cuda_stream),
                    ctypes.byref(self.handle))

    def launch(self) -> None:
        native.call("nr_ostr_graph_launch", self.handle, _stream())

    def close(self) -> None:
        if self.handle and self.handle.value:
            torch.cuda.synchronize()
            native.call("nr_ostr_graph_destroy", self.handle)
            self.handle = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ossart_reconstruct(geom: Geometry, line, *, angles, subset_num: int, iter_num: int,
                       lam: float, use_cos: bool = True, regularized: bool = False,
                       beta: float = 0.0, delta: float = 1.0, supersample: bool = False,
                       x0=None):
    """OS-SART: line integrals [view][i][j] (original order) in, attenuation out.

    Returns the volume [z][y][x]; numpy when line was a host array, else a
    CUDA tensor.
    """
    plan = OSSART(geom, subset_num=subset_num, lam=lam, use_cos=use_cos,
                  regularized=regularized, beta=beta, delta=delta, supersample=supersample)
    plan.setup(angles, line)
    if x0 is None:
        x = torch.zeros(geom.n_voxels, dtype=torch.float32, device=plan.ws.device)
    else:
        x = _in(x0).clone()
    plan.iterate(x, iter_num)
    plan.check()
    return _like_input(line, x)
