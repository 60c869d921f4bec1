"""Drop-in OSTR call surface of the reference's ``ostr.py`` / ``ostr.ipynb``,
backed by the sm_103a kernels of libnrgb300.

Same names, argument order and semantics as the reference:

* geometry, beta/delta, ``iter_num``/``subset_num`` are module-level names
  (``ostr.py:21-75``); every call reads them when it runs;
* ``fprojectCB_1R_GPU_OSTR_cos``, ``fprojectCB_1R_GPU_OSTR_normprj``,
  ``bprojectCB_GPU_SBP``, ``prior_GPU_OSTR`` (Lange) and ``prior_GPU_OSTR_Q2``
  work on device arrays in place: the projectors leave missed rays untouched,
  the back projector and the priors ACCUMULATE (the caller zeroes);
* ``compute_yry``, ``compute_gamma_yry``, ``compute_h``, ``update_est``,
  ``regroup_prj``, ``x_y_flip``, ``temp_fun1``, ``temp_fun2`` return new arrays
  like the reference's Numba helpers, computed on the GPU;
* ``load_prj_std`` / ``load_prj`` read the per-view raw float32 files.

Device arrays may be torch CUDA tensors or any object exposing
``__cuda_array_interface__`` (e.g. Numba device arrays).  Host numpy arrays
are copied to the device, processed there and returned as numpy.

``reconstruct(...)`` and ``OSTR`` are the device-resident path: the whole
subset loop stays on the GPU with the fused kernels.
"""
from __future__ import annotations

import ctypes
import os
import time
from typing import Optional, Tuple

import numpy as np
import torch

from . import native
from .geometry import GAMMA_MODES, POTENTIALS, Geometry, NrBatchCase, NrOstrParams

# ---------------------------------------------------------------------------
# Module-level configuration, as in the reference (ostr.py:21-75).  Values are
# the reference's own defaults.
IMGSIZx = 2000
IMGSIZy = 1000
IMGSIZz = 48
BINSx = 3584
BINSy = 1400
Vsize_x = 0.085
Vsize_y = 0.085
Vsize_z = 1
x_p0 = -93.5
y_p0 = -85.0
z_p0 = -30.0
x_d0 = -152.32
y_d0 = -119
Bsize_x = 0.085
Bsize_y = 0.085
ANGLES = 25
index: list = []
angles: list = []
detectorR = 47.0
sourceR = 608.5
sourceY = 0.0
beta = 150000
delta = 0.003
iter_num = 15
subset_num = 5
IO_Iter = 0
method = 0
basepath = ""
filepath = ""
projection_name = "OSTR_HE.3584x1400."
scatter_name = "OSTR_scatter.3584x1400."
blank_name = "OSTR_blank.3584x1400."
# gamma definition of fprojectCB_1R_GPU_OSTR_normprj: "length" (|src - bin|,
# Tomo_OSTR.cu:1172) or "chord" (in-volume chord, ostr.py:641).
gamma_mode = "length"

_GEOM_NAMES = ("IMGSIZx", "IMGSIZy", "IMGSIZz", "Vsize_x", "Vsize_y", "Vsize_z", "x_p0", "y_p0",
               "z_p0", "BINSx", "BINSy", "Bsize_x", "Bsize_y", "x_d0", "y_d0", "detectorR",
               "sourceR", "sourceY", "ANGLES")


def current_geometry() -> Geometry:
    """The module-level geometry as a Geometry."""
    m = globals()
    return Geometry(nx=int(m["IMGSIZx"]), ny=int(m["IMGSIZy"]), nz=int(m["IMGSIZz"]),
                    vx=float(m["Vsize_x"]), vy=float(m["Vsize_y"]), vz=float(m["Vsize_z"]),
                    x_p0=float(m["x_p0"]), y_p0=float(m["y_p0"]), z_p0=float(m["z_p0"]),
                    nbx=int(m["BINSx"]), nby=int(m["BINSy"]), bx=float(m["Bsize_x"]),
                    by=float(m["Bsize_y"]), x_d0=float(m["x_d0"]), y_d0=float(m["y_d0"]),
                    detectorR=float(m["detectorR"]), sourceR=float(m["sourceR"]),
                    sourceY=float(m["sourceY"]), n_angles=int(m["ANGLES"]))


def set_geometry(g: Geometry) -> None:
    """Sets the module-level geometry names from a Geometry."""
    m = globals()
    m.update(IMGSIZx=g.nx, IMGSIZy=g.ny, IMGSIZz=g.nz, Vsize_x=g.vx, Vsize_y=g.vy, Vsize_z=g.vz,
             x_p0=g.x_p0, y_p0=g.y_p0, z_p0=g.z_p0, BINSx=g.nbx, BINSy=g.nby, Bsize_x=g.bx,
             Bsize_y=g.by, x_d0=g.x_d0, y_d0=g.y_d0, detectorR=g.detectorR, sourceR=g.sourceR,
             sourceY=g.sourceY, ANGLES=g.n_angles)


# ---------------------------------------------------------------------------
# Device buffer plumbing.

def _device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("newrecon_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _as_tensor(a, dtype=torch.float32) -> Tuple[torch.Tensor, bool]:
    """(CUDA contiguous tensor of dtype, aliases_input)."""
    dev = _device()
    if isinstance(a, torch.Tensor):
        t = a
    elif hasattr(a, "__cuda_array_interface__"):
        t = torch.as_tensor(a, device=dev)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a)))
    alias = t.is_cuda and t.dtype == dtype and t.is_contiguous()
    if not alias:
        t = t.to(device=dev, dtype=dtype).contiguous()
    return t, alias


class _Out:
    """A caller's output buffer seen as a float32 CUDA tensor; write back on exit."""

    def __init__(self, a):
        self.orig = a
        self.t, self.alias = _as_tensor(a)

    def ptr(self):
        return ctypes.c_void_p(self.t.data_ptr())

    def done(self):
        if self.alias:
            return
        if isinstance(self.orig, torch.Tensor):
            self.orig.copy_(self.t.view(self.orig.shape).to(self.orig.dtype))
        elif hasattr(self.orig, "__cuda_array_interface__"):
            dst = torch.as_tensor(self.orig, device=self.t.device)
            dst.copy_(self.t.view(dst.shape).to(dst.dtype))
        else:
            np.copyto(np.asarray(self.orig), self.t.view(np.shape(self.orig)).cpu().numpy(),
                      casting="unsafe")


def _in(a, dtype=torch.float32) -> torch.Tensor:
    return _as_tensor(a, dtype)[0]


def _p(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _like_input(ref, t: torch.Tensor):
    """t in the kind of the caller's input: numpy for numpy, a host tensor for
    a host tensor (pinned for a pinned input: the download then runs at the
    link's rate instead of through a pageable bounce, 0.8 ms instead of 8-17 ms
    for a 126 MB volume), the device tensor otherwise."""
    if isinstance(ref, torch.Tensor):
        if ref.is_cuda:
            return t
        if ref.is_pinned():
            out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
            out.copy_(t, non_blocking=True)
            torch.cuda.current_stream(t.device).synchronize()
            return out
        return t.cpu()
    if hasattr(ref, "__cuda_array_interface__"):
        return t
    return t.cpu().numpy()


def _geom_c(g: Optional[Geometry] = None):
    g = current_geometry() if g is None else g
    return ctypes.byref(g.to_c()), g


# ---------------------------------------------------------------------------
# Launch wrappers (Tomo_OSTR.cu:2189-2457; ostr.ipynb:1064,1175,1244; ostr.py:654).

def fprojectCB_1R_GPU_OSTR_cos(estbuf, prj_est, d_angles, d_index, angleStart, angleEnd):
    """prj_est[(a-angleStart)] = cos(theta) * line integral of estbuf, a in [angleStart, angleEnd)."""
    gp, g = _geom_c()
    x = _in(estbuf)
    out = _Out(prj_est)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_fp_ostr", gp, _p(x), out.ptr(), _p(ang), _p(idx), int(angleStart),
                int(angleEnd), _stream())
    out.done()


def fprojectCB_1R_GPU_OSTR_normprj(d_normprj, d_angles, d_index, angleStart, angleEnd):
    """gamma of the views in [angleStart, angleEnd); see module name ``gamma_mode``."""
    gp, g = _geom_c()
    out = _Out(d_normprj)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_fp_gamma", gp, out.ptr(), _p(ang), _p(idx), int(angleStart), int(angleEnd),
                int(GAMMA_MODES[gamma_mode]), _stream())
    out.done()


def bprojectCB_GPU_SBP(d_objbuf, d_prjbuf, d_index, d_angles, angleStart, angleEnd):
    """d_objbuf += SBP of d_prjbuf over views [angleStart, angleEnd)."""
    gp, g = _geom_c()
    out = _Out(d_objbuf)
    prj = _in(d_prjbuf)
    ang = _in(d_angles)
    idx = _in(d_index, torch.int32)
    native.call("nr_bp_sbp", gp, out.ptr(), _p(prj), _p(idx), _p(ang), int(angleStart),
                int(angleEnd), _stream())
    out.done()


def _prior(d_RDD, d_RD, d_est, pot: str, dl: float, z_xy_ratio: float):
    gp, g = _geom_c()
    rdd = _Out(d_RDD)
    rd = _Out(d_RD)
    x = _in(d_est)
    native.call("nr_prior", gp, rdd.ptr(), rd.ptr(), _p(x), int(POTENTIALS[pot]), float(dl),
                float(z_xy_ratio), _stream())
    rdd.done()
    rd.done()


def prior_GPU_OSTR(d_RDD, d_RD, d_est, delta, z_xy_ratio):
    """Lange prior: RDD, RD += (Tomo_OSTR.cu:2216-2245).  delta == 0 raises."""
    if delta == 0:
        raise ValueError("delta cannot be ZERO")  # Tomo_OSTR.cu:2232-2236
    _prior(d_RDD, d_RD, d_est, "lange", delta, z_xy_ratio)


def prior_GPU_OSTR_Q2(d_RDD, d_RD, d_est, z_xy_ratio):
    """Quadratic prior: RDD, RD += (Tomo_OSTR.cu:2189-2213)."""
    _prior(d_RDD, d_RD, d_est, "q2", 1.0, z_xy_ratio)


def prior_GPU_OSTR_potential(d_RDD, d_RD, d_est, potential, delta, z_xy_ratio):
    """Any potential ("q2", "lange", "hyperbola", "huber"): RDD, RD +=."""
    if potential != "q2" and not delta > 0:
        raise ValueError("delta must be positive")
    _prior(d_RDD, d_RD, d_est, potential, delta if potential != "q2" else 1.0, z_xy_ratio)


# ---------------------------------------------------------------------------
# Host helpers of the reference (Tomo_OSTR_gold.cpp:93-295; ostr.py:153-213;
# ostr.ipynb:348-374,1185-1193), on the GPU.

def compute_yry(host_prj_allangle, host_scat_allangle):
    y = _in(host_prj_allangle)
    s = None if host_scat_allangle is None else _in(host_scat_allangle)
    out = torch.empty_like(y)
    native.call("nr_compute_yry", _p(out), _p(y), _p(s), int(y.numel()), _stream())
    return _like_input(host_prj_allangle, out)


def compute_gamma_yry(host_yry_allangle, host_gamma_allangle):
    a = _in(host_yry_allangle)
    b = _in(host_gamma_allangle)
    out = torch.empty_like(a)
    native.call("nr_compute_gamma_yry", _p(out), _p(a), _p(b), int(a.numel()), _stream())
    return _like_input(host_yry_allangle, out)


def compute_h(host_prj_sub, host_blank_sub, host_line_sub, host_scat_sub):
    y = _in(host_prj_sub)
    b = _in(host_blank_sub)
    line = _in(host_line_sub)
    s = None if host_scat_sub is None else _in(host_scat_sub)
    out = torch.empty_like(y)
    native.call("nr_compute_h", _p(out), _p(y), _p(b), _p(line), _p(s), int(y.numel()), _stream())
    return _like_input(host_prj_sub, out)


def update_est(host_est, host_capL, host_RD, host_d, host_RDD):
    """Returns max(0, est - (capL + beta RD)/(d + 2 beta RDD)) (module ``beta``)."""
    est = _in(host_est).clone()
    # keep every input tensor alive across the (asynchronous) launch
    capL, RD, d, RDD = _in(host_capL), _in(host_RD), _in(host_d), _in(host_RDD)
    native.call("nr_update_est", _p(est), _p(capL), _p(RD), _p(d), _p(RDD), float(beta),
                int(est.numel()), _stream())
    return _like_input(host_est, est)


def regroup_prj(host_uponregroup_allangle):
    a = _in(host_uponregroup_allangle)
    out = torch.empty_like(a)
    A = int(ANGLES)
    native.call("nr_regroup", _p(out), _p(a), A, int(subset_num), int(a.numel() // A), _stream())
    return _like_input(host_uponregroup_allangle, out)


def x_y_flip(host_prjbuf_temp):
    """One view (or several, back to back) from file layout [j][i] to [i][j]."""
    a = _in(host_prjbuf_temp)
    nb = int(BINSx) * int(BINSy)
    out = torch.empty_like(a)
    native.call("nr_x_y_flip", _p(out), _p(a), int(BINSx), int(BINSy), int(a.numel() // nb),
                _stream())
    return _like_input(host_prjbuf_temp, out)


def temp_fun1(angleStart, b_size, sub_b_size, host_prj_allangle):
    """The subset slice of an all-view array (ostr.ipynb:1185)."""
    a = host_prj_allangle
    lo = int(angleStart) * int(b_size)
    sl = a[lo:lo + int(sub_b_size)]
    if isinstance(sl, torch.Tensor):
        return sl.clone()
    return np.array(sl, copy=True)


def temp_fun2(subset_num_, f_size, host_capL):
    """subset_num * capL (ostr.ipynb:1193; Tomo_OSTR_gold.cpp:767-771)."""
    c = _in(host_capL).clone()
    native.call("nr_scale", _p(c), float(subset_num_), int(min(int(f_size), c.numel())), _stream())
    return _like_input(host_capL, c)


def import_param():
    """Identity view index (Tomo_OSTR_gold.cpp:1474-1488)."""
    return np.arange(int(ANGLES), dtype=np.int32)


def load_prj_std(data_type):
    """All views of prelog (0), scatter (1) or blank (2) data, [view][i][j] (ostr.py:111-151)."""
    sub = {0: ("OSTR_prelog/", projection_name), 1: ("OSTR_scatter/", scatter_name)}.get(
        int(data_type), ("OSTR_blank/", blank_name))
    b = int(BINSx) * int(BINSy)
    views = []
    for v in range(int(ANGLES)):
        fn = os.path.join(basepath, sub[0] + sub[1] + str(v + 1).zfill(4))
        views.append(np.fromfile(fn, dtype=np.float32)[:b])
    return x_y_flip(np.concatenate(views))


def load_prj():
    """Prelog + scatter stored back to back per view file (ostr.py:93-109)."""
    b = int(BINSx) * int(BINSy)
    prj, sct = [], []
    for v in range(int(ANGLES)):
        fn = basepath + filepath + str(v + 1).zfill(4) + ".raw"
        d = np.fromfile(fn, dtype=np.float32)
        prj.append(d[:b])
        sct.append(d[b:2 * b])
    return x_y_flip(np.concatenate(prj)), x_y_flip(np.concatenate(sct))


# ---------------------------------------------------------------------------
# Device-resident OSTR.

class OSTR:
    """The whole OSTR loop on the GPU, over a caller-owned workspace.

    >>> plan = OSTR(geom, subset_num=25, beta=100, delta=0.003, potential="huber")
    >>> plan.setup(angles, prj, blank)          # [view][i][j], original view order
    >>> x = plan.iterate(x0, 50)                # [z][y][x], in place on device
    """

    def __init__(self, geom: Geometry, *, subset_num: int, beta: float, delta: float,
                 potential: str = "lange", gamma_mode: str = "length", has_scatter: bool = False,
                 stage: bool = False, upd_tile: int = 0):
        """stage=True stages the projection's volume slab by slab in shared
        memory by TMA instead of gathering it through L1/L2 (same result;
        slower on the clinical workload).  upd_tile=1 gives each thread of the
        update two voxels side by side in x (one-view subsets); upd_tile=2
        streams the update's planes by TMA through a shared-memory ring filled
        by a producer warp (where IMGSIZx is a multiple of 4).  Every variant
        gives the same result bit for bit.  autotune() picks them per geometry."""
        if upd_tile not in (0, 1, 2):
            raise ValueError("upd_tile must be 0 (one voxel per thread), 1 (two) or 2 (TMA ring)")
        geom.validate(subset_num)
        self.geom = geom
        self.params = NrOstrParams(int(subset_num), int(POTENTIALS[potential]),
                                   int(GAMMA_MODES[gamma_mode]), int(bool(has_scatter)),
                                   float(beta), float(delta if potential != "q2" else 1.0))
        self.params.fp_stage = 1 if stage else 0
        self.params.upd_tile = int(upd_tile)
        self.gc = geom.to_c()
        self.history = None      # objectives of a monotone iterate()
        self.rejected_at = None  # the iteration a monotone iterate() undid
        self.subset_history = None  # per sub-iteration record of monotone="subset"
        self.rejected_steps = 0
        size = ctypes.c_size_t(0)
        native.call("nr_ostr_workspace_size", ctypes.byref(self.gc), ctypes.byref(self.params),
                    ctypes.byref(size))
        self.ws_bytes = int(size.value)
        # one byte tensor; the CUDA caching allocator returns 512-byte aligned blocks
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=_device())
        self.objective_out = torch.zeros(2, dtype=torch.float64, device=self.ws.device)

    def _ws(self):
        return ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_size_t(self.ws_bytes)

    def setup(self, angles, prj, blank, scat=None) -> None:
        ang = _in(angles)
        y = _in(prj)
        b = _in(blank)
        s = None if scat is None else _in(scat)
        if (s is None) != (self.params.has_scatter == 0):
            raise ValueError("scatter given does not match has_scatter")
        ws, n = self._ws()
        native.call("nr_ostr_setup", ctypes.byref(self.gc), ctypes.byref(self.params), _p(ang),
                    _p(y), _p(b), _p(s), ws, n, _stream())
        self._keep = (ang, y, b, s)

    def iterate(self, x: torch.Tensor, n_iters: int, monotone=False,
                check_every: int = 1) -> torch.Tensor:
        """n_iters iterations (every subset once each) on x in place.

        monotone=True accepts an iteration only if it does not raise the FP64
        penalized-likelihood objective (ordered subsets do not guarantee a
        monotone decrease near convergence): the first iteration that would
        raise it, or make it NaN, is undone and the loop stops there.
        ``history`` then holds the objectives of the accepted iterates (the
        start included) and ``rejected_at`` the rejected iteration, or None.
        Each check costs one objective evaluation (a projection of all views
        and the penalty).  check_every=k checks after every k-th iteration
        only (and after the last): a checkpoint whose objective rose, or is
        NaN, is undone back to the previous accepted checkpoint and the loop
        stops there, so the objective decreases from checkpoint to checkpoint
        and the checks cost 1/k as much; ``rejected_at`` is then the first
        iteration of the undone block.

        monotone="subset" decides every sub-iteration instead: the step of
        subset a from x to x' is kept only if it does not raise the FP64
        subset objective M L_a + beta R (L_a the data term of subset a's
        views, M the subset count, R the penalty); otherwise x stays and the
        loop goes on with the next subset.  L_a(x) comes from the projection
        that makes the step's gradient (nr_ostr_project_fp64); each check adds
        the projection of the subset's views at x' and one penalty
        evaluation.  ``subset_history`` holds (iteration, subset, before,
        after, kept) per sub-iteration and ``rejected_steps`` the count of
        steps not kept."""
        if monotone == "subset":
            return self._iterate_subset_monotone(x, n_iters)
        if monotone not in (False, True):
            raise ValueError('monotone must be False, True or "subset"')
        ws, n = self._ws()
        if not monotone:
            native.call("nr_ostr_iterate", ctypes.byref(self.gc), ctypes.byref(self.params),
                        _p(x), int(n_iters), ws, n, _stream())
            return x
        if int(check_every) < 1:
            raise ValueError("check_every must be at least 1")
        prev = torch.empty_like(x)
        hist = [self.total_objective(x)]
        self.rejected_at = None
        k = 0
        while k < int(n_iters):
            block = min(int(check_every), int(n_iters) - k)
            prev.copy_(x)
            native.call("nr_ostr_iterate", ctypes.byref(self.gc), ctypes.byref(self.params),
                        _p(x), block, ws, n, _stream())
            f = self.total_objective(x)
            if not f <= hist[-1]:
                x.copy_(prev)
                self.rejected_at = k
                break
            hist.append(f)
            k += block
        self.history = hist
        return x

    def _iterate_subset_monotone(self, x: torch.Tensor, n_iters: int) -> torch.Tensor:
        M = int(self.params.subset_num)
        beta = float(self.params.beta)
        xn = torch.empty_like(x)
        vals = torch.zeros(3, dtype=torch.float64, device=x.device)
        self.penalty(x, vals[2:3])
        pen_x = float(vals[2].item())
        log = []
        for k in range(int(n_iters)):
            for a in range(M):
                self.project_fp64(x, a, vals[0:1])      # h and L_a(x)
                self.update(x, xn, a)
                self.project_fp64(xn, a, vals[1:2])     # L_a(x')
                self.penalty(xn, vals[2:3])             # R(x')
                before_data, after_data, pen_new = (float(v) for v in vals.cpu())
                before, after = self._subset_values(M * before_data + beta * pen_x,
                                                    M * after_data + beta * pen_new)
                kept = after <= before
                if kept:
                    x.copy_(xn)
                    pen_x = pen_new
                log.append((k, a, before, after, kept))
        self.subset_history = log
        self.rejected_steps = sum(1 for e in log if not e[4])
        return x

    @staticmethod
    def _subset_values(before: float, after: float) -> Tuple[float, float]:
        """The subset objectives a monotone="subset" step is judged by (a seam
        for tests that plant a rising step on the host)."""
        return before, after

    def project_fp64(self, x: torch.Tensor, subset: int,
                     out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Fused FP + h of one subset into the workspace, as project(), and the
        subset's FP64 data term into out (one device double; returned)."""
        if out is None:
            out = torch.zeros(1, dtype=torch.float64, device=x.device)
        ws, n = self._ws()
        native.call("nr_ostr_project_fp64", ctypes.byref(self.gc), ctypes.byref(self.params),
                    _p(x), int(subset), _p(out), ws, n, _stream())
        return out

    def penalty(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """The FP64 penalty R(x) (objective()'s second part) into out (one
        device double; returned)."""
        if out is None:
            out = torch.zeros(1, dtype=torch.float64, device=x.device)
        ws, n = self._ws()
        native.call("nr_ostr_penalty", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    _p(out), ws, n, _stream())
        return out

    def subiter(self, x: torch.Tensor, subset: int) -> torch.Tensor:
        ws, n = self._ws()
        native.call("nr_ostr_subiter", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    int(subset), ws, n, _stream())
        return x

    def project(self, x: torch.Tensor, subset: int) -> None:
        """Fused FP + h of one subset into the workspace."""
        ws, n = self._ws()
        native.call("nr_ostr_project", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    int(subset), ws, n, _stream())

    def update(self, x: torch.Tensor, x_out: torch.Tensor, subset: int) -> None:
        """Fused SBP + penalty + update of one subset: x_out from x."""
        ws, n = self._ws()
        native.call("nr_ostr_update", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    _p(x_out), int(subset), ws, n, _stream())

    SECTIONS = {"d": (0, torch.float32), "h": (1, torch.float32), "y": (2, torch.float32),
                "gamma_yry": (3, torch.float32), "index": (4, torch.int32)}

    def section(self, name: str) -> torch.Tensor:
        """A view of a workspace section ("d", "h", "y", "gamma_yry", "index")."""
        code, dt = self.SECTIONS[name]
        ws, n = self._ws()
        ptr = ctypes.c_void_p(0)
        nb = ctypes.c_size_t(0)
        native.call("nr_ostr_workspace_section", ctypes.byref(self.gc),
                    ctypes.byref(self.params), int(code), ws, n, ctypes.byref(ptr),
                    ctypes.byref(nb))
        off = int(ptr.value) - self.ws.data_ptr()
        return self.ws[off:off + int(nb.value)].view(dt)

    def autotune(self, x: Optional[torch.Tensor] = None, use_cache: bool = True) -> dict:
        """Picks the fused kernels' variants for this geometry (newrecon_gb300.autotune)."""
        from . import autotune

        k, z, rec = autotune.tune(self, x, use_cache=use_cache)
        return rec

    def graph(self, x: torch.Tensor, n_iters: int) -> "OstrGraph":
        """n_iters iterations on x captured once as a CUDA graph; replay with .launch()."""
        return OstrGraph(self, x, n_iters)

    def objective(self, x: torch.Tensor) -> Tuple[float, float]:
        """(data term, penalty) in FP64; total = data + beta * penalty."""
        ws, n = self._ws()
        native.call("nr_ostr_objective", ctypes.byref(self.gc), ctypes.byref(self.params), _p(x),
                    _p(self.objective_out), ws, n, _stream())
        v = self.objective_out.cpu()
        return float(v[0]), float(v[1])

    def total_objective(self, x: torch.Tensor) -> float:
        d, p = self.objective(x)
        return d + self.params.beta * p

    def check(self) -> int:
        """Raises NrError if a kernel flagged NaN/Inf or a timeout; returns the flags."""
        ws, n = self._ws()
        flags = ctypes.c_int32(0)
        native.call("nr_ostr_check", ws, n, ctypes.byref(flags), _stream())
        return int(flags.value)


class OstrGraph:
    """A captured iteration loop (nr_ostr_graph_*): x and the plan's workspace
    are fixed; each launch() runs the iterations again on the current x."""

    def __init__(self, plan: OSTR, x: torch.Tensor, n_iters: int):
        self.plan = plan
        self.x = x
        self.n_iters = int(n_iters)
        self.handle = ctypes.c_void_p(0)
        self._stream = torch.cuda.Stream()
        self._stream.wait_stream(torch.cuda.current_stream())
        ws, n = plan._ws()
        native.call("nr_ostr_graph_create", ctypes.byref(plan.gc), ctypes.byref(plan.params),
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


class Batch:
    """Many independent reconstructions advanced together by shared batched
    launches (nr_batch_*: one launch per kernel covers every case's work
    items): each case has its own geometry, view count, potential and
    iteration count.

    >>> b = Batch([dict(geom=g1, angles=a1, prj=y1, blank=b1, subset_num=9, iter_num=50,
    ...                 beta=50, delta=0.002, potential="hyperbola"), ...])
    >>> volumes = b.run()            # or: gr = b.graph(); gr.launch()

    tune=True runs the autotuner on each case's plan first (cached per
    geometry): the batched update then walks each case with its tuned slab
    depth and tile.  The batched projection always uses 4-step gathers.

    mode: "shared" advances all cases by the shared launches; "sequential"
    runs the cases one after another through their own iteration loops (a
    case of 2^26 voxels or more fills the GPU alone, and interleaving such
    cases only widens the working set: 0.96x at 2048 x 1024 x 70, against
    1.03x for shared launches over cases of 8-30 M voxels); "auto" picks
    "sequential" when every case has at least SEQUENTIAL_VOXELS voxels.  Both
    modes give the same volumes bit for bit.
    """

    SEQUENTIAL_VOXELS = 1 << 26

    @staticmethod
    def choose_mode(voxel_counts, mode: str = "auto") -> str:
        if mode not in ("auto", "shared", "sequential"):
            raise ValueError('mode must be "auto", "shared" or "sequential"')
        if mode != "auto":
            return mode
        return ("sequential" if min(voxel_counts) >= Batch.SEQUENTIAL_VOXELS else "shared")

    def __init__(self, cases, tune: bool = False, mode: str = "auto"):
        if not 1 <= len(cases) <= 64:
            raise ValueError("a batch holds 1 to 64 cases")
        self.mode = Batch.choose_mode([c["geom"].n_voxels for c in cases], mode)
        self.iters = [int(c["iter_num"]) for c in cases]
        self.plans, self.x = [], []
        arr = (NrBatchCase * len(cases))()
        for k, c in enumerate(cases):
            scat = c.get("scat")
            plan = OSTR(c["geom"], subset_num=c["subset_num"], beta=c["beta"], delta=c["delta"],
                        potential=c.get("potential", "lange"),
                        gamma_mode=c.get("gamma_mode", "length"), has_scatter=scat is not None)
            plan.setup(c["angles"], c["prj"], c["blank"], scat)
            x0 = c.get("x0")
            x = (torch.zeros(c["geom"].n_voxels, dtype=torch.float32, device=plan.ws.device)
                 if x0 is None else _in(x0).clone())
            if tune:
                plan.autotune(x)
            if "upd_planes" in c:  # an explicit slab depth (8, 16 or 32) wins
                plan.params.upd_planes = int(c["upd_planes"])
            if "upd_tile" in c:    # and an explicit update tile (0, 1 or 2)
                plan.params.upd_tile = int(c["upd_tile"])
            self.plans.append(plan)
            self.x.append(x)
            arr[k] = NrBatchCase(plan.gc, plan.params, int(c["iter_num"]),
                                 ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(plan.ws.data_ptr()), plan.ws_bytes)
        self._cases = arr
        size = ctypes.c_size_t(0)
        native.call("nr_batch_table_size", len(cases), ctypes.byref(size))
        # host memory: each batch launch carries the table as its kernel parameter
        self.table = np.zeros(int(size.value), dtype=np.uint8)
        steps = ctypes.c_int32(0)
        native.call("nr_batch_prepare", arr, len(cases), self._table_ptr(), size,
                    ctypes.byref(steps), _stream())
        self.n_steps = int(steps.value)

    def _table_ptr(self) -> ctypes.c_void_p:
        return ctypes.c_void_p(self.table.ctypes.data)

    def run(self):
        """All steps and the finish on the current stream; returns the volumes."""
        if self.mode == "sequential":
            for p, x, n in zip(self.plans, self.x, self.iters):
                p.iterate(x, n)
        else:
            for k in range(self.n_steps):
                native.call("nr_batch_step", self._table_ptr(), k, _stream())
            native.call("nr_batch_finish", self._table_ptr(), _stream())
        self.check()
        return self.x

    def check(self) -> None:
        for p in self.plans:
            p.check()

    def graph(self, n_steps: Optional[int] = None):
        """The batch loop as CUDA graphs: in "shared" mode one graph of every
        step (or the first n_steps, for timing a part of the run) and the
        finish; in "sequential" mode, for the whole run, each case's
        iteration loop as its own graph, launched one after another."""
        if self.mode == "sequential" and (n_steps is None or n_steps >= self.n_steps):
            return SequentialGraph(self)
        return BatchGraph(self, n_steps)


class SequentialGraph:
    """The cases of a Batch one after another, each case's whole iteration
    loop captured as its own graph (OstrGraph)."""

    def __init__(self, batch: Batch):
        self.graphs = [p.graph(x, n) for p, x, n in zip(batch.plans, batch.x, batch.iters)]

    def launch(self) -> None:
        for g in self.graphs:
            g.launch()

    def close(self) -> None:
        for g in self.graphs:
            g.close()


class BatchGraph:
    """The batch loop (all steps + finish) captured once as a CUDA graph.
    Each launch() runs it again from the cases' current volumes.  With n_steps
    below the batch's step count the graph runs only the first steps; the
    volumes are then intermediate states (for timing and profiling)."""

    def __init__(self, batch: Batch, n_steps: Optional[int] = None):
        self.batch = batch
        self.handle = ctypes.c_void_p(0)
        self._stream = torch.cuda.Stream()
        self._stream.wait_stream(torch.cuda.current_stream())
        steps = batch.n_steps if n_steps is None else int(n_steps)
        native.call("nr_batch_graph_create", batch._table_ptr(), steps,
                    ctypes.c_void_p(self._stream.cuda_stream), ctypes.byref(self.handle))

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


def reconstruct(geom: Geometry, prj, blank, scatter=None, *, angles, subset_num: int,
                iter_num: int, beta: float, delta: float, potential: str = "lange",
                gamma_mode: str = "length", x0=None, monotone=False, check_every: int = 1,
                tune="cached", stream=None, timing: Optional[dict] = None):
    """OSTR reconstruction: transmission counts in, attenuation (1/mm) out.

    prj, blank, scatter: [view][i][j] in original view order (the layout
    load_prj produces).  Returns the volume [z][y][x]; numpy when prj was a
    host array, else a CUDA tensor.  monotone=True stops before the first
    iteration that would raise the FP64 objective; monotone="subset" keeps
    only the sub-iteration steps that do not raise the FP64 subset objective
    (OSTR.iterate; check_every=k checks the iteration-level objective every
    k iterations).  tune:
    "cached" runs the kernel variants the autotuner cached for this GPU and
    geometry (the defaults when it has none), True tunes first when the
    cache has none, False runs the defaults.  Every variant gives the same
    result bit for bit.  stream: a torch.cuda.Stream to run every copy and
    kernel on (default: the current stream).  The call returns once that
    stream has finished the reconstruction (the status check waits for it).
    timing: a dict that receives the device time of each phase in seconds
    (CUDA events on the stream): "upload_s" (host to device copies of the
    counts, blank scan, angles and x0), "setup_s" (gamma and d), "iterate_s"
    (the iterations), "download_s" (the status check and the volume's copy
    back), and "wall_s", the host's clock around the whole call.
    """
    if not (tune == "cached" or tune is True or tune is False):
        raise ValueError('tune must be "cached", True or False')
    if stream is not None:
        if not isinstance(stream, torch.cuda.Stream):
            raise TypeError("stream must be a torch.cuda.Stream")
        with torch.cuda.stream(stream):
            return reconstruct(geom, prj, blank, scatter, angles=angles, subset_num=subset_num,
                               iter_num=iter_num, beta=beta, delta=delta, potential=potential,
                               gamma_mode=gamma_mode, x0=x0, monotone=monotone,
                               check_every=check_every, tune=tune, timing=timing)
    t_wall = time.perf_counter()
    ev = None
    if timing is not None:
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    plan = OSTR(geom, subset_num=subset_num, beta=beta, delta=delta, potential=potential,
                gamma_mode=gamma_mode, has_scatter=scatter is not None)
    if ev:
        ev[0].record()
    ang, y, b = _in(angles), _in(prj), _in(blank)
    s = None if scatter is None else _in(scatter)
    x = None if x0 is None else _in(x0).clone()
    if ev:
        ev[1].record()
    plan.setup(ang, y, b, s)
    if tune is True:
        plan.autotune()
    elif tune == "cached":
        from . import autotune

        autotune.apply_cached(plan)
    if x is None:
        x = torch.zeros(geom.n_voxels, dtype=torch.float32, device=plan.ws.device)
    if ev:
        ev[2].record()
    plan.iterate(x, iter_num, monotone=monotone, check_every=check_every)
    if ev:
        ev[3].record()
    plan.check()
    out = _like_input(prj, x)
    if ev:
        ev[4].record()
        ev[4].synchronize()
        for k, name in enumerate(("upload_s", "setup_s", "iterate_s", "download_s")):
            timing[name] = ev[k].elapsed_time(ev[k + 1]) / 1e3
        timing["wall_s"] = time.perf_counter() - t_wall
    return out
