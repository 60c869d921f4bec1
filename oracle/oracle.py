"""TEST INFRASTRUCTURE ONLY: ctypes bindings of the CPU oracle and of the CPU
build of the reference.

``Oracle(dtype)``  -- oracle/ostr_oracle.cpp, the restatement of the
                      reference's OSTR path, in float64 (the FP64 oracle) or
                      float32 (the timed CPU baseline).
``Reference()``    -- oracle/_ref/libostr_ref.so, the reference's own kernel
                      bodies and gold driver compiled for the CPU by
                      oracle/build_ref.sh (only on a machine that holds the
                      reference sources).
"""
from __future__ import annotations

import ctypes
import os
import tempfile
from typing import Optional

import numpy as np

from newrecon_gb300.geometry import Geometry, NrOstrParams, NrSartParams, POTENTIALS, GAMMA_MODES

from .build import ORACLE_SO, REF_SO

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """The C++ restatement (double or float)."""

    _lib = None

    def __init__(self, dtype=np.float64, threads: int = 0):
        if Oracle._lib is None:
            if not os.path.isfile(ORACLE_SO):
                raise RuntimeError(f"oracle library missing: {ORACLE_SO} (run python -m oracle.build)")
            Oracle._lib = ctypes.CDLL(ORACLE_SO)
            Oracle._lib.orc_max_threads.restype = ctypes.c_int
        self.lib = Oracle._lib
        self.dtype = np.dtype(dtype)
        self.suf = "f64" if self.dtype == np.float64 else "f32"
        if threads:
            self.lib.orc_set_threads(int(threads))

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(int(n))

    @property
    def max_threads(self) -> int:
        return int(self.lib.orc_max_threads())

    def _arr(self, a) -> np.ndarray:
        return np.ascontiguousarray(a, dtype=self.dtype)

    def _fn(self, name):
        return getattr(self.lib, f"orc_{name}_{self.suf}")

    def fp_ostr(self, g: Geometry, x, angles, index, a0: int, a1: int, out=None) -> np.ndarray:
        x = self._arr(x).ravel()
        out = np.zeros((a1 - a0) * g.n_bins, self.dtype) if out is None else out
        gc = g.to_c()
        self._fn("fp_ostr")(ctypes.byref(gc), _ptr(x), _ptr(out),
                            _ptr(np.ascontiguousarray(angles, np.float32)),
                            _ptr(np.ascontiguousarray(index, np.int32)),
                            ctypes.c_int(a0), ctypes.c_int(a1))
        return out

    def fp_gamma(self, g: Geometry, angles, index, a0: int, a1: int, mode="length",
                 out=None) -> np.ndarray:
        out = np.zeros((a1 - a0) * g.n_bins, self.dtype) if out is None else out
        gc = g.to_c()
        self._fn("fp_gamma")(ctypes.byref(gc), _ptr(out),
                             _ptr(np.ascontiguousarray(angles, np.float32)),
                             _ptr(np.ascontiguousarray(index, np.int32)),
                             ctypes.c_int(a0), ctypes.c_int(a1),
                             ctypes.c_int(GAMMA_MODES[mode] if isinstance(mode, str) else int(mode)))
        return out

    def bp_sbp(self, g: Geometry, prj, index, angles, a0: int, a1: int, vol=None) -> np.ndarray:
        vol = np.zeros(g.n_voxels, self.dtype) if vol is None else vol
        prj = self._arr(prj).ravel()
        gc = g.to_c()
        self._fn("bp_sbp")(ctypes.byref(gc), _ptr(vol), _ptr(prj),
                           _ptr(np.ascontiguousarray(index, np.int32)),
                           _ptr(np.ascontiguousarray(angles, np.float32)),
                           ctypes.c_int(a0), ctypes.c_int(a1))
        return vol

    def prior(self, g: Geometry, x, potential, delta: float, zxy: Optional[float] = None,
              RDD=None, RD=None):
        x = self._arr(x).ravel()
        RDD = np.zeros(g.n_voxels, self.dtype) if RDD is None else RDD
        RD = np.zeros(g.n_voxels, self.dtype) if RD is None else RD
        pot = POTENTIALS[potential] if isinstance(potential, str) else int(potential)
        zxy = g.z_xy_ratio if zxy is None else zxy
        gc = g.to_c()
        self._fn("prior")(ctypes.byref(gc), _ptr(RDD), _ptr(RD), _ptr(x), ctypes.c_int(pot),
                          ctypes.c_double(delta), ctypes.c_double(zxy))
        return RDD, RD

    def compute_yry(self, prj, scat=None) -> np.ndarray:
        prj = self._arr(prj).ravel()
        scat = None if scat is None else self._arr(scat).ravel()
        out = np.empty_like(prj)
        self._fn("compute_yry")(_ptr(out), _ptr(prj), _ptr(scat), ctypes.c_int64(prj.size))
        return out

    def compute_h(self, prj, blank, line, scat=None) -> np.ndarray:
        prj = self._arr(prj).ravel()
        blank = self._arr(blank).ravel()
        line = self._arr(line).ravel()
        scat = None if scat is None else self._arr(scat).ravel()
        out = np.empty_like(prj)
        self._fn("compute_h")(_ptr(out), _ptr(prj), _ptr(blank), _ptr(line), _ptr(scat),
                              ctypes.c_int64(prj.size))
        return out

    def update_est(self, est, capL, RD, d, RDD, beta: float) -> np.ndarray:
        est = self._arr(est).ravel().copy()
        self._fn("update_est")(_ptr(est), _ptr(self._arr(capL)), _ptr(self._arr(RD)),
                               _ptr(self._arr(d)), _ptr(self._arr(RDD)),
                               ctypes.c_double(beta), ctypes.c_int64(est.size))
        return est

    def regroup(self, arr, n_angles: int, subset_num: int) -> np.ndarray:
        arr = self._arr(arr).ravel()
        out = np.empty_like(arr)
        self._fn("regroup")(_ptr(out), _ptr(arr), ctypes.c_int(n_angles),
                            ctypes.c_int(subset_num), ctypes.c_int64(arr.size // n_angles))
        return out

    def reorder_index(self, n_angles: int, subset_num: int) -> np.ndarray:
        idx = np.arange(n_angles, dtype=np.int32)
        self.lib.orc_reorder_index(_ptr(idx), ctypes.c_int(n_angles), ctypes.c_int(subset_num))
        return idx

    def reconstruct(self, g: Geometry, angles, prj, blank, scat=None, *, subset_num: int,
                    iter_num: int, beta: float, delta: float, potential="lange",
                    gamma_mode="length", x0=None, return_d: bool = False):
        p = NrOstrParams(subset_num, POTENTIALS[potential] if isinstance(potential, str) else int(potential),
                         GAMMA_MODES[gamma_mode] if isinstance(gamma_mode, str) else int(gamma_mode),
                         0 if scat is None else 1, beta, delta)
        gc = g.to_c()
        x = np.zeros(g.n_voxels, self.dtype) if x0 is None else self._arr(x0).ravel().copy()
        d = np.zeros(g.n_voxels, self.dtype)
        gam = np.zeros(g.n_angles * g.n_bins, self.dtype)
        self._fn("reconstruct")(ctypes.byref(gc), ctypes.byref(p),
                                _ptr(np.ascontiguousarray(angles, np.float32)),
                                _ptr(self._arr(prj).ravel()), _ptr(self._arr(blank).ravel()),
                                _ptr(None if scat is None else self._arr(scat).ravel()),
                                _ptr(x), ctypes.c_int(iter_num), _ptr(d), _ptr(gam))
        if return_d:
            return x, d, gam
        return x

    def subiter(self, g: Geometry, angles, index, a0: int, a1: int, prj_sub, blank_sub, d, x,
                *, subset_num: int, beta: float, delta: float, potential="lange",
                scat_sub=None) -> None:
        """One sub-iteration in place on x (subset views [a0, a1) of index)."""
        p = NrOstrParams(subset_num, POTENTIALS[potential] if isinstance(potential, str) else int(potential),
                         0, 0 if scat_sub is None else 1, beta, delta)
        gc = g.to_c()
        assert x.dtype == self.dtype and x.flags.c_contiguous
        self._fn("subiter")(ctypes.byref(gc), ctypes.byref(p),
                            _ptr(np.ascontiguousarray(angles, np.float32)),
                            _ptr(np.ascontiguousarray(index, np.int32)), ctypes.c_int(a0),
                            ctypes.c_int(a1), _ptr(self._arr(prj_sub)), _ptr(self._arr(blank_sub)),
                            _ptr(None if scat_sub is None else self._arr(scat_sub)),
                            _ptr(self._arr(d)), _ptr(x))

    # --- SART family -------------------------------------------------------
    def fp_sart(self, g: Geometry, x, angles, index, a0: int, a1: int, use_cos: bool,
                est=None, norm=None):
        """(est, norm) of the SART projector; missed rays keep est/norm's values."""
        x = self._arr(x).ravel()
        n = (a1 - a0) * g.n_bins
        est = np.zeros(n, self.dtype) if est is None else est
        norm = np.zeros(n, self.dtype) if norm is None else norm
        gc = g.to_c()
        self._fn("fp_sart")(ctypes.byref(gc), _ptr(x), _ptr(est), _ptr(norm),
                            _ptr(np.ascontiguousarray(angles, np.float32)),
                            _ptr(np.ascontiguousarray(index, np.int32)),
                            ctypes.c_int(a0), ctypes.c_int(a1), ctypes.c_int(int(bool(use_cos))))
        return est, norm

    def fp_4r(self, g: Geometry, x, angles, index, a0: int, a1: int, use_cos: bool = False,
              layout: str = "ji", sub=None) -> np.ndarray:
        """The fixed 2 x 2 super-sampled projector; sub (optional) gets the sub-ray sums."""
        x = self._arr(x).ravel()
        out = np.zeros((a1 - a0) * g.n_bins, self.dtype)
        gc = g.to_c()
        self._fn("fp_4r")(ctypes.byref(gc), _ptr(x), _ptr(out), _ptr(sub),
                          _ptr(np.ascontiguousarray(angles, np.float32)),
                          _ptr(np.ascontiguousarray(index, np.int32)), ctypes.c_int(a0),
                          ctypes.c_int(a1), ctypes.c_int(int(bool(use_cos))),
                          ctypes.c_int({"ij": 0, "ji": 1}[layout]))
        return out

    def sart_prj_diff(self, prj, est, norm) -> np.ndarray:
        prj, est, norm = self._arr(prj).ravel(), self._arr(est).ravel(), self._arr(norm).ravel()
        out = np.empty_like(prj)
        self._fn("sart_prj_diff")(_ptr(out), _ptr(prj), _ptr(est), _ptr(norm),
                                  ctypes.c_int64(prj.size))
        return out

    def bp_ossart(self, g: Geometry, x, diff, index, angles, a0: int, a1: int, lam: float,
                  prior=None, beta: float = 0.0) -> np.ndarray:
        """OS-SART update of a copy of x."""
        x = self._arr(x).ravel().copy()
        gc = g.to_c()
        self._fn("bp_ossart")(ctypes.byref(gc), _ptr(x), _ptr(self._arr(diff).ravel()),
                              _ptr(None if prior is None else self._arr(prior).ravel()),
                              _ptr(np.ascontiguousarray(index, np.int32)),
                              _ptr(np.ascontiguousarray(angles, np.float32)),
                              ctypes.c_int(a0), ctypes.c_int(a1), ctypes.c_double(lam),
                              ctypes.c_double(beta))
        return x

    def prior_sart(self, g: Geometry, x, delta: float, prior=None) -> np.ndarray:
        prior = np.zeros(g.n_voxels, self.dtype) if prior is None else prior
        gc = g.to_c()
        self._fn("prior_sart")(ctypes.byref(gc), _ptr(prior), _ptr(self._arr(x).ravel()),
                               ctypes.c_double(delta))
        return prior

    def line_integrals(self, prj, blank, scat=None) -> np.ndarray:
        prj, blank = self._arr(prj).ravel(), self._arr(blank).ravel()
        scat = None if scat is None else self._arr(scat).ravel()
        out = np.empty_like(prj)
        self._fn("line_integrals")(_ptr(out), _ptr(prj), _ptr(blank), _ptr(scat),
                                   ctypes.c_int64(prj.size))
        return out

    def ossart(self, g: Geometry, angles, line, *, subset_num: int, iter_num: int, lam: float,
               use_cos: bool = True, regularized: bool = False, beta: float = 0.0,
               delta: float = 1.0, supersample: bool = False, x0=None) -> np.ndarray:
        """The OS-SART loop (nr_sart_iterate's semantics)."""
        p = NrSartParams(subset_num, int(bool(use_cos)), int(bool(regularized)), 0, 0, lam, beta,
                         delta, int(bool(supersample)))
        gc = g.to_c()
        x = np.zeros(g.n_voxels, self.dtype) if x0 is None else self._arr(x0).ravel().copy()
        self._fn("ossart")(ctypes.byref(gc), ctypes.byref(p),
                           _ptr(np.ascontiguousarray(angles, np.float32)),
                           _ptr(self._arr(line).ravel()), _ptr(x), ctypes.c_int(iter_num))
        return x

    def objective(self, g: Geometry, angles, prj, blank, x, *, potential, delta, scat=None):
        """FP64 objective parts (data, penalty); total = data + beta * penalty."""
        p = NrOstrParams(1, POTENTIALS[potential] if isinstance(potential, str) else int(potential),
                         0, 0 if scat is None else 1, 0.0, delta)
        gc = g.to_c()
        out = np.zeros(2, np.float64)
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64).ravel()
        self.lib.orc_objective_f64(ctypes.byref(gc), ctypes.byref(p),
                                   _ptr(np.ascontiguousarray(angles, np.float32)),
                                   _ptr(f(prj)), _ptr(f(blank)), _ptr(f(scat)), _ptr(f(x)),
                                   _ptr(out))
        return float(out[0]), float(out[1])


class Reference:
    """The reference's own code compiled for the CPU (float32 only)."""

    _lib = None

    def __init__(self):
        if Reference._lib is None:
            if not os.path.isfile(REF_SO):
                raise RuntimeError(f"reference CPU build missing: {REF_SO} (run oracle/build_ref.sh)")
            Reference._lib = ctypes.CDLL(REF_SO)
        self.lib = Reference._lib

    def set_geometry(self, g: Geometry, subset_num: int = 1, beta: float = 0.0,
                     delta: float = 1.0) -> None:
        gc = g.to_c()
        self.lib.ref_set_geometry(ctypes.byref(gc), ctypes.c_int(subset_num),
                                  ctypes.c_float(beta), ctypes.c_float(delta))
        self.g = g

    @staticmethod
    def _f(a) -> np.ndarray:
        return np.ascontiguousarray(a, np.float32).ravel().copy()

    def fp_ostr_cos(self, x, angles, index, a0, a1, line=None) -> np.ndarray:
        g = self.g
        line = np.zeros((a1 - a0) * g.n_bins, np.float32) if line is None else self._f(line)
        self.lib.ref_fp_ostr_cos(_ptr(self._f(x)), _ptr(line), _ptr(self._f(angles)),
                                 _ptr(np.ascontiguousarray(index, np.int32)),
                                 ctypes.c_int(a0), ctypes.c_int(a1))
        return line

    def fp_normprj(self, angles, index, a0, a1) -> np.ndarray:
        g = self.g
        out = np.zeros((a1 - a0) * g.n_bins, np.float32)
        self.lib.ref_fp_normprj(_ptr(out), _ptr(self._f(angles)),
                                _ptr(np.ascontiguousarray(index, np.int32)),
                                ctypes.c_int(a0), ctypes.c_int(a1))
        return out

    def bp_sbp(self, prj, index, angles, a0, a1, vol=None) -> np.ndarray:
        vol = np.zeros(self.g.n_voxels, np.float32) if vol is None else self._f(vol)
        self.lib.ref_bp_sbp(_ptr(vol), _ptr(self._f(prj)),
                            _ptr(np.ascontiguousarray(index, np.int32)), _ptr(self._f(angles)),
                            ctypes.c_int(a0), ctypes.c_int(a1))
        return vol

    def prior_lange(self, x, delta, zxy):
        n = self.g.n_voxels
        RDD = np.zeros(n, np.float32)
        RD = np.zeros(n, np.float32)
        self.lib.ref_prior_lange(_ptr(RDD), _ptr(RD), _ptr(self._f(x)), ctypes.c_float(delta),
                                 ctypes.c_float(zxy))
        return RDD, RD

    def prior_q2(self, x, zxy):
        n = self.g.n_voxels
        RDD = np.zeros(n, np.float32)
        RD = np.zeros(n, np.float32)
        self.lib.ref_prior_q2(_ptr(RDD), _ptr(RD), _ptr(self._f(x)), ctypes.c_float(zxy))
        return RDD, RD

    def prior_hyperbola_grad(self, x, delta):
        out = np.zeros(self.g.n_voxels, np.float32)
        self.lib.ref_prior_hyperbola_grad(_ptr(out), _ptr(self._f(x)), ctypes.c_float(delta))
        return out

    def fp_sart(self, x, angles, index, a0, a1, use_cos, est=None, norm=None):
        g = self.g
        n = (a1 - a0) * g.n_bins
        est = np.zeros(n, np.float32) if est is None else self._f(est)
        norm = np.zeros(n, np.float32) if norm is None else self._f(norm)
        self.lib.ref_fp_sart(_ptr(self._f(x)), _ptr(est), _ptr(norm), _ptr(self._f(angles)),
                             _ptr(np.ascontiguousarray(index, np.int32)), ctypes.c_int(a0),
                             ctypes.c_int(a1), ctypes.c_int(int(bool(use_cos))))
        return est, norm

    def fp_4r_subrays(self, x, angles, index, a0, a1):
        """The reference's 4R sub-ray kernel: [view][2 BINSy][2 BINSx], zero-initialised."""
        g = self.g
        sub = np.zeros((a1 - a0) * 4 * g.n_bins, np.float32)
        self.lib.ref_fp_4r_subrays(_ptr(self._f(x)), _ptr(sub), _ptr(self._f(angles)),
                                   _ptr(np.ascontiguousarray(index, np.int32)),
                                   ctypes.c_int(a0), ctypes.c_int(a1))
        return sub

    def sart_prj_diff(self, prj, est, norm, index, a0, a1):
        out = np.zeros(np.size(prj), np.float32)
        self.lib.ref_sart_prj_diff(_ptr(out), _ptr(self._f(prj)), _ptr(self._f(est)),
                                   _ptr(self._f(norm)),
                                   _ptr(np.ascontiguousarray(index, np.int32)),
                                   ctypes.c_int(a0), ctypes.c_int(a1))
        return out

    def bp_ossart(self, x, diff, index, angles, a0, a1, lam, prior=None, beta=0.0):
        x = self._f(x)
        self.lib.ref_bp_ossart(_ptr(x), _ptr(self._f(diff)),
                               _ptr(None if prior is None else self._f(prior)),
                               _ptr(np.ascontiguousarray(index, np.int32)), _ptr(self._f(angles)),
                               ctypes.c_int(a0), ctypes.c_int(a1), ctypes.c_float(lam),
                               ctypes.c_float(beta))
        return x

    def prior_sart(self, x, delta):
        out = np.zeros(self.g.n_voxels, np.float32)
        self.lib.ref_prior_sart(_ptr(out), _ptr(self._f(x)), ctypes.c_float(delta))
        return out

    def ossart(self, angles, line, *, subset_num, iter_num, lam, use_cos=True,
               regularized=False, beta=0.0, delta=1.0, x0=None):
        """OS-SART composed from the reference's own SART launch wrappers.

        The reference has no OS-SART driver (Recon_Method 3 is empty), so this
        loop is the composition the kernels imply, in the OSTR driver's subset
        order: per subset, est/norm zeroed, fprojectCB_1R_GPU_SART[_cos],
        SART_prj_diff, [prior zeroed + prior_GPU_SART], bprojectCB_4B_GPU_SART[_R].
        """
        g = self.g
        A, M = g.n_angles, subset_num
        Vs, B = A // M, g.n_bins
        idx = np.arange(A, dtype=np.int32)
        ridx = np.concatenate([idx[i::M] for i in range(M)]).astype(np.int32)
        lr = np.asarray(line, np.float32).reshape(A, B)[ridx]
        x = np.zeros(g.n_voxels, np.float32) if x0 is None else self._f(x0)
        for _ in range(iter_num):
            for a in range(M):
                a0, a1 = a * Vs, (a + 1) * Vs
                est, norm = self.fp_sart(x, angles, ridx, a0, a1, use_cos)
                diff = self.sart_prj_diff(lr[a0:a1].ravel(), est, norm, ridx, a0, a1)
                prior = self.prior_sart(x, delta) if regularized else None
                x = self.bp_ossart(x, diff, ridx, angles, a0, a1, lam, prior, beta)
        return x

    def compute_yry(self, prj, scat):
        out = np.zeros(np.size(prj), np.float32)
        self.lib.ref_compute_yry(_ptr(out), _ptr(self._f(prj)), _ptr(self._f(scat)))
        return out

    def compute_h(self, prj, blank, line, scat):
        out = np.zeros(np.size(prj), np.float32)
        self.lib.ref_compute_h(_ptr(out), _ptr(self._f(prj)), _ptr(self._f(blank)),
                               _ptr(self._f(line)), _ptr(self._f(scat)))
        return out

    def update_est(self, est, capL, RD, d, RDD):
        est = self._f(est)
        self.lib.ref_update_est(_ptr(est), _ptr(self._f(capL)), _ptr(self._f(RD)),
                                _ptr(self._f(d)), _ptr(self._f(RDD)))
        return est

    def regroup_prj(self, arr):
        arr = self._f(arr)
        self.lib.ref_regroup_prj(_ptr(arr))
        return arr

    def x_y_flip(self, view_ji):
        out = np.zeros(np.size(view_ji), np.float32)
        self.lib.ref_x_y_flip(_ptr(self._f(view_ji)), _ptr(out))
        return out

    def reconstruct(self, angles, prj, blank, scat, *, method: int, subset_num: int,
                    iter_num: int, beta: float, delta: float, x0=None):
        """Runs the reference's Reconstruction() (gold driver) through files.

        prj/blank/scat: [view][i][j] (after x_y_flip); written in the scanner
        file layout [j][i] that load_prj flips back.  method 0 = Q2, 1 = Lange.
        Returns the volume after the last iteration.
        """
        g = self.g
        self.set_geometry(g, subset_num, beta, delta)
        with tempfile.TemporaryDirectory() as d:
            np.ascontiguousarray(angles, np.float32).tofile(os.path.join(d, "angles.bin"))
            for name, arr in (("prj", prj), ("scat", scat), ("blank", blank)):
                a = np.asarray(arr, np.float32).reshape(g.n_angles, g.nbx, g.nby)
                for v in range(g.n_angles):
                    np.ascontiguousarray(a[v].T).tofile(os.path.join(d, f"{name}{v + 1:04d}"))
            ini = os.path.join(d, "ini.bin")
            if x0 is not None:
                np.ascontiguousarray(x0, np.float32).tofile(ini)
            self.lib.ref_reconstruct(ctypes.c_int(method), ctypes.c_int(iter_num),
                                     ctypes.c_int(iter_num), d.encode(),
                                     os.path.join(d, "angles.bin").encode(), ini.encode())
            out = os.path.join(d, f"recon{iter_num - 1}")
            return np.fromfile(out, np.float32)
