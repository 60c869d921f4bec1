"""ctypes binding of libnrgb300.so (the C ABI declared in include/nrgb300.h).

The library is the only compute path: when it is missing or no CUDA device is
present every entry point raises; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional

from .geometry import NrGeom, NrOstrParams, NrSartParams

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libnrgb300.so")

STATUS = {
    0: "NR_OK",
    1: "NR_ERR_BAD_GEOMETRY",
    2: "NR_ERR_BAD_ARGUMENT",
    3: "NR_ERR_LAUNCH",
    4: "NR_ERR_NONFINITE",
    5: "NR_ERR_TIMEOUT",
    6: "NR_ERR_WORKSPACE",
    7: "NR_ERR_CUDA",
}

# Every symbol include/nrgb300.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_F = ctypes.c_float
_GP = ctypes.POINTER(NrGeom)
_PP = ctypes.POINTER(NrOstrParams)
_SP = ctypes.POINTER(NrSartParams)
SIGNATURES = {
    "nr_validate_geometry": (_I32, [_GP, _I32]),
    "nr_fp_ostr": (_I32, [_GP, _P, _P, _P, _P, _I32, _I32, _P]),
    "nr_fp_gamma": (_I32, [_GP, _P, _P, _P, _I32, _I32, _I32, _P]),
    "nr_bp_sbp": (_I32, [_GP, _P, _P, _P, _P, _I32, _I32, _P]),
    "nr_prior": (_I32, [_GP, _P, _P, _P, _I32, _F, _F, _P]),
    "nr_compute_yry": (_I32, [_P, _P, _P, _I64, _P]),
    "nr_compute_gamma_yry": (_I32, [_P, _P, _P, _I64, _P]),
    "nr_compute_h": (_I32, [_P, _P, _P, _P, _P, _I64, _P]),
    "nr_update_est": (_I32, [_P, _P, _P, _P, _P, _F, _I64, _P]),
    "nr_scale": (_I32, [_P, _F, _I64, _P]),
    "nr_regroup": (_I32, [_P, _P, _I32, _I32, _I64, _P]),
    "nr_x_y_flip": (_I32, [_P, _P, _I32, _I32, _I32, _P]),
    "nr_ostr_workspace_size": (_I32, [_GP, _PP, ctypes.POINTER(ctypes.c_size_t)]),
    "nr_ostr_setup": (_I32, [_GP, _PP, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "nr_ostr_iterate": (_I32, [_GP, _PP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_ostr_subiter": (_I32, [_GP, _PP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_ostr_objective": (_I32, [_GP, _PP, _P, _P, _P, ctypes.c_size_t, _P]),
    "nr_ostr_subset": (_I32, [_GP, _PP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_objective_fp64": (_I32, [_GP, _PP, _P, _P, _P, ctypes.c_size_t, _P]),
    "nr_workspace_size": (_I32, [_GP, _PP, ctypes.POINTER(ctypes.c_size_t)]),
    "nr_ostr_project": (_I32, [_GP, _PP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_ostr_project_fp64": (_I32, [_GP, _PP, _P, _I32, _P, _P, ctypes.c_size_t, _P]),
    "nr_ostr_penalty": (_I32, [_GP, _PP, _P, _P, _P, ctypes.c_size_t, _P]),
    "nr_test_expire_wait": (_I32, [_P, _I32, _P]),
    "nr_ostr_update": (_I32, [_GP, _PP, _P, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_ostr_workspace_section": (_I32, [_GP, _PP, _I32, _P, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_size_t)]),
    "nr_ostr_graph_create": (_I32, [_GP, _PP, _P, _I32, _P, ctypes.c_size_t, _P,
                                    ctypes.POINTER(ctypes.c_void_p)]),
    "nr_ostr_graph_launch": (_I32, [_P, _P]),
    "nr_ostr_graph_destroy": (_I32, [_P]),
    "nr_batch_table_size": (_I32, [_I32, ctypes.POINTER(ctypes.c_size_t)]),
    "nr_batch_prepare": (_I32, [_P, _I32, _P, ctypes.c_size_t, ctypes.POINTER(_I32), _P]),
    "nr_batch_step": (_I32, [_P, _I32, _P]),
    "nr_batch_finish": (_I32, [_P, _P]),
    "nr_batch_graph_create": (_I32, [_P, _I32, _P, ctypes.POINTER(ctypes.c_void_p)]),
    "nr_cnn_param_count": (_I32, [ctypes.POINTER(_I64)]),
    "nr_cnn_workspace_size": (_I32, [_P, _I32, ctypes.POINTER(ctypes.c_size_t)]),
    "nr_cnn_forward": (_I32, [_P, _P, _P, _F, _P, _P, ctypes.c_size_t, _P]),
    "nr_cnn_loss_grad": (_I32, [_P, _P, _P, _P, _F, _P, _P, _P, ctypes.c_size_t, _P]),
    "nr_cnn_adam": (_I32, [_P, _P, _P, _P, _I64, _I32, _F, _P]),
    "nr_cnn_train_step": (_I32, [_P, _P, _P, _P, _I32, _F, _P, _P, _F, _P, _P, ctypes.c_size_t,
                                 _P]),
    "nr_cnn_check": (_I32, [_P, ctypes.POINTER(_I32), _P]),
    "nr_ostr_check": (_I32, [_P, ctypes.c_size_t, ctypes.POINTER(_I32), _P]),
    "nr_penalty_fp64_static": (_I32, [_GP, _P, _I32, _F, _P, _P]),
    "nr_fp_sart": (_I32, [_GP, _P, _P, _P, _P, _P, _I32, _I32, _I32, _P]),
    "nr_fp_4r": (_I32, [_GP, _P, _P, _P, _P, _P, _I32, _I32, _I32, _I32, _P]),
    "nr_sart_prj_diff": (_I32, [_P, _P, _P, _P, _I64, _P]),
    "nr_bp_ossart": (_I32, [_GP, _P, _P, _P, _P, _P, _I32, _I32, _F, _F, _P]),
    "nr_prior_sart": (_I32, [_GP, _P, _P, _F, _P]),
    "nr_sart_line_integrals": (_I32, [_P, _P, _P, _P, _I64, _P]),
    "nr_sart_workspace_size": (_I32, [_GP, _SP, ctypes.POINTER(ctypes.c_size_t)]),
    "nr_sart_setup": (_I32, [_GP, _SP, _P, _P, _P, ctypes.c_size_t, _P]),
    "nr_sart_iterate": (_I32, [_GP, _SP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_sart_subiter": (_I32, [_GP, _SP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_sart_project": (_I32, [_GP, _SP, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_sart_update": (_I32, [_GP, _SP, _P, _P, _I32, _P, ctypes.c_size_t, _P]),
    "nr_sart_graph_create": (_I32, [_GP, _SP, _P, _I32, _P, ctypes.c_size_t, _P,
                                    ctypes.POINTER(ctypes.c_void_p)]),
    "nr_sart_workspace_section": (_I32, [_GP, _SP, _I32, _P, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_size_t)]),
    "nr_de_subtract": (_I32, [_P, _P, _P, _I32, _I64, ctypes.c_double, _P, _I64, _I64, _P, _P]),
    "nr_hist8": (_I32, [_P, _I64, _P, _P]),
    "nr_hist_entropy": (_I32, [_P, _I64, ctypes.POINTER(ctypes.c_double)]),
    "nr_otsu_level": (_I32, [_P, ctypes.POINTER(ctypes.c_double)]),
    "nr_version": (ctypes.c_char_p, []),
}


class NrError(RuntimeError):
    """A non-zero nr_status from the library."""

    def __init__(self, fn: str, code: int):
        super().__init__(f"{fn} failed: {STATUS.get(code, code)}")
        self.code = code
        self.fn = fn


_lib: Optional[ctypes.CDLL] = None
_lock = threading.Lock()


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libnrgb300.so (once) and declares every signature."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.isfile(path):
            raise RuntimeError(
                f"libnrgb300.so not built ({path}); run `python -m newrecon_gb300._build` "
                "(there is no CPU fallback)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name: str, *args) -> None:
    """Calls an nr_* entry point and raises NrError on a non-zero status."""
    rc = getattr(load(), name)(*args)
    if rc != 0:
        raise NrError(name, int(rc))


def version() -> str:
    return load().nr_version().decode()
