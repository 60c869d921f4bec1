"""Scanner and grid geometry of the DBT OSTR reconstruction.

The field set is the reference's geometry globals (``Tomo_OSTR.cu:21-36,47-50``;
``ostr.py:21-52``): a volume of ``IMGSIZx x IMGSIZy x IMGSIZz`` voxels with its
corner at ``(x_p0, y_p0, z_p0)``, a stationary flat detector at
``z = -detectorR`` with its corner at ``(x_d0, y_d0)``, and a source that
rotates about the y axis at radius ``sourceR``:
``(sourceR sin t, sourceY, sourceR cos t)`` (``Tomo_OSTR.cu:1340-1356``).

``Geometry`` mirrors the C struct ``nr_geom`` of ``include/nrgb300.h`` and is
passed by value to every kernel.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np


class NrGeom(ctypes.Structure):
    """ctypes image of ``nr_geom`` (include/nrgb300.h)."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("vx", ctypes.c_float), ("vy", ctypes.c_float), ("vz", ctypes.c_float),
        ("x_p0", ctypes.c_float), ("y_p0", ctypes.c_float), ("z_p0", ctypes.c_float),
        ("nbx", ctypes.c_int32), ("nby", ctypes.c_int32),
        ("bx", ctypes.c_float), ("by", ctypes.c_float),
        ("x_d0", ctypes.c_float), ("y_d0", ctypes.c_float),
        ("detectorR", ctypes.c_float), ("sourceR", ctypes.c_float),
        ("sourceY", ctypes.c_float),
        ("n_angles", ctypes.c_int32),
    ]


class NrOstrParams(ctypes.Structure):
    """ctypes image of ``nr_ostr_params`` (include/nrgb300.h)."""

    _fields_ = [
        ("subset_num", ctypes.c_int32), ("potential", ctypes.c_int32),
        ("gamma_mode", ctypes.c_int32), ("has_scatter", ctypes.c_int32),
        ("beta", ctypes.c_float), ("delta", ctypes.c_float),
        ("fp_batch", ctypes.c_int32), ("upd_planes", ctypes.c_int32),
        ("fp_stage", ctypes.c_int32), ("upd_tile", ctypes.c_int32),
    ]


class NrSartParams(ctypes.Structure):
    """ctypes image of ``nr_sart_params`` (include/nrgb300.h)."""

    _fields_ = [
        ("subset_num", ctypes.c_int32), ("use_cos", ctypes.c_int32),
        ("regularized", ctypes.c_int32), ("fp_batch", ctypes.c_int32),
        ("upd_planes", ctypes.c_int32), ("lam", ctypes.c_float),
        ("beta", ctypes.c_float), ("delta", ctypes.c_float),
        ("supersample", ctypes.c_int32),
    ]


class NrBatchCase(ctypes.Structure):
    """ctypes image of ``nr_batch_case`` (include/nrgb300.h)."""

    _fields_ = [
        ("g", NrGeom), ("p", NrOstrParams), ("n_iters", ctypes.c_int32),
        ("x", ctypes.c_void_p), ("workspace", ctypes.c_void_p), ("ws_bytes", ctypes.c_size_t),
    ]


POTENTIALS = {"q2": 0, "lange": 1, "hyperbola": 2, "huber": 3}
GAMMA_MODES = {"length": 0, "chord": 1}


@dataclasses.dataclass
class Geometry:
    """Volume grid + detector + source geometry (all lengths in mm)."""

    nx: int
    ny: int
    nz: int
    vx: float
    vy: float
    vz: float
    x_p0: float
    y_p0: float
    z_p0: float
    nbx: int
    nby: int
    bx: float
    by: float
    x_d0: float
    y_d0: float
    detectorR: float
    sourceR: float
    sourceY: float
    n_angles: int

    # Reference spellings (ostr.py:21-52) as read-only aliases.
    IMGSIZx = property(lambda s: s.nx)
    IMGSIZy = property(lambda s: s.ny)
    IMGSIZz = property(lambda s: s.nz)
    Vsize_x = property(lambda s: s.vx)
    Vsize_y = property(lambda s: s.vy)
    Vsize_z = property(lambda s: s.vz)
    BINSx = property(lambda s: s.nbx)
    BINSy = property(lambda s: s.nby)
    Bsize_x = property(lambda s: s.bx)
    Bsize_y = property(lambda s: s.by)
    ANGLES = property(lambda s: s.n_angles)

    @property
    def n_voxels(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def n_bins(self) -> int:
        return self.nbx * self.nby

    @property
    def z_xy_ratio(self) -> float:
        """Vsize_z / Vsize_x, the prior's z weighting (Tomo_OSTR_gold.cpp:380-386)."""
        return self.vz / self.vx

    def to_c(self) -> NrGeom:
        return NrGeom(*(getattr(self, f) for f, _ in NrGeom._fields_))

    def validate(self, subset_num: Optional[int] = None) -> None:
        """Raise ValueError where the reference would print and exit(1)."""
        for f in ("nx", "ny", "nz", "nbx", "nby", "n_angles"):
            if int(getattr(self, f)) <= 0:
                raise ValueError(f"geometry: {f} must be positive")
        for f in ("vx", "vy", "vz", "bx", "by"):
            if not float(getattr(self, f)) > 0:
                raise ValueError(f"geometry: {f} must be positive")
        if self.vx != self.vy:
            # Tomo_OSTR_gold.cpp:380-386
            raise ValueError("geometry: Vsize_x must equal Vsize_y (the prior's z_xy_ratio)")
        if subset_num is not None:
            if subset_num <= 0 or self.n_angles % subset_num != 0:
                # Tomo_OSTR.cu:2627-2630
                raise ValueError("subset_num must divide the number of views")

    @classmethod
    def dbt(cls, nx: int, ny: int, nz: int, voxel_xy: float, voxel_z: float,
            nbx: int, nby: int, bin_size: float, n_angles: int,
            sdd: float = 660.0, support_height: float = 20.0) -> "Geometry":
        """Stationary-detector DBT geometry with the reference's conventions.

        Chest wall at y = 0 with the breast at y < 0 (``y_p0 = -Ny Vy``,
        ``y_d0 = -BINSy By``, as ``ostr.py:33-37``), volume and detector
        centred in x, breast support (z_p0 = 0) and rotation centre
        ``support_height`` above the detector, source ``sdd`` above the
        detector.
        """
        return cls(nx=nx, ny=ny, nz=nz, vx=voxel_xy, vy=voxel_xy, vz=voxel_z,
                   x_p0=-nx * voxel_xy / 2.0, y_p0=-ny * voxel_xy, z_p0=0.0,
                   nbx=nbx, nby=nby, bx=bin_size, by=bin_size,
                   x_d0=-nbx * bin_size / 2.0, y_d0=-nby * bin_size,
                   detectorR=support_height, sourceR=sdd - support_height,
                   sourceY=0.0, n_angles=n_angles)


def view_angles(n_views: int, half_span_deg: float) -> np.ndarray:
    """Evenly spaced float32 view angles (radians) over [-span, +span]."""
    if n_views == 1:
        return np.zeros(1, np.float32)
    deg = np.linspace(-half_span_deg, half_span_deg, n_views)
    return np.radians(deg).astype(np.float32)


@dataclasses.dataclass
class ReconConfig:
    """One workload: geometry, scan statistics, phantom and OSTR settings."""

    name: str
    geom: Geometry
    angles: np.ndarray
    I0: float
    subset_num: int
    iter_num: int
    potential: str
    beta: float
    delta: float
    n_glandular: int
    n_calc: int
    thickness_mm: float
    seed: int = 0


def config(name: str, seed: int = 0) -> ReconConfig:
    """The named workloads.

    ``small``    256x128x24 @ 0.4x0.4x1.0 mm, detector 320x160 @ 0.4 mm,
                 9 views over +-12 deg, I0 1e4, 10 iters x 9 subsets,
                 hyperbola delta 0.002, beta 50 (runs on the CPU oracle).
    ``clinical`` 1024x512x60 @ 0.14x0.14x1.0 mm, detector 1664x832 @ 0.14 mm,
                 25 views over +-25 deg, I0 5e3, 50 iters x 25 subsets,
                 Huber delta 0.003, beta 100.
    ``fullres``  2048x1024x70 @ 0.085x0.085x1.0 mm, detector 3328x1664 @ 0.085 mm,
                 15 views over +-7.5 deg, I0 4e3, hyperbola delta 0.002, beta 200.
    ``tiny``     a seconds-scale case for unit tests.
    """
    if name == "small":
        g = Geometry.dbt(256, 128, 24, 0.4, 1.0, 320, 160, 0.4, 9)
        return ReconConfig(name, g, view_angles(9, 12.0), 1e4, 9, 10, "hyperbola",
                           50.0, 0.002, 30, 10, 24.0, seed)
    if name == "clinical":
        g = Geometry.dbt(1024, 512, 60, 0.14, 1.0, 1664, 832, 0.14, 25)
        return ReconConfig(name, g, view_angles(25, 25.0), 5e3, 25, 50, "huber",
                           100.0, 0.003, 200, 40, 60.0, seed)
    if name == "fullres":
        g = Geometry.dbt(2048, 1024, 70, 0.085, 1.0, 3328, 1664, 0.085, 15)
        return ReconConfig(name, g, view_angles(15, 7.5), 4e3, 15, 50, "hyperbola",
                           200.0, 0.002, 400, 60, 70.0, seed)
    if name == "tiny":
        g = Geometry.dbt(40, 24, 8, 0.8, 1.0, 48, 32, 0.8, 6)
        return ReconConfig(name, g, view_angles(6, 15.0), 1e4, 3, 2, "lange",
                           20.0, 0.01, 4, 2, 8.0, seed)
    raise KeyError(f"unknown workload {name!r}")


CONFIG_NAMES: List[str] = ["tiny", "small", "clinical", "fullres"]


def batch_configs(n_cases: int = 16, seed: int = 0, iter_num: int = 50,
                  scale: float = 1.0) -> List[ReconConfig]:
    """The batched workload: independent cases with uneven thickness and views.

    Per case (seeded): thickness U(30, 80) slices of 1 mm, in-plane size
    U(512, 1024) x U(256, 512) voxels of 0.14 mm, 9, 15 or 25 views over
    +-U(7.5, 25) deg with one view per subset, I0 U(3e3, 2e4), glandular
    fraction U(10 %, 50 %) (the case's n_glandular holds the percentage);
    detector 1664 x 832 of 0.14 mm, hyperbola delta 0.002, beta 50.  `scale`
    shrinks every length in voxels / bins (for tests).
    """
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n_cases):
        nz = int(round(rng.uniform(30, 80) * scale)) or 1
        nx = max(8, int(round(rng.uniform(512, 1024) * scale)))
        ny = max(8, int(round(rng.uniform(256, 512) * scale)))
        views = int(rng.choice([9, 15, 25]))
        span = float(rng.uniform(7.5, 25.0))
        I0 = float(rng.uniform(3e3, 2e4))
        gland = float(rng.uniform(0.10, 0.50))
        g = Geometry.dbt(nx, ny, nz, 0.14, 1.0, max(8, int(round(1664 * scale))),
                         max(8, int(round(832 * scale))), 0.14, views)
        out.append(ReconConfig(f"batch{c}", g, view_angles(views, span), I0, views, iter_num,
                               "hyperbola", 50.0, 0.002, int(round(100 * gland)), 20,
                               float(nz), seed * 1000 + c))
    return out


def geometry_dict(g: Geometry) -> Dict[str, float]:
    return dataclasses.asdict(g)


def isclose_geom(a: Geometry, b: Geometry) -> bool:
    return all(math.isclose(float(getattr(a, f)), float(getattr(b, f)))
               for f, _ in NrGeom._fields_)
