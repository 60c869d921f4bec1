"""The reference's parameter file and raw data files.

``Tomo_OSTR <datafile>`` (``Tomo_OSTR.cu:2561-2702``) reads a whitespace-separated
key/value file with the label-search parsers of ``readdata.cu:54-439`` and the
per-view raw float32 files of ``Tomo_OSTR_gold.cpp:33-179``.  This module reads
and writes the same files so that existing datasets drive the GPU path
unchanged:

* a label is a whitespace token; its value(s) are the following token(s);
  the first occurrence wins; a missing label, or a numeric value that is "#"
  or starts with a letter, is an error (the reference prints and exit(1)s:
  here ``DatFileError``); integers convert like C ``atoi``, floats like ``atof``;
* projection / scatter / blank scans are one file per view named
  ``folder + name + NNNN`` with NNNN = view + 1 zero-padded to 4 digits
  (``Tomo_OSTR_gold.cpp:141-155``), each ``[BINSy][BINSx]`` float32 (the
  scanner layout; ``x_y_flip`` turns it into the in-memory ``[i][j]``); a
  missing file is an error as in the reference, and so is a short one, which
  the reference would read as far as it goes and zero-fill;
* the angle file holds ANGLES float32 radians; the initial guess and the
  outputs are raw float32 ``[z][y][x]`` volumes; output k is written to
  ``output_recon_folder + output_recon_name + str(k)`` after iteration k+1
  when (k+1) % Readout_Every_X_Iters == 0 (``Tomo_OSTR_gold.cpp:870-885``).
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import List, Optional

import numpy as np

from .geometry import Geometry


class DatFileError(ValueError):
    """A parameter the reference's parser would reject (it exits)."""


def _tokens(path: str) -> List[str]:
    with open(path, "r", errors="replace") as f:
        return f.read().split()


def _find(toks: List[str], label: str, n: int, path: str) -> List[str]:
    for k, t in enumerate(toks):
        if t == label:
            vals = toks[k + 1:k + 1 + n]
            if len(vals) < n:
                break
            return vals
    raise DatFileError(f'The parameter label "{label}" wasn\'t found in the file "{path}"')


def _check_numeric(vals: List[str], label: str, path: str) -> None:
    for v in vals:
        if v == "#" or (v and v[0].isalpha()):
            raise DatFileError(f'Something wrong in the {path} about this label "{label}"')


def _atoi(s: str) -> int:
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


def _atof(s: str) -> float:
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|inf|nan)", s, re.I)
    return float(m.group(0)) if m else 0.0


def read_int(path: str, label: str, n: int = 1):
    """readINTEGERpara (readdata.cu:54-118)."""
    vals = _find(_tokens(path), label, n, path)
    _check_numeric(vals, label, path)
    out = [_atoi(v) for v in vals]
    return out[0] if n == 1 else out


def read_float(path: str, label: str, n: int = 1):
    """readFLOATpara (readdata.cu:243-301)."""
    vals = _find(_tokens(path), label, n, path)
    _check_numeric(vals, label, path)
    out = [_atof(v) for v in vals]
    return out[0] if n == 1 else out


def read_string(path: str, label: str) -> str:
    """readSTRINGpara (readdata.cu:168-240): the next token."""
    return _find(_tokens(path), label, 1, path)[0]


def read_optional(path: str, label: str, kind: str, default):
    """An optional parameter: default when the label is absent, else as read_int /
    read_float (a malformed value still raises)."""
    if label not in _tokens(path):
        return default
    return read_int(path, label) if kind == "int" else read_float(path, label)


@dataclasses.dataclass
class DatConfig:
    """Every parameter ``main`` reads (Tomo_OSTR.cu:2578-2650)."""

    geom: Geometry
    beta: float
    delta: float
    iter_num: int
    subset_num: int
    recon_method: int
    io_iter: int
    ini_guess: str
    angle_name: str
    projection_folder: str
    projection_name: str
    scatter_folder: str
    scatter_name: str
    blank_folder: str
    blank_name: str
    output_recon_folder: str
    output_recon_name: str
    launch: dict  # the reference's launch-shape parameters (read, not needed here)
    # OS-SART (Recon_Method 3), optional labels with no reference counterpart:
    # SART_lambda (relaxation, default 1), SART_use_cos (default 1) and
    # SART_beta (prior weight, default 0 = no prior; the prior uses Delta)
    sart_lambda: float = 1.0
    sart_use_cos: int = 1
    sart_beta: float = 0.0


def load(path: str) -> DatConfig:
    if not os.path.isfile(path):
        raise DatFileError("Error: datafile not found!!")
    ri = lambda k: read_int(path, k)
    rf = lambda k: read_float(path, k)
    rs = lambda k: read_string(path, k)
    g = Geometry(nx=ri("image_size_x"), ny=ri("image_size_y"), nz=ri("image_size_z"),
                 vx=rf("Voxel_size_x_mm"), vy=rf("Voxel_size_y_mm"), vz=rf("Voxel_size_z_mm"),
                 x_p0=rf("object_xpos_mm"), y_p0=rf("object_ypos_mm"), z_p0=rf("object_zpos_mm"),
                 nbx=ri("bin_samples_x"), nby=ri("bin_samples_y"),
                 bx=rf("Bin_size_x_mm"), by=rf("Bin_size_y_mm"),
                 x_d0=rf("detector_x0_mm"), y_d0=rf("detector_y0_mm"),
                 detectorR=rf("detector_COR_mm"), sourceR=rf("source_COR_mm"),
                 sourceY=rf("source_Y_shift_mm"), n_angles=ri("angular_samples"))
    launch = {k: ri(k) for k in ("BACKPRJ_ThreX", "BACKPRJ_ThreY", "BACKPRJ_GridX",
                                 "BACKPRJ_GridY", "nBatchXdim", "nBatchBINSx", "nBatchBINSy",
                                 "PRJ_ThreX", "PRJ_ThreY", "PRJ_GridX", "PRJ_GridY")}
    cfg = DatConfig(geom=g, beta=rf("Beta"), delta=rf("Delta"), iter_num=ri("iteration_number"),
                    subset_num=ri("subset_number"), recon_method=ri("Recon_Method"),
                    io_iter=ri("Readout_Every_X_Iters"), ini_guess=rs("ini_guess"),
                    angle_name=rs("angle_name"), projection_folder=rs("projection_folder"),
                    projection_name=rs("projection_name"), scatter_folder=rs("scatter_folder"),
                    scatter_name=rs("scatter_name"), blank_folder=rs("blank_folder"),
                    blank_name=rs("blank_name"), output_recon_folder=rs("output_recon_folder"),
                    output_recon_name=rs("output_recon_name"), launch=launch,
                    sart_lambda=read_optional(path, "SART_lambda", "float", 1.0),
                    sart_use_cos=read_optional(path, "SART_use_cos", "int", 1),
                    sart_beta=read_optional(path, "SART_beta", "float", 0.0))
    if cfg.subset_num <= 0 or g.n_angles % cfg.subset_num != 0:
        # Tomo_OSTR.cu:2627-2630
        raise DatFileError("Error!! subset_number is not a divisor of angular_samples.")
    return cfg


def write(path: str, cfg: DatConfig) -> None:
    """Writes a parameter file the reference's parser (and load) accept."""
    g = cfg.geom
    rows = [("image_size_x", g.nx), ("image_size_y", g.ny), ("image_size_z", g.nz),
            ("Voxel_size_x_mm", g.vx), ("Voxel_size_y_mm", g.vy), ("Voxel_size_z_mm", g.vz),
            ("object_xpos_mm", g.x_p0), ("object_ypos_mm", g.y_p0), ("object_zpos_mm", g.z_p0),
            ("detector_x0_mm", g.x_d0), ("detector_y0_mm", g.y_d0),
            ("detector_COR_mm", g.detectorR), ("source_COR_mm", g.sourceR),
            ("source_Y_shift_mm", g.sourceY), ("angular_samples", g.n_angles),
            ("bin_samples_x", g.nbx), ("bin_samples_y", g.nby),
            ("Bin_size_x_mm", g.bx), ("Bin_size_y_mm", g.by)]
    rows += sorted(cfg.launch.items())
    rows += [("Readout_Every_X_Iters", cfg.io_iter), ("Recon_Method", cfg.recon_method),
             ("Beta", cfg.beta), ("Delta", cfg.delta), ("iteration_number", cfg.iter_num),
             ("subset_number", cfg.subset_num), ("ini_guess", cfg.ini_guess),
             ("angle_name", cfg.angle_name), ("projection_folder", cfg.projection_folder),
             ("projection_name", cfg.projection_name), ("scatter_folder", cfg.scatter_folder),
             ("scatter_name", cfg.scatter_name), ("blank_folder", cfg.blank_folder),
             ("blank_name", cfg.blank_name), ("output_recon_folder", cfg.output_recon_folder),
             ("output_recon_name", cfg.output_recon_name), ("SART_lambda", cfg.sart_lambda),
             ("SART_use_cos", cfg.sart_use_cos), ("SART_beta", cfg.sart_beta)]
    with open(path, "w") as f:
        for k, v in rows:
            f.write(f"{k}\t{v!r}\n" if isinstance(v, float) else f"{k}\t{v}\n")


def view_filename(folder: str, name: str, view: int) -> str:
    """folder + name + (view+1) zero-padded to 4 digits (Tomo_OSTR_gold.cpp:141-155)."""
    return f"{folder}{name}{view + 1:04d}"


def read_views(folder: str, name: str, n_views: int, nbx: int, nby: int) -> np.ndarray:
    """All views in the scanner layout: float32 [view][BINSy][BINSx]."""
    b = nbx * nby
    out = np.empty((n_views, nby, nbx), np.float32)
    for v in range(n_views):
        fn = view_filename(folder, name, v)
        if not os.path.isfile(fn):
            raise DatFileError(f"File {fn} is missing")
        d = np.fromfile(fn, dtype=np.float32, count=b)
        if d.size != b:
            raise DatFileError(f"File {fn} is shorter than {b} floats")
        out[v] = d.reshape(nby, nbx)
    return out


def write_views(folder: str, name: str, views_ji: np.ndarray) -> None:
    """Writes [view][BINSy][BINSx] float32 views in the scanner layout."""
    for v in range(views_ji.shape[0]):
        np.ascontiguousarray(views_ji[v], np.float32).tofile(view_filename(folder, name, v))


def read_angles(path: str, n: int) -> np.ndarray:
    a = np.fromfile(path, dtype=np.float32, count=n)
    if a.size != n:
        raise DatFileError("error in reading h_angles !")
    return a


def read_volume(path: str, n: int) -> Optional[np.ndarray]:
    """The initial guess as load_data reads it (Tomo_OSTR_gold.cpp:33-63, 577-586).

    None when the file cannot be opened (the reference then starts from 0);
    a short file fills the front of the volume and leaves the rest 0.
    """
    if not os.path.isfile(path):
        return None
    a = np.zeros(n, np.float32)
    d = np.fromfile(path, dtype=np.float32, count=n)
    a[:d.size] = d
    return a


def output_filename(cfg: DatConfig, k: int) -> str:
    return f"{cfg.output_recon_folder}{cfg.output_recon_name}{k}"
