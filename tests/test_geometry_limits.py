"""Geometry validation on the host (no GPU): nr_validate_geometry refuses what
the kernels cannot index.  Voxel and bin indices are 32-bit, so a volume or a
projection set of 2^31 elements or more is refused, as are empty sizes,
non-positive pitches, Vx != Vy (the reference's z_xy_ratio requires it,
Tomo_OSTR_gold.cpp:380-386) and a subset count that does not divide the views."""
import ctypes
import dataclasses

import pytest


@pytest.fixture(scope="module")
def native(native_lib_path):
    from newrecon_gb300 import native

    native.load(native_lib_path)
    return native


def status(native, g, subsets=1):
    gc = g.to_c()
    return native.load().nr_validate_geometry(ctypes.byref(gc), subsets)


def test_size_limits(native):
    from newrecon_gb300.geometry import config

    g = config("tiny").geom
    assert status(native, g) == 0
    ok = dataclasses.replace(g, nx=1024, ny=1024, nz=2047)        # 2^31 - 2^20 voxels
    assert status(native, ok) == 0
    assert status(native, dataclasses.replace(g, nx=1024, ny=1024, nz=2048)) == 1  # 2^31
    assert status(native, dataclasses.replace(g, nbx=4096, nby=4096, n_angles=127)) == 0
    assert status(native, dataclasses.replace(g, nbx=4096, nby=4096, n_angles=128)) == 1


@pytest.mark.parametrize("field,value", [("nx", 0), ("nz", -1), ("nby", 0), ("n_angles", 0),
                                         ("vx", 0.0), ("vz", -1.0), ("bx", 0.0),
                                         ("vy", float("nan"))])
def test_degenerate_geometry_refused(native, field, value):
    from newrecon_gb300.geometry import config

    g = dataclasses.replace(config("tiny").geom, **{field: value})
    assert status(native, g) == 1


def test_pitch_and_subsets(native):
    from newrecon_gb300.geometry import config

    g = config("tiny").geom  # 6 views
    assert status(native, dataclasses.replace(g, vy=g.vx * 1.5)) == 1
    assert status(native, g, 3) == 0
    assert status(native, g, 4) == 1
