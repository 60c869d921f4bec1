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


def test_device_path_refuses_tables_past_32_bits(native):
    """The fused update indexes its back-projection tables (views x planes x
    columns or rows) in 32 bits: the device-resident paths refuse a geometry
    whose tables would hold 2^31 entries or more."""
    from newrecon_gb300.geometry import NrOstrParams, NrSartParams, config

    g = config("tiny").geom
    size = ctypes.c_size_t(0)
    lib = native.load()
    ok = dataclasses.replace(g, nx=4096, ny=1, nz=4096, n_angles=127, nbx=8, nby=8)
    big = dataclasses.replace(ok, n_angles=128)               # 128 * 4096 * 4096 = 2^31
    for geom, want in ((ok, 0), (big, 1)):
        gc = geom.to_c()
        p = NrOstrParams(geom.n_angles, 1, 0, 0, 1.0, 0.002)  # one view per subset
        assert lib.nr_ostr_workspace_size(ctypes.byref(gc), ctypes.byref(p), ctypes.byref(size)) == want
        sp = NrSartParams()
        sp.subset_num = geom.n_angles
        assert lib.nr_sart_workspace_size(ctypes.byref(gc), ctypes.byref(sp), ctypes.byref(size)) == want


def test_contract_names_alias_the_fused_entry_points(native):
    """nr_workspace_size answers as nr_ostr_workspace_size (and refuses what it
    refuses); nr_ostr_subset / nr_objective_fp64 refuse a missing workspace as
    nr_ostr_subiter / nr_ostr_objective do, before any CUDA call."""
    from newrecon_gb300.geometry import NrOstrParams, config

    lib = native.load()
    g = config("small").geom
    gc = g.to_c()
    for m in (1, 3, 9):
        p = NrOstrParams(m, 2, 0, 0, 50.0, 0.002)
        a, b = ctypes.c_size_t(0), ctypes.c_size_t(0)
        assert lib.nr_workspace_size(ctypes.byref(gc), ctypes.byref(p), ctypes.byref(a)) == \
            lib.nr_ostr_workspace_size(ctypes.byref(gc), ctypes.byref(p), ctypes.byref(b))
        assert a.value == b.value
        assert lib.nr_ostr_subset(ctypes.byref(gc), ctypes.byref(p), None, 0, None, 0, None) == \
            lib.nr_ostr_subiter(ctypes.byref(gc), ctypes.byref(p), None, 0, None, 0, None) != 0
        assert lib.nr_objective_fp64(ctypes.byref(gc), ctypes.byref(p), None, None, None, 0, None) == \
            lib.nr_ostr_objective(ctypes.byref(gc), ctypes.byref(p), None, None, None, 0, None) != 0
    p = NrOstrParams(4, 2, 0, 0, 50.0, 0.002)  # 9 views: 4 subsets do not divide them
    a = ctypes.c_size_t(0)
    assert lib.nr_workspace_size(ctypes.byref(gc), ctypes.byref(p), ctypes.byref(a)) == 1


def test_update_tile_choice_is_checked(native):
    """upd_tile takes NR_TILE_1 (0), NR_TILE_2 (1) or NR_TILE_TMA (2); anything
    else is refused."""
    from newrecon_gb300.geometry import NrOstrParams, config

    lib = native.load()
    gc = config("small").geom.to_c()
    size = ctypes.c_size_t(0)
    for tile, ok in ((0, True), (1, True), (2, True), (3, False), (-1, False)):
        p = NrOstrParams(9, 2, 0, 0, 50.0, 0.002)
        p.upd_tile = tile
        st = lib.nr_ostr_workspace_size(ctypes.byref(gc), ctypes.byref(p), ctypes.byref(size))
        assert (st == 0) == ok, (tile, st)
