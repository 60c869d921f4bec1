"""The autotuner's choice among the update variants (host logic, no GPU)."""
from newrecon_gb300 import autotune


def times(one, two):
    """{(tile, planes): ms} from the one-voxel and two-voxel times at 8, 16, 32 planes."""
    out = {(0, z): v for z, v in zip(autotune.UPD_PLANES, one)}
    out.update({(1, z): v for z, v in zip(autotune.UPD_PLANES, two)})
    return out


def test_fastest_one_voxel_variant_wins():
    assert autotune.choose_update(times([6.6, 6.5, 6.7], [6.9, 7.0, 7.1])) == (0, 16)


def test_two_voxel_tile_needs_the_margin():
    # the clinical timings: the two-voxel tile leads by 0.3 %, inside the margin
    assert autotune.choose_update(times([6.61, 6.51, 6.63], [6.50, 6.54, 6.86])) == (0, 16)
    # the full-resolution timings: it leads by 4.7 %
    assert autotune.choose_update(times([18.76, 18.26, 18.04], [17.82, 17.42, 17.19])) == (1, 32)


def test_many_view_subsets_time_only_the_one_voxel_tile():
    one_only = {(0, 8): 3.0, (0, 16): 2.5, (0, 32): 2.7}
    assert autotune.choose_update(one_only) == (0, 16)
