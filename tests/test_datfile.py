"""The parameter-file parser and the raw per-view files (CPU only).

The parser follows readdata.cu:54-301 (label search over whitespace tokens,
"#"/alphabetic numeric values rejected, atoi/atof conversion); the files
follow Tomo_OSTR_gold.cpp:108-179 (folder + name + 4-digit view number,
[BINSy][BINSx] per view, x_y_flip to the in-memory [i][j]).
"""
import os

import numpy as np
import pytest

from newrecon_gb300 import datfile
from newrecon_gb300.geometry import config

HERE = os.path.dirname(os.path.abspath(__file__))


def _cfg(tmp, **kw):
    g = config("tiny").geom
    c = datfile.DatConfig(
        geom=g, beta=2.5, delta=0.003, iter_num=3, subset_num=3, recon_method=1, io_iter=2,
        ini_guess=str(tmp / "none"), angle_name=str(tmp / "angles.raw"),
        projection_folder=str(tmp) + "/", projection_name="prj_",
        scatter_folder=str(tmp) + "/", scatter_name="sct_", blank_folder=str(tmp) + "/",
        blank_name="blk_", output_recon_folder=str(tmp) + "/", output_recon_name="rec_",
        launch={k: 16 for k in ("BACKPRJ_ThreX", "BACKPRJ_ThreY", "BACKPRJ_GridX",
                                "BACKPRJ_GridY", "nBatchXdim", "nBatchBINSx", "nBatchBINSy",
                                "PRJ_ThreX", "PRJ_ThreY", "PRJ_GridX", "PRJ_GridY")})
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def test_write_load_round_trip(tmp_path):
    c = _cfg(tmp_path)
    p = tmp_path / "recon.dat"
    datfile.write(str(p), c)
    d = datfile.load(str(p))
    assert d == c


def test_label_search_semantics(tmp_path):
    p = tmp_path / "f.dat"
    p.write_text("# comment  image_size_x\n"
                 "a 12abc  b -7 c 1.5e-3mm  d .25 e +3.  f 4 4 5\n"
                 "a 99\n  s  some/path/\n")
    # the first occurrence of the token wins; "image_size_x" after "#" is a label
    # token too (the reference does not skip comments), so its value is "a"
    with pytest.raises(datfile.DatFileError, match="Something wrong"):
        datfile.read_int(str(p), "image_size_x")
    assert datfile.read_int(str(p), "a") == 12          # atoi stops at the first non-digit
    assert datfile.read_int(str(p), "b") == -7
    assert datfile.read_float(str(p), "c") == pytest.approx(1.5e-3)
    assert datfile.read_float(str(p), "d") == pytest.approx(0.25)
    assert datfile.read_float(str(p), "e") == pytest.approx(3.0)
    assert datfile.read_int(str(p), "f", 3) == [4, 4, 5]
    assert datfile.read_string(str(p), "s") == "some/path/"
    with pytest.raises(datfile.DatFileError, match="wasn't found"):
        datfile.read_int(str(p), "missing")


def test_comment_and_alpha_values_rejected(tmp_path):
    p = tmp_path / "f.dat"
    p.write_text("x # 3\ny abc\nz -\n")
    for label in ("x", "y"):
        with pytest.raises(datfile.DatFileError, match="Something wrong"):
            datfile.read_float(str(p), label)
    # "-" is neither "#" nor alphabetic: accepted, converts to 0 like atoi
    assert datfile.read_int(str(p), "z") == 0
    # strings take the next token, whatever it is
    assert datfile.read_string(str(p), "x") == "#"


def test_subset_must_divide_views(tmp_path):
    p = tmp_path / "bad.dat"
    datfile.write(str(p), _cfg(tmp_path, subset_num=4))  # 6 views
    with pytest.raises(datfile.DatFileError, match="divisor"):
        datfile.load(str(p))
    with pytest.raises(datfile.DatFileError, match="not found"):
        datfile.load(str(tmp_path / "absent.dat"))


def test_view_file_names():
    assert datfile.view_filename("d/", "prj_", 0) == "d/prj_0001"
    assert datfile.view_filename("d/", "prj_", 98) == "d/prj_0099"
    assert datfile.view_filename("", "p", 999) == "p1000"
    assert datfile.view_filename("", "p", 12344) == "p12345"


def test_views_are_scanner_layout(tmp_path):
    """Files hold [BINSy][BINSx]; the reference's x_y_flip of view 0 is the in-memory view."""
    z = np.load(os.path.join(HERE, "golden", "tiny.npz"))
    g = z["geom"]
    nbx, nby, A = int(g[9]), int(g[10]), int(g[18])
    y = z["y"].reshape(A, nbx, nby)
    datfile.write_views(str(tmp_path) + "/", "prj_", y.transpose(0, 2, 1))
    v = datfile.read_views(str(tmp_path) + "/", "prj_", A, nbx, nby)
    # the bytes of view 0 are the reference's x_y_flip input, its output the view
    np.testing.assert_array_equal(v[0].ravel(), z["flip_in"])
    np.testing.assert_array_equal(z["flip"], y[0].ravel())
    np.testing.assert_array_equal(v.transpose(0, 2, 1), y)
    os.remove(datfile.view_filename(str(tmp_path) + "/", "prj_", A - 1))
    with pytest.raises(datfile.DatFileError, match="missing"):
        datfile.read_views(str(tmp_path) + "/", "prj_", A, nbx, nby)
    np.zeros(5, np.float32).tofile(datfile.view_filename(str(tmp_path) + "/", "prj_", A - 1))
    with pytest.raises(datfile.DatFileError, match="shorter"):
        datfile.read_views(str(tmp_path) + "/", "prj_", A, nbx, nby)


def test_angles_and_initial_guess(tmp_path):
    a = np.linspace(-0.2, 0.2, 6).astype(np.float32)
    a.tofile(tmp_path / "ang")
    np.testing.assert_array_equal(datfile.read_angles(str(tmp_path / "ang"), 6), a)
    with pytest.raises(datfile.DatFileError):
        datfile.read_angles(str(tmp_path / "ang"), 7)
    assert datfile.read_volume(str(tmp_path / "nothing"), 10) is None
    short = datfile.read_volume(str(tmp_path / "ang"), 10)  # front filled, rest 0
    np.testing.assert_array_equal(short, np.concatenate([a, np.zeros(4, np.float32)]))
    np.testing.assert_array_equal(datfile.read_volume(str(tmp_path / "ang"), 4), a[:4])
    c = _cfg(tmp_path)
    assert datfile.output_filename(c, 11) == str(tmp_path) + "/rec_11"
