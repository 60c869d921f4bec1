"""``python -m newrecon_gb300.tomo_ostr <datafile>`` end to end on the GPU.

The golden tiny/ragged scans are written as the reference's files (a
parameter file, an angle file, per-view [BINSy][BINSx] scans), the command
runs, and its outputs are compared with the reference gold driver's
Reconstruction() of the same scans (Lange and Q2), to the fused path's bar.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
LAUNCH = ("BACKPRJ_ThreX", "BACKPRJ_ThreY", "BACKPRJ_GridX", "BACKPRJ_GridY", "nBatchXdim",
          "nBatchBINSx", "nBatchBINSy", "PRJ_ThreX", "PRJ_ThreY", "PRJ_GridX", "PRJ_GridY")


def rel_rmse(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30)


def _write_case(tmp, z, method, io_iter):
    from newrecon_gb300 import datfile
    from newrecon_gb300.geometry import Geometry, NrGeom

    g = Geometry(**{f: int(v) if t.__name__.startswith("c_int") else float(np.float32(v))
                    for (f, t), v in zip(NrGeom._fields_, z["geom"])})
    A = g.n_angles
    d = str(tmp) + "/"
    for name, arr in (("prj_", z["y"]), ("sct_", z["s"]), ("blk_", z["b"])):
        datfile.write_views(d, name, arr.reshape(A, g.nbx, g.nby).transpose(0, 2, 1))
    z["angles"].astype(np.float32).tofile(d + "angles.raw")
    cfg = datfile.DatConfig(
        geom=g, beta=float(z["beta"]), delta=float(z["delta"]), iter_num=int(z["iters"]),
        subset_num=int(z["subset_num"]), recon_method=method, io_iter=io_iter,
        ini_guess=d + "no_initial_guess", angle_name=d + "angles.raw",
        projection_folder=d, projection_name="prj_", scatter_folder=d, scatter_name="sct_",
        blank_folder=d, blank_name="blk_", output_recon_folder=d, output_recon_name="rec_",
        launch={k: 16 for k in LAUNCH})
    datfile.write(d + "recon.dat", cfg)
    return cfg, d + "recon.dat"


@pytest.mark.parametrize("name", ["tiny", "ragged"])
@pytest.mark.parametrize("method,key", [(1, "recon_lange"), (0, "recon_q2")])
def test_datafile_command_matches_gold_driver(tmp_path, name, method, key):
    from newrecon_gb300 import native, tomo_ostr

    native.load()
    z = dict(np.load(os.path.join(HERE, "golden", f"{name}.npz")))
    iters = int(z["iters"])
    cfg, path = _write_case(tmp_path, z, method, io_iter=1)
    written = tomo_ostr.run(path, log=lambda *_: None)
    # Readout_Every_X_Iters = 1: one file per iteration, named by the 0-based iteration
    assert written == [str(tmp_path) + f"/rec_{k}" for k in range(iters)]
    out = np.fromfile(written[-1], dtype=np.float32)
    r = rel_rmse(out, z[key])
    print(f"{name}/method {method} vs gold driver: rel RMSE {r:.2e}")
    assert r < 1e-4
    assert (out >= 0).all()


@pytest.mark.parametrize("name", ["tiny", "ragged"])
def test_datafile_ossart_matches_reference_kernels(tmp_path, name):
    """Recon_Method 3 runs OS-SART on the log of the scans; against the OS-SART
    loop composed from the reference's SART kernels on the same line integrals."""
    from newrecon_gb300 import native, tomo_ostr

    native.load()
    z = dict(np.load(os.path.join(HERE, "golden", f"{name}.npz")))
    zs = np.load(os.path.join(HERE, "golden", f"sart_{name}.npz"))
    z["iters"] = zs["iters"]
    z["delta"] = zs["delta"]
    cfg, path = _write_case(tmp_path, z, 3, io_iter=0)
    cfg.sart_lambda = float(zs["lam"])
    cfg.sart_beta = float(zs["beta"])
    from newrecon_gb300 import datfile

    datfile.write(path, cfg)
    written = tomo_ostr.run(path, log=lambda *_: None)
    assert written == [str(tmp_path) + f"/rec_{int(zs['iters']) - 1}"]
    out = np.fromfile(written[-1], dtype=np.float32)
    r = rel_rmse(out, zs["ossart_reg"])
    print(f"{name}/OS-SART vs reference kernels: rel RMSE {r:.2e}")
    assert r < 1e-4


def test_initial_guess_and_readout_period(tmp_path):
    """An initial guess file is read; with a period of 2 only every 2nd iteration is written."""
    from newrecon_gb300 import native, ostr, tomo_ostr

    native.load()
    z = dict(np.load(os.path.join(HERE, "golden", "tiny.npz")))
    z["iters"] = np.int32(4)
    cfg, path = _write_case(tmp_path, z, 1, io_iter=2)
    x0 = np.random.default_rng(3).uniform(0, 0.05, size=cfg.geom.n_voxels).astype(np.float32)
    x0.tofile(cfg.ini_guess)
    written = tomo_ostr.run(path, log=lambda *_: None)
    assert written == [str(tmp_path) + "/rec_1", str(tmp_path) + "/rec_3"]
    out = np.fromfile(written[-1], dtype=np.float32)
    ref = ostr.reconstruct(cfg.geom, z["y"], z["b"], z["s"], angles=z["angles"],
                           subset_num=cfg.subset_num, iter_num=4, beta=cfg.beta,
                           delta=cfg.delta, potential="lange", x0=x0)
    assert rel_rmse(out, ref) < 1e-6
