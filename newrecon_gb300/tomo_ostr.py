"""``python -m newrecon_gb300.tomo_ostr <datafile>``: the reference's
``Tomo_OSTR <datafile>`` command on the GPU path.

Reads the parameter file and the per-view raw scans (``datfile``), flips them
to the in-memory layout on the GPU, runs ``Recon_Method`` 0 (OSTR, Q2 prior)
or 1 (OSTR, Lange prior) -- the two methods ``Reconstruction()`` dispatches
(``Tomo_OSTR_gold.cpp:1493-1528``) -- or 3, OS-SART, which the reference
leaves empty there: the scans become line integrals log(blank/(prj-scatter))
and the device-resident OS-SART loop runs with the optional labels
SART_lambda / SART_use_cos / SART_beta (and Delta for the prior).  Every
method starts from the initial guess as stored when it can be read (else 0;
``Tomo_OSTR_gold.cpp:567-589``) and writes the volume every
``Readout_Every_X_Iters`` iterations.  ``Readout_Every_X_Iters`` <= 0 (a
modulo by zero in the reference) writes the last iteration only.
"""
from __future__ import annotations

import sys
import time
from typing import List

import numpy as np
import torch

from . import datfile, native, ostr, sart

METHODS = {0: "q2", 1: "lange", 3: "ossart"}


def run(path: str, log=print) -> List[str]:
    """Runs the reconstruction a parameter file describes; returns the files written."""
    cfg = datfile.load(path)
    if cfg.recon_method not in METHODS:
        # Tomo_OSTR_gold.cpp:1519-1520: method 2 (convex OSEM) is an empty placeholder
        raise datfile.DatFileError(
            f"Recon_Method {cfg.recon_method}: only 0 (OSTR Q2), 1 (OSTR Lange), 3 (OS-SART)")
    g = cfg.geom
    g.validate(cfg.subset_num)
    t0 = time.perf_counter()
    angles = datfile.read_angles(cfg.angle_name, g.n_angles)
    raw = {}
    for key, folder, name in (("prj", cfg.projection_folder, cfg.projection_name),
                              ("scat", cfg.scatter_folder, cfg.scatter_name),
                              ("blank", cfg.blank_folder, cfg.blank_name)):
        views = datfile.read_views(folder, name, g.n_angles, g.nbx, g.nby)
        t = torch.from_numpy(views.ravel()).cuda()
        flipped = torch.empty_like(t)
        native.call("nr_x_y_flip", ostr._p(flipped), ostr._p(t), g.nbx, g.nby, g.n_angles,
                    ostr._stream())
        raw[key] = flipped
    if cfg.recon_method == 3:
        plan = sart.OSSART(g, subset_num=cfg.subset_num, lam=cfg.sart_lambda,
                           use_cos=bool(cfg.sart_use_cos), regularized=cfg.sart_beta != 0,
                           beta=cfg.sart_beta, delta=cfg.delta)
        plan.setup(angles, sart.line_integrals(raw["prj"], raw["blank"], raw["scat"]))
    else:
        plan = ostr.OSTR(g, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                         potential=METHODS[cfg.recon_method], has_scatter=True)
        plan.setup(angles, raw["prj"], raw["blank"], raw["scat"])
    x0 = datfile.read_volume(cfg.ini_guess, g.n_voxels)
    x = (torch.zeros(g.n_voxels, device="cuda") if x0 is None
         else torch.from_numpy(x0).cuda())
    written = []
    step = cfg.io_iter if cfg.io_iter > 0 else cfg.iter_num
    done = 0
    while done < cfg.iter_num:
        n = min(step, cfg.iter_num - done)
        plan.iterate(x, n)
        done += n
        plan.check()
        if cfg.io_iter <= 0 and done < cfg.iter_num:
            continue
        if cfg.io_iter > 0 and done % cfg.io_iter != 0:
            continue
        fn = datfile.output_filename(cfg, done - 1)
        x.cpu().numpy().astype(np.float32).tofile(fn)
        written.append(fn)
        log(f"iteration {done}: wrote {fn}")
    torch.cuda.synchronize()
    log(f"Recon successfully done!! ({time.perf_counter() - t0:.2f} s)")
    return written


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("Please ONLY enter the name of datafile!")
        return 1
    native.load()
    run(argv[0])
    return 0


if __name__ == "__main__":
    sys.exit(main())
