"""Generates the golden fixtures of the OSTR path from the reference's own code.

Runs the CPU build of the reference (oracle/build_ref.sh compiles the kernel
bodies of Tomo_OSTR.cu and the gold driver Tomo_OSTR_gold.cpp from the
reference sources) on seeded inputs and stores inputs + outputs as .npz:

    python tests/golden/make_golden.py            # needs the reference sources
    python tests/golden/make_golden.py --sart     # the SART fixtures only

Fixtures (all float32 unless noted):

``tiny.npz``    40x24x8 volume, 48x32 detector, 6 views, 3 subsets: FP_cos,
                gamma (length), SBP, Lange/Q2 priors, hyperbola gradient,
                yry, h, update_est, regroup, x_y_flip, and Reconstruction()
                for Lange (method 1) and Q2 (method 0), 2 iterations.
``ragged.npz``  33x17x5 volume, 41x23 detector, 4 views, 2 subsets, non-zero
                scatter, random volume: the same set on odd sizes.
``small.npz``   the 256x128x24 / 320x160 / 9-view workload: gold-driver
                Lange reconstruction, 10 iterations x 9 subsets, stored as
                per-slice sums plus 8192 seeded voxel samples (the full volume
                is 3 MB), and FP_cos of the phantom for view 0 sampled the
                same way.
``sart_tiny.npz``, ``sart_ragged.npz``
                the SART family on the tiny and ragged cases: the SART
                projector (plain and cos), the projection difference, the SART
                prior, both OS-SART back projections, OS-SART loops
                composed from the reference's own launch wrappers, and the
                4R sub-rays of the reference's kernel with their merge.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from newrecon_gb300.geometry import Geometry, config, view_angles  # noqa: E402
from newrecon_gb300.phantom import breast_phantom, poisson_counts  # noqa: E402
from oracle.oracle import Oracle, Reference  # noqa: E402


def _geom_arr(g: Geometry) -> np.ndarray:
    return np.array([getattr(g, f) for f, _ in g.to_c()._fields_], np.float64)


def full_set(name: str, g: Geometry, angles, subset_num, beta, delta, x, y, b, s, iters):
    R = Reference()
    R.set_geometry(g, subset_num, beta, delta)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    rng = np.random.default_rng(1234)
    out = dict(geom=_geom_arr(g), angles=angles, subset_num=np.int32(subset_num),
               beta=np.float32(beta), delta=np.float32(delta), iters=np.int32(iters),
               x=x, y=y, b=b, s=s)
    out["fp_cos"] = R.fp_ostr_cos(x, angles, idx, 0, A)
    # a subset range on the reordered index, as the driver uses it
    ridx = Oracle(np.float64).reorder_index(A, subset_num)
    Vs = A // subset_num
    out["ridx"] = ridx
    out["fp_cos_sub1"] = R.fp_ostr_cos(x, angles, ridx, Vs, 2 * Vs)
    out["gamma_length"] = R.fp_normprj(angles, idx, 0, A)
    h = rng.normal(size=A * g.n_bins).astype(np.float32)
    out["bp_in"] = h
    out["bp"] = R.bp_sbp(h, idx, angles, 0, A)
    out["bp_sub1"] = R.bp_sbp(h[: Vs * g.n_bins], ridx, angles, Vs, 2 * Vs)
    out["lange_RDD"], out["lange_RD"] = R.prior_lange(x, delta, g.z_xy_ratio)
    out["q2_RDD"], out["q2_RD"] = R.prior_q2(x, g.z_xy_ratio)
    out["hyp_grad"] = R.prior_hyperbola_grad(x, delta)
    out["yry"] = R.compute_yry(y, s)
    line = out["fp_cos"]
    out["h"] = R.compute_h(y, b, line, s)
    capL = rng.normal(size=g.n_voxels).astype(np.float32)
    d = np.abs(rng.normal(size=g.n_voxels)).astype(np.float32) + 1.0
    out["upd_capL"], out["upd_d"] = capL, d
    out["upd"] = R.update_est(x, capL, out["lange_RD"], d, out["lange_RDD"])
    out["regroup_y"] = R.regroup_prj(y)
    view0_ji = np.ascontiguousarray(y.reshape(A, g.nbx, g.nby)[0].T).ravel()
    out["flip_in"] = view0_ji
    out["flip"] = R.x_y_flip(view0_ji)
    out["recon_lange"] = R.reconstruct(angles, y, b, s, method=1, subset_num=subset_num,
                                       iter_num=iters, beta=beta, delta=delta)
    out["recon_q2"] = R.reconstruct(angles, y, b, s, method=0, subset_num=subset_num,
                                    iter_num=iters, beta=beta, delta=delta)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"wrote {name}.npz")


def sart_set(name: str, g: Geometry, angles, subset_num, x, y, b, s, lam, beta, delta, iters):
    """The SART family from the reference's own kernels (Tomo_OSTR.cu:1177-1311,
    1737-2183 through its launch wrappers), and OS-SART loops composed from
    them (the reference has no OS-SART driver)."""
    R = Reference()
    R.set_geometry(g, subset_num, 0.0, delta)
    A = g.n_angles
    idx = np.arange(A, dtype=np.int32)
    ridx = Oracle(np.float64).reorder_index(A, subset_num)
    Vs = A // subset_num
    rng = np.random.default_rng(4321)
    nu = y.astype(np.float64) - s
    line = np.where((nu > 0) & (b > 0), np.log(np.maximum(b, 1e-30) / np.maximum(nu, 1e-30)),
                    0.0).astype(np.float32)
    out = dict(geom=_geom_arr(g), angles=angles, subset_num=np.int32(subset_num),
               lam=np.float32(lam), beta=np.float32(beta), delta=np.float32(delta),
               iters=np.int32(iters), x=x, line=line)
    out["fp_est"], out["fp_norm"] = R.fp_sart(x, angles, idx, 0, A, False)
    out["fpc_est"], out["fpc_norm"] = R.fp_sart(x, angles, idx, 0, A, True)
    e1, n1 = R.fp_sart(x, angles, ridx, Vs, 2 * Vs, True)
    out["fpc_sub1_est"], out["fpc_sub1_norm"] = e1, n1
    out["diff_sub1"] = R.sart_prj_diff(line.reshape(A, -1)[ridx[Vs:2 * Vs]].ravel(), e1, n1,
                                       ridx, Vs, 2 * Vs)
    out["prior"] = R.prior_sart(x, delta)
    dif = (rng.normal(size=Vs * g.n_bins) * 0.01).astype(np.float32)
    out["bp_in"] = dif
    out["bp_plain"] = R.bp_ossart(x, dif, ridx, angles, Vs, 2 * Vs, lam)
    out["bp_reg"] = R.bp_ossart(x, dif, ridx, angles, Vs, 2 * Vs, lam, out["prior"], beta)
    # the 4R sub-rays from the reference's kernel; the merge as intended
    # (Tomo_OSTR.cu:1517-1550 with its fourth index assigned), in float32
    sub = R.fp_4r_subrays(x, angles, idx, 0, A).reshape(A, 2 * g.nby, 2 * g.nbx)
    out["fp4r_sub"] = sub.ravel()
    s00, s10 = sub[:, 0::2, 0::2], sub[:, 0::2, 1::2]
    s01, s11 = sub[:, 1::2, 0::2], sub[:, 1::2, 1::2]
    out["fp4r_merged_ji"] = ((((s00 + s10) + s01) + s11) / np.float32(4)).astype(np.float32).ravel()
    out["ossart"] = R.ossart(angles, line, subset_num=subset_num, iter_num=iters, lam=lam,
                             use_cos=True)
    out["ossart_nocos"] = R.ossart(angles, line, subset_num=subset_num, iter_num=iters, lam=lam,
                                   use_cos=False)
    out["ossart_reg"] = R.ossart(angles, line, subset_num=subset_num, iter_num=iters, lam=lam,
                                 use_cos=True, regularized=True, beta=beta, delta=delta)
    np.savez_compressed(os.path.join(HERE, f"sart_{name}.npz"), **out)
    print(f"wrote sart_{name}.npz")


def main() -> None:
    if "--sart" in sys.argv:
        sart_main()
        return
    # tiny: the phantom, its Poisson scan, no scatter
    cfg = config("tiny")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = Oracle(np.float64).fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles)
    y = poisson_counts(line, cfg.I0, 0)
    b = np.full_like(y, cfg.I0)
    s = np.zeros_like(y)
    full_set("tiny", g, cfg.angles, cfg.subset_num, cfg.beta, cfg.delta, x, y, b, s, cfg.iter_num)

    # ragged: odd sizes, off-centre detector, random volume, scatter
    g = Geometry(nx=33, ny=17, nz=5, vx=0.7, vy=0.7, vz=1.3, x_p0=-11.0, y_p0=-12.5,
                 z_p0=1.0, nbx=41, nby=23, bx=0.9, by=0.8, x_d0=-19.0, y_d0=-17.0,
                 detectorR=25.0, sourceR=600.0, sourceY=-3.0, n_angles=4)
    rng = np.random.default_rng(7)
    angles = view_angles(4, 20.0)
    x = (rng.uniform(0.0, 0.1, size=g.n_voxels)).astype(np.float32)
    x[rng.uniform(size=x.size) < 0.05] = 0.0
    line = Oracle(np.float64).fp_ostr(g, x, angles, np.arange(4, dtype=np.int32), 0, 4)
    y = poisson_counts(line, 3000.0, 3)
    b = rng.uniform(2800.0, 3200.0, size=y.size).astype(np.float32)
    s = rng.uniform(0.0, 60.0, size=y.size).astype(np.float32)
    y[rng.uniform(size=y.size) < 0.01] = 0.0
    full_set("ragged", g, angles, 2, 5.0, 0.02, x, y, b, s, 2)

    # small: the 256x128x24 workload, sampled outputs
    cfg = config("small")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    idx = np.arange(g.n_angles, dtype=np.int32)
    O = Oracle(np.float64)
    line = O.fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles)
    y = poisson_counts(line, cfg.I0, 0)
    b = np.full_like(y, cfg.I0)
    s = np.zeros_like(y)
    R = Reference()
    R.set_geometry(g, cfg.subset_num, cfg.beta, cfg.delta)
    fp0 = R.fp_ostr_cos(x, cfg.angles, idx, 0, 1)
    rec = R.reconstruct(cfg.angles, y, b, s, method=1, subset_num=cfg.subset_num,
                        iter_num=cfg.iter_num, beta=cfg.beta, delta=cfg.delta)
    rng = np.random.default_rng(99)
    vs = np.sort(rng.choice(g.n_voxels, 8192, replace=False)).astype(np.int64)
    bs = np.sort(rng.choice(g.n_bins, 8192, replace=False)).astype(np.int64)
    np.savez_compressed(
        os.path.join(HERE, "small.npz"), geom=_geom_arr(g), seed=np.int32(0),
        recon_lange_slice_sums=rec.reshape(g.nz, -1).astype(np.float64).sum(axis=1),
        recon_lange_idx=vs, recon_lange_val=rec[vs],
        fp0_idx=bs, fp0_val=fp0[bs], fp0_sum=np.float64(fp0.astype(np.float64).sum()),
        phantom_sum=np.float64(x.astype(np.float64).sum()),
        counts_sum=np.float64(y.astype(np.float64).sum()))
    print("wrote small.npz")


def sart_main() -> None:
    # tiny: the phantom and its Poisson scan
    cfg = config("tiny")
    g = cfg.geom
    x = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = Oracle(np.float64).fp_ostr(g, x, cfg.angles, idx, 0, g.n_angles)
    y = poisson_counts(line, cfg.I0, 0)
    b = np.full_like(y, cfg.I0)
    s = np.zeros_like(y)
    sart_set("tiny", g, cfg.angles, cfg.subset_num, x, y, b, s, 0.8, -0.2, 0.01, 3)
    # ragged: odd sizes, off-centre detector, scatter, dead bins
    g = Geometry(nx=33, ny=17, nz=5, vx=0.7, vy=0.7, vz=1.3, x_p0=-11.0, y_p0=-12.5,
                 z_p0=1.0, nbx=41, nby=23, bx=0.9, by=0.8, x_d0=-19.0, y_d0=-17.0,
                 detectorR=25.0, sourceR=600.0, sourceY=-3.0, n_angles=4)
    rng = np.random.default_rng(7)
    angles = view_angles(4, 20.0)
    x = (rng.uniform(0.0, 0.1, size=g.n_voxels)).astype(np.float32)
    x[rng.uniform(size=x.size) < 0.05] = 0.0
    line = Oracle(np.float64).fp_ostr(g, x, angles, np.arange(4, dtype=np.int32), 0, 4)
    y = poisson_counts(line, 3000.0, 3)
    b = rng.uniform(2800.0, 3200.0, size=y.size).astype(np.float32)
    s = rng.uniform(0.0, 60.0, size=y.size).astype(np.float32)
    y[rng.uniform(size=y.size) < 0.01] = 0.0
    sart_set("ragged", g, angles, 2, x, y, b, s, 0.5, -0.2, 0.02, 2)


if __name__ == "__main__":
    main()
