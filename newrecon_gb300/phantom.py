"""Seeded synthetic breast phantoms and transmission scans.

The reference ships no OSTR data (its scanner files live outside the
repository), so every workload here is synthetic and seeded.  The phantom
follows the precedent of ``ReconDBT/gen_dbtproj_example.m:11-14,104-112``
(ellipsoids in a compressed breast, counts ``Poisson(I0 exp(-line))``):

* a compressed half-ellipse breast (semi-axes 90 x 60 mm in x and y, y <= 0,
  full slab thickness) of adipose tissue, mu = 0.0456 /mm;
* randomly oriented fibroglandular ellipsoids, mu = 0.0802 /mm,
  semi-axes U(2, 12) mm, centred inside the breast;
* calcification spheres, mu = 2.0 /mm, diameter U(0.2, 0.6) mm, sampled with
  sub-voxel supersampling so partial volume is kept;
* air (0) elsewhere.

The phantom is generated on the reconstruction grid and clipped to it, so
the forward model that makes the counts is the one the reconstruction uses.
"""
from __future__ import annotations

import numpy as np

from .geometry import Geometry

MU_ADIPOSE = 0.0456
MU_GLANDULAR = 0.0802
MU_CALC = 2.0


def _centres(n: int, v: float, p0: float) -> np.ndarray:
    return (np.arange(n, dtype=np.float64) + 0.5) * v + p0


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
    ])


def breast_phantom(g: Geometry, seed: int, n_glandular: int, n_calc: int,
                   thickness_mm: float | None = None,
                   glandular_fraction: float | None = None) -> np.ndarray:
    """Float32 volume ``[z][y][x]`` in 1/mm.

    ``glandular_fraction`` (0..1), when given, replaces ``n_glandular`` by
    adding ellipsoids until that fraction of the breast is glandular.
    """
    rng = np.random.default_rng(seed)
    xs = _centres(g.nx, g.vx, g.x_p0)
    ys = _centres(g.ny, g.vy, g.y_p0)
    zs = _centres(g.nz, g.vz, g.z_p0)
    thick = g.nz * g.vz if thickness_mm is None else min(thickness_mm, g.nz * g.vz)
    z_lo = g.z_p0
    z_hi = g.z_p0 + thick
    ax, ay = 90.0, 60.0
    breast2d = ((xs[None, :] / ax) ** 2 + (ys[:, None] / ay) ** 2 <= 1.0) & (ys[:, None] <= 0.0)
    zin = (zs >= z_lo) & (zs <= z_hi)
    vol = np.zeros((g.nz, g.ny, g.nx), np.float32)
    vol[zin] = np.where(breast2d, MU_ADIPOSE, 0.0).astype(np.float32)
    breast_vox = int(breast2d.sum()) * int(zin.sum())

    def inside_breast(p):
        return (p[0] / ax) ** 2 + (p[1] / ay) ** 2 <= 1.0 and p[1] <= 0.0

    # Centres are drawn within the part of the breast the grid covers.
    x_lo, x_hi = g.x_p0, g.x_p0 + g.nx * g.vx
    y_lo, y_hi = g.y_p0, min(0.0, g.y_p0 + g.ny * g.vy)

    def draw_centre():
        for _ in range(1000):
            p = np.array([rng.uniform(x_lo, x_hi), rng.uniform(y_lo, y_hi),
                          rng.uniform(z_lo, z_hi)])
            if inside_breast(p):
                return p
        return np.array([0.5 * (x_lo + x_hi), 0.5 * (y_lo + y_hi), 0.5 * (z_lo + z_hi)])

    def stamp_ellipsoid(c, semi, rot, mu):
        r = float(max(semi))
        ix0 = max(0, int(np.floor((c[0] - r - g.x_p0) / g.vx)))
        ix1 = min(g.nx, int(np.ceil((c[0] + r - g.x_p0) / g.vx)) + 1)
        iy0 = max(0, int(np.floor((c[1] - r - g.y_p0) / g.vy)))
        iy1 = min(g.ny, int(np.ceil((c[1] + r - g.y_p0) / g.vy)) + 1)
        iz0 = max(0, int(np.floor((c[2] - r - g.z_p0) / g.vz)))
        iz1 = min(g.nz, int(np.ceil((c[2] + r - g.z_p0) / g.vz)) + 1)
        if ix0 >= ix1 or iy0 >= iy1 or iz0 >= iz1:
            return 0
        X = xs[ix0:ix1][None, None, :] - c[0]
        Y = ys[iy0:iy1][None, :, None] - c[1]
        Z = zs[iz0:iz1][:, None, None] - c[2]
        # body coordinates u = R^T (p - c)
        u = (rot[0, 0] * X + rot[1, 0] * Y + rot[2, 0] * Z) / semi[0]
        v = (rot[0, 1] * X + rot[1, 1] * Y + rot[2, 1] * Z) / semi[1]
        w = (rot[0, 2] * X + rot[1, 2] * Y + rot[2, 2] * Z) / semi[2]
        m = (u * u + v * v + w * w <= 1.0)
        sub = vol[iz0:iz1, iy0:iy1, ix0:ix1]
        m &= sub > 0  # stays inside the breast
        newly = int(np.count_nonzero(m & (sub != mu)))
        sub[m] = mu
        return newly

    if glandular_fraction is None:
        for _ in range(n_glandular):
            stamp_ellipsoid(draw_centre(), rng.uniform(2.0, 12.0, size=3),
                            _random_rotation(rng), MU_GLANDULAR)
    else:
        target = glandular_fraction * breast_vox
        got = 0
        for _ in range(100000):
            if got >= target:
                break
            got += stamp_ellipsoid(draw_centre(), rng.uniform(2.0, 12.0, size=3),
                                   _random_rotation(rng), MU_GLANDULAR)

    # Calcifications with 4x4x4 supersampling of each voxel they touch.
    ss = 4
    off = (np.arange(ss) + 0.5) / ss - 0.5
    for _ in range(n_calc):
        c = draw_centre()
        rad = 0.5 * rng.uniform(0.2, 0.6)
        ix0 = max(0, int(np.floor((c[0] - rad - g.x_p0) / g.vx)))
        ix1 = min(g.nx, int(np.floor((c[0] + rad - g.x_p0) / g.vx)) + 1)
        iy0 = max(0, int(np.floor((c[1] - rad - g.y_p0) / g.vy)))
        iy1 = min(g.ny, int(np.floor((c[1] + rad - g.y_p0) / g.vy)) + 1)
        iz0 = max(0, int(np.floor((c[2] - rad - g.z_p0) / g.vz)))
        iz1 = min(g.nz, int(np.floor((c[2] + rad - g.z_p0) / g.vz)) + 1)
        for iz in range(iz0, iz1):
            pz = zs[iz] + off * g.vz
            for iy in range(iy0, iy1):
                py = ys[iy] + off * g.vy
                for ix in range(ix0, ix1):
                    px = xs[ix] + off * g.vx
                    d2 = ((px[None, None, :] - c[0]) ** 2 + (py[None, :, None] - c[1]) ** 2
                          + (pz[:, None, None] - c[2]) ** 2)
                    frac = float(np.mean(d2 <= rad * rad))
                    if frac > 0:
                        base = float(vol[iz, iy, ix])
                        vol[iz, iy, ix] = np.float32(base + frac * (MU_CALC - base))
    return vol


def poisson_counts(line: np.ndarray, I0: float, seed: int) -> np.ndarray:
    """Transmission counts ``y ~ Poisson(I0 exp(-line))`` as float32."""
    rng = np.random.default_rng(seed + 0x5EED)
    lam = I0 * np.exp(-line.astype(np.float64))
    return rng.poisson(lam).astype(np.float32)
