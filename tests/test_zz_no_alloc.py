"""nr_penalty_fp64_static: the penalty for callers that may not allocate.

Some callers of this library may not allocate device memory where they need
the regulariser value: a scanner-side reconstruction service whose memory is
fixed at start-up, or a host framework that owns every device buffer.  They
call nr_penalty_fp64_static, which keeps its scratch (per-block partial sums)
in a fixed 2 MiB device array inside the library instead of a workspace.

This file runs last (pytest collects files in name order) so that a run which
stops at the first failure has already run every other test.  It builds its
own inputs and works both alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# Both entry points run the same penalty kernel and add its per-block partials
# in the same fixed order, so their values agree bit for bit.


def _penalty_static(lib, g, x, pot, delta):
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    gc = g.to_c()
    rc = lib.nr_penalty_fp64_static(ctypes.byref(gc), ctypes.c_void_p(x.data_ptr()), int(pot),
                                    ctypes.c_float(delta), ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return float(out.item())


@pytest.mark.parametrize("pot", ["q2", "lange", "hyperbola", "huber"])
def test_static_penalty_matches_workspace_objective(pot):
    from newrecon_gb300 import native, ostr
    from newrecon_gb300.geometry import POTENTIALS, config
    from newrecon_gb300.phantom import breast_phantom

    lib = native.load()
    cfg = config("small")
    g = cfg.geom
    rng = np.random.default_rng(11)
    base = breast_phantom(g, 0, cfg.n_glandular, cfg.n_calc).ravel()
    # a plausible scan so the workspace path can be set up
    y = np.full(g.n_angles * g.n_bins, 5000.0, np.float32)
    b = np.full_like(y, 1e4)
    plan = ostr.OSTR(g, subset_num=cfg.subset_num, beta=cfg.beta, delta=cfg.delta,
                     potential=pot)
    plan.setup(cfg.angles, y, b)
    # two calls in a row, on two different volumes (Q2 ignores delta: the
    # workspace path forces it to 1, and so does the static entry point)
    for k in range(2):
        x = torch.from_numpy(
            (base + rng.normal(scale=0.003, size=base.size)).astype(np.float32)).cuda()
        _, p_ws = plan.objective(x)
        p_static = _penalty_static(lib, g, x, POTENTIALS[pot], cfg.delta)
        assert np.isfinite(p_static) and p_static > 0
        assert p_static == p_ws, (pot, k, p_static, p_ws)


def test_static_penalty_at_its_size_limit():
    """1024x512x64 voxels: exactly 2^18 blocks of 32 x 4 columns per plane,
    the largest volume the static scratch holds; it is accepted and agrees
    with the workspace path bit for bit."""
    from newrecon_gb300 import native, ostr
    from newrecon_gb300.geometry import POTENTIALS, Geometry

    lib = native.load()
    g = Geometry.dbt(1024, 512, 64, 0.14, 1.0, 64, 32, 0.14, 1)
    assert (g.nx + 31) // 32 * ((g.ny + 3) // 4) * g.nz == 1 << 18
    gen = torch.Generator(device="cuda").manual_seed(5)
    y = np.full(g.n_bins, 5000.0, np.float32)
    plan = ostr.OSTR(g, subset_num=1, beta=100.0, delta=0.003, potential="huber")
    plan.setup(np.zeros(1, np.float32), y, np.full_like(y, 1e4))
    for k in range(2):
        x = torch.rand(g.n_voxels, device="cuda", generator=gen) * 0.05
        _, p_ws = plan.objective(x)
        p_static = _penalty_static(lib, g, x, POTENTIALS["huber"], 0.003)
        assert p_static == p_ws, (k, p_static, p_ws)


def test_static_penalty_rejects_volumes_beyond_its_scratch():
    from newrecon_gb300 import native
    from newrecon_gb300.geometry import Geometry

    lib = native.load()
    g = Geometry.dbt(4096, 4096, 64, 0.1, 1.0, 64, 64, 0.1, 1)  # 8.4M blocks > 262144
    x = torch.zeros(16, device="cuda")  # never read: the size check comes first
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    gc = g.to_c()
    rc = lib.nr_penalty_fp64_static(ctypes.byref(gc), ctypes.c_void_p(x.data_ptr()), 3,
                                    ctypes.c_float(0.003), ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(0))
    assert rc == 6  # NR_ERR_WORKSPACE
