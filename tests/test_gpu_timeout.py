"""The bounded-wait failure paths, run on the GPU without a real expiry.

nr_test_expire_wait sets a workspace's test hook: the chosen wait of every
block reports that it gave up once it has in fact succeeded, so nothing is
in flight when the failure path runs.  Each test checks that the host reads
NR_ERR_TIMEOUT, that the flag is cleared by the check, and that the next
call on the same workspace works (for the convolution: that the failure
path released its tensor memory, or the next launch could not allocate).
No GPU wait is left to run out and no fault is provoked.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NR_ERR_TIMEOUT = 5


@pytest.fixture(scope="module")
def mod():
    from newrecon_gb300 import native, ostr

    native.load()
    return ostr


def expire(ws: torch.Tensor, wait_index: int) -> None:
    from newrecon_gb300 import native

    native.call("nr_test_expire_wait", ctypes.c_void_p(ws.data_ptr()), int(wait_index),
                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def scan(mod, g, angles, seed=3, I0=1e4):
    from newrecon_gb300.phantom import poisson_counts

    rng = np.random.default_rng(seed)
    x = (rng.random(g.n_voxels, dtype=np.float32) * 0.05).astype(np.float32)
    mod.set_geometry(g)
    idx = np.arange(g.n_angles, dtype=np.int32)
    line = torch.zeros(g.n_angles * g.n_bins, device="cuda")
    mod.fprojectCB_1R_GPU_OSTR_cos(torch.from_numpy(x).cuda(), line,
                                   torch.from_numpy(angles).cuda(),
                                   torch.from_numpy(idx).cuda(), 0, g.n_angles)
    y = poisson_counts(line.cpu().numpy(), I0, seed)
    return torch.from_numpy(y).cuda(), torch.full((y.size,), I0, device="cuda")


def plan_for(mod, g, angles, y, b, **kw):
    plan = mod.OSTR(g, subset_num=g.n_angles, beta=20.0, delta=0.01, potential="huber", **kw)
    plan.setup(angles, y, b)
    return plan


@pytest.mark.parametrize("at", [0, 2, 5])
def test_update_ring_expiry_is_reported_and_recovers(mod, at):
    """The TMA-fed update: a consumer wait that gives up flags the timeout;
    the check reports it and clears it, and the next iterations on the same
    workspace give the reference result."""
    from newrecon_gb300.geometry import Geometry, view_angles
    from newrecon_gb300.native import NrError

    g = Geometry.dbt(96, 20, 18, 0.5, 1.0, 110, 26, 0.5, 6)
    angles = view_angles(6, 15.0)
    y, b = scan(mod, g, angles)
    plan = plan_for(mod, g, angles, y, b, upd_tile=2)
    x = torch.zeros(g.n_voxels, device="cuda")
    expire(plan.ws, at)
    plan.iterate(x, 1)
    with pytest.raises(NrError) as e:
        plan.check()
    assert e.value.code == NR_ERR_TIMEOUT
    assert plan.check() == 0  # the flag and the hook are cleared
    x1 = torch.zeros(g.n_voxels, device="cuda")
    plan.iterate(x1, 2)
    assert plan.check() == 0
    ref = plan_for(mod, g, angles, y, b, upd_tile=0)
    x2 = torch.zeros(g.n_voxels, device="cuda")
    ref.iterate(x2, 2)
    torch.cuda.synchronize()
    assert torch.equal(x1, x2)


def test_staged_projection_expiry_falls_back_to_global_reads(mod):
    """The TMA-staged projection: after a slab wait gives up the block walks
    the rest from global memory and issues no further copy, so the result is
    still the direct walk's, bit for bit, and the timeout is reported."""
    from newrecon_gb300.geometry import Geometry, view_angles
    from newrecon_gb300.native import NrError

    g = Geometry.dbt(96, 40, 24, 0.5, 1.0, 110, 46, 0.5, 6)
    angles = view_angles(6, 15.0)
    y, b = scan(mod, g, angles, 4)
    staged = plan_for(mod, g, angles, y, b, stage=True)
    direct = plan_for(mod, g, angles, y, b)
    x = torch.from_numpy(np.random.default_rng(2).random(g.n_voxels, dtype=np.float32)
                         * 0.05).cuda()
    for at in (0, 1, 3):
        expire(staged.ws, at)
        staged.project(x, 0)
        with pytest.raises(NrError) as e:
            staged.check()
        assert e.value.code == NR_ERR_TIMEOUT
        direct.project(x, 0)
        torch.cuda.synchronize()
        assert torch.equal(staged.section("h"), direct.section("h")), at
    staged.project(x, 1)
    assert staged.check() == 0


@pytest.mark.parametrize("dims", [(128, 40, 8, 1), (252, 40, 8, 1)], ids=["walk128", "dx3"])
def test_convolution_expiry_releases_tensor_memory(mod, dims):
    """The tensor-core convolutions (the 128-wide walk for nx = 128, the
    dx-stacked kernel for nx = 252): a tile wait that gives up flags the
    timeout, drains and releases TMEM; with the hook off the next forward
    pass on the same workspace is the reference's bit for bit.  Every CTA
    takes at least one run of 4 rows, so tiles 0 and 1 exist everywhere."""
    from newrecon_gb300 import native, warmstart
    from newrecon_gb300.native import NrError
    from oracle import cnn_oracle as co

    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.uniform(0.0, 0.1, size=int(np.prod(dims))).astype(np.float32)).cuda()
    net = warmstart.WarmStartCNN(co.init_params(3, last_scale=0.5), scale=20.0)
    ref = net.forward(x, dims).clone()
    net.check()
    _, ws = net._workspace(dims, False)
    for at in (0, 1):
        expire(ws, at)
        net.forward(x, dims)
        flags = ctypes.c_int32(0)
        with pytest.raises(NrError) as e:
            native.call("nr_cnn_check", ctypes.c_void_p(ws.data_ptr()), ctypes.byref(flags),
                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert e.value.code == NR_ERR_TIMEOUT and flags.value & 2
    expire(ws, -1)
    out = net.forward(x, dims)
    net.check()
    torch.cuda.synchronize()
    assert torch.equal(out, ref)


def test_weight_gradient_expiry_is_reported_and_recovers(mod):
    """The training pass (convolutions and the tensor-core weight gradient):
    with the hook on, the gradient's staging wait of K block 0 or 1 gives up,
    the block drains its MMAs and copies and releases TMEM; the check reports
    the timeout, and with the hook off the gradient on the same workspace is
    the first one's bit for bit."""
    from newrecon_gb300 import native, warmstart
    from newrecon_gb300.native import NrError
    from oracle import cnn_oracle as co

    dims = (160, 16, 8, 2)  # 512 row blocks: 3 or 4 per CTA
    rng = np.random.default_rng(6)
    n = int(np.prod(dims))
    x = torch.from_numpy(rng.uniform(0.0, 0.1, size=n).astype(np.float32)).cuda()
    t = (x + 0.01).contiguous()
    net = warmstart.WarmStartCNN(co.init_params(3, last_scale=0.5), scale=20.0)
    _, ref = net.loss_grad(x, t, dims)
    ref = ref.clone()
    net.check()
    _, ws = net._workspace(dims, True)
    for at in (0, 1):
        expire(ws, at)
        net.loss_grad(x, t, dims)
        flags = ctypes.c_int32(0)
        with pytest.raises(NrError) as e:
            native.call("nr_cnn_check", ctypes.c_void_p(ws.data_ptr()), ctypes.byref(flags),
                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert e.value.code == NR_ERR_TIMEOUT and flags.value & 2
    expire(ws, -1)
    _, g = net.loss_grad(x, t, dims)
    net.check()
    torch.cuda.synchronize()
    assert torch.equal(g, ref)
