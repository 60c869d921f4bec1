"""The warm-start CNN's tensor-core kernels against the FP64 NumPy reference.

The reference rounds to BF16 exactly where the GPU stores BF16 (weights,
scaled input, activations, back-propagated gradients), so the remaining
difference is FP32 accumulation order plus the odd BF16 rounding flip it
causes: relative L2 error <= 2e-3 for outputs, <= 1e-2 per layer gradient.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.fixture(scope="module")
def ws():
    from newrecon_gb300 import native, warmstart

    native.load()
    return warmstart


# (nx, ny, nz, nb): a partial x-tile, two x-tiles (one partial), one full tile,
# four x-tiles, and one row per plane (ny = 1: every row-set but the centre
# lies outside the patch) in three stacked patches of two planes.  The
# 32-channel layers run the dx-stacked kernel (126-wide tiles) for nx = 20,
# 150, 384 and 200 and the 128-wide walk for nx = 128.
DIMS = [(20, 6, 5, 2), (150, 3, 4, 1), (128, 4, 3, 1), (384, 8, 5, 1), (200, 1, 2, 3)]
DIM_IDS = ["partial", "two_tiles", "full_tile", "four_tiles", "one_row"]


def data(dims, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz, nb = dims
    x = rng.uniform(0.0, 0.1, size=(nb, nz, ny, nx)).astype(np.float32)
    t = (x + rng.normal(scale=0.01, size=x.shape)).astype(np.float32)
    return x, t


@pytest.mark.parametrize("dims", DIMS, ids=DIM_IDS)
def test_forward_matches_reference(ws, dims):
    from oracle import cnn_oracle as co

    p = co.init_params(3, last_scale=0.5)
    x, _ = data(dims, 1)
    net = ws.WarmStartCNN(p, scale=20.0)
    out = net.forward(torch.from_numpy(x.ravel()).cuda(), dims).cpu().numpy()
    net.check()
    f, _ = co.forward(p, x, 20.0, bf=True)
    ref = np.maximum(x + f / 20.0, 0.0)
    assert rel(out, ref.ravel()) < 2e-3
    # the residual itself (the network's contribution) to the same bar
    assert rel(out - x.ravel(), (ref - x).ravel()) < 2e-3


# 512 row blocks: every CTA of the tensor-core weight gradient accumulates 3 or 4
# of them in TMEM, through both halves of its double-buffered operands
MANY = (160, 16, 8, 2)


@pytest.mark.parametrize("dims", DIMS + [MANY], ids=DIM_IDS + ["many_blocks"])
def test_gradients_match_reference(ws, dims):
    from oracle import cnn_oracle as co

    p = co.init_params(4, last_scale=0.5)
    x, t = data(dims, 2)
    net = ws.WarmStartCNN(p, scale=20.0)
    loss, grad = net.loss_grad(torch.from_numpy(x.ravel()).cuda(),
                               torch.from_numpy(t.ravel()).cuda(), dims)
    net.check()
    grad = grad.cpu().numpy()
    lref, gref = co.loss_grad(p, x, t, 20.0, bf=True)
    assert abs(loss - lref) <= 2e-3 * abs(lref)
    wo, bo, P = co.param_offsets()
    for l in range(6):
        ni, no = co.LAYERS[l]
        sw = slice(wo[l], wo[l] + 27 * ni * no)
        sb = slice(bo[l], bo[l] + no)
        assert rel(grad[sw], gref[sw]) < 1e-2, ("W", l, rel(grad[sw], gref[sw]))
        assert rel(grad[sb], gref[sb]) < 1e-2, ("b", l, rel(grad[sb], gref[sb]))


def test_gradients_are_deterministic(ws):
    """A fixed grid, a fixed order of row blocks per CTA and a fixed-order
    reduction: the same inputs give the same gradient bit for bit."""
    from oracle import cnn_oracle as co

    x, t = data(MANY, 3)
    net = ws.WarmStartCNN(co.init_params(5, last_scale=0.5), scale=20.0)
    xd, td = torch.from_numpy(x.ravel()).cuda(), torch.from_numpy(t.ravel()).cuda()
    _, g1 = net.loss_grad(xd, td, MANY)
    g1 = g1.clone()
    _, g2 = net.loss_grad(xd, td, MANY)
    net.check()
    assert torch.equal(g1, g2)


def test_adam_matches_reference(ws):
    from oracle import cnn_oracle as co

    rng = np.random.default_rng(5)
    p = co.init_params(5, last_scale=1.0)
    net = ws.WarmStartCNN(p)
    pr, m, v = p.astype(np.float64), np.zeros(p.size), np.zeros(p.size)
    for step in range(1, 4):
        g = rng.normal(size=p.size).astype(np.float32)
        net.adam(torch.from_numpy(g).cuda(), lr=1e-3)
        pr, m, v = co.adam(pr, m, v, g.astype(np.float64), step, 1e-3)
    assert rel(net.state(), pr) < 1e-6


def test_training_reduces_loss(ws):
    """A few Adam steps on a fixed batch reduce the loss (end-to-end backward)."""
    dims = (128, 8, 6, 2)
    rng = np.random.default_rng(6)
    x = rng.uniform(0.02, 0.06, size=(2, 6, 8, 128)).astype(np.float32)
    t = (x * 1.3 + 0.005).astype(np.float32)  # a smooth, learnable residual
    net = ws.WarmStartCNN(seed=7)
    xt = torch.from_numpy(x.ravel()).cuda()
    tt = torch.from_numpy(t.ravel()).cuda()
    l0 = float(net.train_step(xt, tt, dims, lr=2e-3).item())
    for _ in range(30):
        net.train_step(xt, tt, dims, lr=2e-3)
    l1 = float(net.train_step(xt, tt, dims, lr=2e-3).item())
    net.check()
    assert l1 < 0.5 * l0, (l0, l1)
