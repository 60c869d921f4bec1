"""TEST INFRASTRUCTURE ONLY: FP64 NumPy reference of the warm-start CNN.

Forward, loss and analytic backward of the network in nr_cnn_* (six 3x3x3
convolutions 1 -> 32 x5 -> 1, ReLU, residual output), for gradient checks of
the GPU kernels.  With ``bf16=True`` the tensors the GPU stores in BF16
(weights, the scaled input, post-activations and back-propagated gradients)
are rounded to BF16 at the same points, so the remaining difference is FP32
accumulation order only; with ``bf16=False`` it is the exact FP64 network
(finite-difference checks).
"""
from __future__ import annotations

import numpy as np

LAYERS = [(1, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 1)]
TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def param_offsets():
    w, b, o = [], [], 0
    for ni, no in LAYERS:
        w.append(o)
        o += 27 * no * ni
        b.append(o)
        o += no
    return w, b, o


def unpack(params):
    wo, bo, _ = param_offsets()
    Ws, bs = [], []
    for l, (ni, no) in enumerate(LAYERS):
        Ws.append(params[wo[l]:wo[l] + 27 * no * ni].reshape(27, no, ni).astype(np.float64))
        bs.append(params[bo[l]:bo[l] + no].astype(np.float64))
    return Ws, bs


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def shift(a, dz, dy, dx):
    """out[b, z, y, x, ...] = a[b, z+dz, y+dy, x+dx, ...], zero outside each patch."""
    out = np.zeros_like(a)
    nz, ny, nx = a.shape[1:4]
    zs = slice(max(0, -dz), min(nz, nz - dz))
    ys = slice(max(0, -dy), min(ny, ny - dy))
    xs = slice(max(0, -dx), min(nx, nx - dx))
    zt = slice(max(0, dz), min(nz, nz + dz))
    yt = slice(max(0, dy), min(ny, ny + dy))
    xt = slice(max(0, dx), min(nx, nx + dx))
    out[:, zs, ys, xs] = a[:, zt, yt, xt]
    return out


def conv(a, W, b=None):
    """a [B, Z, Y, X, ni], W [27, no, ni] -> [B, Z, Y, X, no]."""
    out = 0.0
    for t, (dz, dy, dx) in enumerate(TAPS):
        out = out + np.einsum("bzyxi,oi->bzyxo", shift(a, dz, dy, dx), W[t])
    if b is not None:
        out = out + b
    return out


def forward(params, x, s, bf=True):
    """x [B, Z, Y, X]; returns f [B,Z,Y,X] (scaled residual) and the post-activations."""
    Ws, bs = unpack(params)
    q = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    Wq = [q(W) for W in Ws]
    a = q(s * x.astype(np.float64))[..., None]
    posts = [a]
    for l in range(5):
        a = q(np.maximum(conv(a, Wq[l], bs[l]), 0.0))
        posts.append(a)
    f = conv(a, Wq[5], bs[5])[..., 0]
    return f, posts


def loss_grad(params, x, target, s, bf=True):
    """Loss mean((f - s (target - x))^2) and its gradient (flat, like params)."""
    Ws, bs = unpack(params)
    q = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    Wq = [q(W) for W in Ws]
    f, posts = forward(params, x, s, bf)
    r = s * (target.astype(np.float64) - x.astype(np.float64))
    V = f.size
    loss = float(np.mean((f - r) ** 2))
    g = (2.0 * (f - r) / V)[..., None]  # dL/df, FP32 on the GPU
    if bf:
        g = g.astype(np.float32).astype(np.float64)
    gW = [None] * 6
    gb = [None] * 6
    for l in range(5, -1, -1):
        # the first layer's weight gradient reads the FP32 input volume (s x)
        a_in = (s * x.astype(np.float64))[..., None] if l == 0 else posts[l]
        gW[l] = np.stack([np.einsum("bzyxo,bzyxi->oi", g, shift(a_in, dz, dy, dx))
                          for (dz, dy, dx) in TAPS])
        gb[l] = g.sum(axis=(0, 1, 2, 3))
        if l == 0:
            break
        # input gradient: full correlation with the flipped taps, then the ReLU mask
        gi = q(g) if l == 5 else g  # the 1-channel gradient is gathered as BF16
        din = 0.0
        for t, (dz, dy, dx) in enumerate(TAPS):
            din = din + np.einsum("bzyxo,oi->bzyxi", shift(gi, -dz, -dy, -dx), Wq[l][t])
        g = q(din * (posts[l] > 0))
    wo, bo, P = param_offsets()
    out = np.zeros(P)
    for l in range(6):
        out[wo[l]:wo[l] + gW[l].size] = gW[l].ravel()
        out[bo[l]:bo[l] + gb[l].size] = gb[l]
    return loss, out


def init_params(seed: int, last_scale: float = 0.0) -> np.ndarray:
    """He-normal conv weights, zero biases, last layer scaled by last_scale."""
    rng = np.random.default_rng(seed)
    wo, bo, P = param_offsets()
    p = np.zeros(P, np.float32)
    for l, (ni, no) in enumerate(LAYERS):
        std = np.sqrt(2.0 / (27 * ni))
        w = rng.normal(scale=std, size=27 * no * ni)
        if l == 5:
            w = w * last_scale
        p[wo[l]:wo[l] + w.size] = w
    return p


def adam(p, m, v, g, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1 = 1 - b1 ** step
    c2 = 1 - b2 ** step
    p = p - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return p, m, v
