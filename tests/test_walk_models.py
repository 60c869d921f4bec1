"""CPU models of the walking convolution's protocol and tile arithmetic (no GPU).

These restate, in Python, the index arithmetic of csrc/cnn.cu that the GPU
tests can only observe through their results:

* the row-set ring of ``conv32_walk_kernel`` / ``conv32_w3_kernel`` /
  ``wgrad_walk_kernel``: a producer loading row-sets in order into ``W_R``
  slots, an issuer reading row-sets i, i + 1, i + 2 for tile i of a run and
  releasing row-set i after it (and the run's last two after its last tile).
  An event simulation with random interleavings checks that every tile reads
  the rows it needs, that no slot is overwritten while still to be read, that
  every load is waited for and released exactly once, and that the protocol
  cannot deadlock;
* the dx-stacked tile of ``conv32_w3_kernel``: 126 outputs per 128-row tile,
  the weights of the three dx taps read as one N = 96 operand from the packed
  buffer (``bpk_index`` and the 512-byte row-group stride), and the output as
  D[r - 1][dx 0] + D[r][dx 1] + D[r + 1][dx 2] with the lane-quarter exchange,
  against a direct 3x3x3 convolution;
* the 32 -> 32 weight gradient of ``wgrad_walk_kernel`` (the tap's shift moved
  onto three gradient copies, two of them built by row shifts) against a direct
  weight gradient, and the BF16 hi/lo split of the 1-channel layers' FP32
  operands.
"""
import random

import numpy as np
import pytest

C = 32


def _ring_run(ny, nz, nb, xt, L, grid, cta, slots, seed):
    """One CTA's items of a walk plan, simulated with random interleaving."""
    nchunk = (ny + L - 1) // L
    nitems = nb * nz * xt * nchunk
    items = list(range(cta, nitems, grid))

    def pos(it):
        col, ch = divmod(it, nchunk)
        return col, ch * L, min(L, ny - ch * L)

    loads = []      # (item, input row Y) in load order
    tiles = []      # (item, [(load index, row)], released loads, first-use loads)
    G = 0
    for it in items:
        _, y0, ly = pos(it)
        loads += [(it, y0 - 1 + j) for j in range(ly + 2)]
        for i in range(ly):
            reads = [(G + i + dy, y0 + i + dy - 1) for dy in range(3)]
            rel = [G + i] + ([G + ly, G + ly + 1] if i == ly - 1 else [])
            first = [G + i + dy for dy in range(3) if i == 0 or dy == 2]
            tiles.append((it, reads, rel, first))
        G += ly + 2
    assert G == len(loads)
    assert sorted(r for t in tiles for r in t[2]) == list(range(len(loads)))
    rng = random.Random(seed)
    released, waited, slot_of = set(), set(), {}
    loaded = ti = 0
    while ti < len(tiles):
        can_load = loaded < len(loads) and (loaded < slots or (loaded - slots) in released)
        can_tile = all(g < loaded for g, _ in tiles[ti][1])
        assert can_load or can_tile, "deadlock"
        if can_load and (not can_tile or rng.random() < 0.5):
            slot_of[loaded % slots] = loaded
            loaded += 1
            continue
        it, reads, rel, first = tiles[ti]
        for g, row in reads:
            assert slot_of[g % slots] == g, "slot overwritten before its last read"
            assert loads[g] == (it, row), "wrong row"
            assert g not in released
        for g in first:
            assert g not in waited
            waited.add(g)
        released.update(rel)
        ti += 1
    assert waited == set(range(len(loads)))


@pytest.mark.parametrize("slots", [5, 6])
def test_row_set_ring_protocol(slots):
    for ny, nz, nb, xt in [(6, 5, 2, 1), (3, 4, 1, 2), (1, 1, 1, 1), (2, 3, 1, 1), (40, 8, 1, 2)]:
        for L in (1, 2, 4, 32):
            nitems = nb * nz * xt * ((ny + L - 1) // L)
            for grid in sorted({1, 3, min(nitems, 152)}):
                for cta in range(min(grid, 3)):
                    _ring_run(ny, nz, nb, xt, L, grid, cta, slots, seed=31 * cta + L)


def _bpk(n, k):
    """Element index of (row n, K k) in a packed 32-K operand (csrc/cnn.cu)."""
    return (n >> 3) * 256 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7)


def _shift(a, dz, dy, dx):
    out = np.zeros_like(a)
    nz, ny, nx = a.shape[1:4]
    zs = slice(max(0, -dz), nz - max(0, dz)); zd = slice(max(0, dz), nz + min(0, dz))
    ys = slice(max(0, -dy), ny - max(0, dy)); yd = slice(max(0, dy), ny + min(0, dy))
    xs = slice(max(0, -dx), nx - max(0, dx)); xd = slice(max(0, dx), nx + min(0, dx))
    out[:, zs, ys, xs] = a[:, zd, yd, xd]
    return out


@pytest.mark.parametrize("dims", [(20, 3, 3, 2), (130, 2, 2, 1), (252, 2, 1, 1), (126, 1, 2, 1)])
@pytest.mark.parametrize("nout", [32, 16])
def test_dx_stacked_tile_arithmetic(dims, nout):
    nx, ny, nz, nb = dims
    rng = np.random.default_rng(1)
    a = rng.standard_normal((nb, nz, ny, nx, C))
    W = rng.standard_normal((27, nout, C))               # [tap][o][i]
    pk = np.zeros(27 * nout * C)
    for t in range(27):
        for n in range(nout):
            for k in range(C):
                pk[t * nout * C + _bpk(n, k)] = W[t, n, k]
    out = np.zeros((nb, nz, ny, nx, nout))
    TW = 126
    for b in range(nb):
        for z in range(nz):
            for y in range(ny):
                for x0 in range(0, nx, TW):
                    D = np.zeros((128, 3 * nout))
                    for dz in range(3):
                        for dy in range(3):
                            zz, yy = z + dz - 1, y + dy - 1
                            strip = np.zeros((130, C))
                            if 0 <= zz < nz and 0 <= yy < ny:
                                lo, hi = max(x0 - 1, 0), min(x0 + 129, nx)
                                strip[lo - (x0 - 1):hi - (x0 - 1)] = a[b, zz, yy, lo:hi]
                            # N = 3 nout rows from tap (dz, dy, 0): SBO 512 B, LBO 128 B
                            base = (dz * 9 + dy * 3) * nout * C * 2
                            B = np.array([[pk[(base + (n >> 3) * 512 + (k >> 3) * 128 + (n & 7) * 16
                                               + (k & 7) * 2) // 2] for k in range(C)]
                                          for n in range(3 * nout)])
                            D += strip[:128] @ B.T
                    for wq in range(4):
                        for lane in range(32):
                            r, x = 32 * wq + lane, x0 - 1 + 32 * wq + lane
                            up = D[r - 1, :nout] if lane > 0 else (D[r - 1, :nout] if wq > 0 else 0)
                            dn = D[r + 1, 2 * nout:] if lane < 31 else (
                                D[r + 1, 2 * nout:] if wq < 3 else 0)
                            if 1 <= r <= TW and x < nx:
                                out[b, z, y, x] = (up + D[r, nout:2 * nout]) + dn
    ref = sum(_shift(a, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) @ W[t].T for t in range(27))
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_weight_gradient_shifted_copies():
    """``wgrad_walk_kernel``: per K block (128 voxels x0 .. x0 + 127 of a row)
    A = three copies of the gradient strip, copy c staged from x0 + 1 - c and
    built from the one strip loaded from x0 - 1 by shifting rows by 2 - c; B =
    the row-sets' strips (staged from x0 - 1, read from row 1); D[(c, o)][(dy,
    dz, i)] summed over K blocks is dW[9 dz + 3 dy + c][o][i]."""
    rng = np.random.default_rng(4)
    nb, nz, ny, nx = 2, 3, 4, 200
    a = rng.standard_normal((nb, nz, ny, nx, C))
    g = rng.standard_normal((nb, nz, ny, nx, C))

    def strip(t, b, z, y, x0):  # rows x0 - 1 .. x0 + 128, zero outside the patch
        s = np.zeros((130, C))
        if 0 <= z < nz and 0 <= y < ny:
            lo, hi = max(x0 - 1, 0), min(x0 + 129, nx)
            s[lo - (x0 - 1):hi - (x0 - 1)] = t[b, z, y, lo:hi]
        return s

    D = np.zeros((3, C, 3, 3, C))  # [c][o][dy][dz][i]
    for b in range(nb):
        for z in range(nz):
            for y in range(ny):
                for x0 in range(0, nx, 128):
                    g2 = strip(g, b, z, y, x0)                       # copy 2
                    copies = [g2[2 - c:2 - c + 128] for c in range(3)]  # rows r + 2 - c
                    for dy in range(3):
                        for dz in range(3):
                            s = strip(a, b, z + dz - 1, y + dy - 1, x0)[1:129]
                            for c in range(3):
                                D[c, :, dy, dz, :] += copies[c].T @ s
    ref = np.stack([np.einsum("bzyxo,bzyxi->oi", g, _shift(a, t // 9 - 1, (t // 3) % 3 - 1,
                                                            t % 3 - 1)) for t in range(27)])
    got = np.zeros_like(ref)
    for c in range(3):
        for dy in range(3):
            for dz in range(3):
                got[dz * 9 + dy * 3 + c] = D[c, :, dy, dz, :]
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_bf16_hi_lo_split():
    """The split operands of the 1-channel layers' weight gradients: hi =
    bf16(u), lo = bf16(u - hi) reproduces u to 2^-17 relative (round to nearest
    even, as __float2bfloat16_rn), and u - hi is exact in FP32."""
    def bf16(v):
        v = np.asarray(v, np.float32)
        u = v.view(np.uint32).astype(np.uint64)
        r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
        return r.astype(np.uint32).view(np.float32)

    rng = np.random.default_rng(5)
    u = (rng.standard_normal(1 << 16) * np.exp(rng.uniform(-20, 20, 1 << 16))).astype(np.float32)
    hi = bf16(u)
    d = (u - hi).astype(np.float32)
    assert np.array_equal(d.astype(np.float64), u.astype(np.float64) - hi.astype(np.float64))
    lo = bf16(d)
    err = np.abs((hi.astype(np.float64) + lo) - u) / np.abs(u)
    assert err.max() <= 2.0 ** -17
