"""numpy restatement of the learned-warm-start U-Net (forward and backward).

TEST INFRASTRUCTURE ONLY: the GPU network (osinco3d_gb300/csrc/o3d_unet_host.cu,
k_unet.cu) is checked against this.  The reference has no network; this
oracle restates the architecture and its exact parameter layout:

* tensors are channels-last arrays of shape (nz, ny, nx, C) (x fastest);
* a 3x3x3 convolution sums over taps t = (dz+1)*9 + (dy+1)*3 + (dx+1) of
  X[p + (dx, dy, dz)] @ W[t] with W[t] of shape (K, N); periodic axes wrap,
  the others read zeros;
* encoder level l: conv+ReLU twice (C_l = base * 2^l channels), 2x2x2 average
  pooling between levels; decoder: nearest upsampling, concatenation
  [upsampled, skip], conv+ReLU twice; head: 1x1 conv to one channel;
* flat FP32 parameter vector: per layer W ([27][K][N]) then b (N), in the
  order enc_a[0], enc_b[0], ..., enc_a[L-1], enc_b[L-1], dec_a[0], dec_b[0],
  ..., dec_a[L-2], dec_b[L-2], then head weights (C_0) and head bias.

With `bf16=True` weights, the packed input, every stored activation and
every stored activation gradient are rounded to BF16 where the GPU rounds
them, so the comparison isolates accumulation-order differences.
"""
from __future__ import annotations

import numpy as np


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


class Layout:
    def __init__(self, base: int, levels: int):
        self.base, self.levels = base, levels
        self.layers = {}
        off = 0

        def add(name, K, N):
            nonlocal off
            self.layers[name] = (off, off + 27 * K * N, K, N)
            off += 27 * K * N + N

        for l in range(levels):
            add(f"ea{l}", 16 if l == 0 else self.ch(l - 1), self.ch(l))
            add(f"eb{l}", self.ch(l), self.ch(l))
        for l in range(levels - 1):
            add(f"da{l}", 3 * self.ch(l), self.ch(l))
            add(f"db{l}", self.ch(l), self.ch(l))
        self.head_w = off
        off += self.ch(0)
        self.head_b = off
        off += 1
        self.n = off

    def ch(self, l: int) -> int:
        return self.base << l

    def get(self, params, name):
        w0, b0, K, N = self.layers[name]
        W = params[w0:w0 + 27 * K * N].reshape(27, K, N)
        b = params[b0:b0 + N]
        return W, b


def _shift(x, d, per):
    """x[p + d] along the three spatial axes (periodic wrap or zero fill)."""
    out = x
    for ax, (dd, pp) in enumerate(zip(d, per)):
        if dd == 0:
            continue
        axis = 2 - ax  # (x, y, z) -> array axes (2, 1, 0)
        rolled = np.roll(out, -dd, axis=axis)
        if not pp:
            idx = [slice(None)] * 4
            idx[axis] = slice(-1, None) if dd > 0 else slice(0, 1)
            rolled[tuple(idx)] = 0.0
        out = rolled
    return out


def _taps():
    for t in range(27):
        yield t, (t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1)


def conv(x, W, b, per):
    nz, ny, nx, K = x.shape
    y = np.zeros((nz, ny, nx, W.shape[2]))
    for t, d in _taps():
        y += (_shift(x, d, per).reshape(-1, K) @ W[t]).reshape(nz, ny, nx, -1)
    return y + (b if b is not None else 0.0)


def conv_back(x, W, dy, per):
    """Returns dX, dW, db of y = conv(x, W, b) given dy."""
    nz, ny, nx, K = x.shape
    dW = np.zeros_like(W)
    dx = np.zeros_like(x)
    dyf = dy.reshape(-1, dy.shape[-1])
    for t, d in _taps():
        xs = _shift(x, d, per).reshape(-1, K)
        dW[t] = xs.T @ dyf
        g = (dyf @ W[t].T).reshape(nz, ny, nx, K)
        dx += _shift(g, tuple(-e for e in d), per)
    return dx, dW, dyf.sum(axis=0)


def pool(x):
    nz, ny, nx, C = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, C).mean(axis=(1, 3, 5))


def pool_back(dy):
    return np.repeat(np.repeat(np.repeat(dy, 2, 0), 2, 1), 2, 2) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_back(dy):
    nz, ny, nx, C = dy.shape
    return dy.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, C).sum(axis=(1, 3, 5))


def forward_backward(params, inp, target, dims, per, base, levels, bf16_round=True):
    """inp: (in_ch, nvox) channel-major with x fastest; target: (nvox,).
    Returns (out (nvox,), loss, grad (n_params,))."""
    L = Layout(base, levels)
    R = bf16 if bf16_round else (lambda a: np.asarray(a, dtype=np.float64))
    nx, ny, nz = dims
    p = np.asarray(params, dtype=np.float64)
    Wq = {}
    for name in L.layers:
        W, b = L.get(p, name)
        Wq[name] = (R(W), b)
    x0 = np.zeros((nz, ny, nx, 16))
    for c in range(inp.shape[0]):
        x0[..., c] = inp[c].reshape(nz, ny, nx)
    x0 = R(x0)
    relu = lambda a: np.maximum(a, 0.0)
    ea, skip, pools, cat, da, d = {}, {}, {}, {}, {}, {}
    h = x0
    for l in range(levels):
        pools[l] = h
        ea[l] = R(relu(conv(h, *Wq[f"ea{l}"], per)))
        skip[l] = R(relu(conv(ea[l], *Wq[f"eb{l}"], per)))
        if l < levels - 1:
            h = R(pool(skip[l]))
    below = skip[levels - 1]
    for l in range(levels - 2, -1, -1):
        cat[l] = np.concatenate([up(below), skip[l]], axis=-1)
        da[l] = R(relu(conv(cat[l], *Wq[f"da{l}"], per)))
        d[l] = R(relu(conv(da[l], *Wq[f"db{l}"], per)))
        below = d[l]
    wh = p[L.head_w:L.head_w + L.ch(0)]
    bh = p[L.head_b]
    out = (d[0] @ wh + bh).reshape(-1)
    n = out.size
    diff = out - target
    loss = float(np.mean(diff * diff))
    dout = (2.0 * diff / n).reshape(nz, ny, nx)
    grad = np.zeros(L.n)

    def put(name, dW, db):
        w0, b0, K, N = L.layers[name]
        grad[w0:w0 + 27 * K * N] = dW.reshape(-1)
        grad[b0:b0 + N] = db

    grad[L.head_w:L.head_w + L.ch(0)] = (d[0].reshape(-1, L.ch(0)) * dout.reshape(-1, 1)).sum(axis=0)
    grad[L.head_b] = dout.sum()
    g = R(dout[..., None] * wh[None, None, None, :] * (d[0] > 0))
    gskip = {}
    for l in range(0, levels - 1):
        dx, dW, db = conv_back(da[l], Wq[f"db{l}"][0], g, per)
        put(f"db{l}", dW, db)
        gda = R(dx * (da[l] > 0))
        dx, dW, db = conv_back(cat[l], Wq[f"da{l}"][0], gda, per)
        put(f"da{l}", dW, db)
        gcat = R(dx * (cat[l] > 0))
        cu = L.ch(l + 1)
        gskip[l] = gcat[..., cu:]
        g = R(up_back(gcat[..., :cu]))
    gskip[levels - 1] = g
    gpool_next = None
    for l in range(levels - 1, -1, -1):
        gs = gskip[l]
        if l < levels - 1:
            gs = R(R(gs + pool_back(gpool_next)) * (skip[l] > 0))
        dx, dW, db = conv_back(ea[l], Wq[f"eb{l}"][0], gs, per)
        put(f"eb{l}", dW, db)
        gea = R(dx * (ea[l] > 0))
        dx, dW, db = conv_back(pools[l], Wq[f"ea{l}"][0], gea, per)
        put(f"ea{l}", dW, db)
        gpool_next = R(dx)
    return out, loss, grad
