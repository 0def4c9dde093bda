"""CPU oracle of the learned Poisson warm-start network -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` imports this module, as the checker of the GPU network
(``iskra_gb300/csrc/lws.cu``: forward pass, loss and parameter gradients).
The reference has no learned part (its Poisson solve is the direct ``A\\b`` of
``FiniteDifferenceMethod/src/generalized_poisson.jl:372-378``); the network is
specified by this project: a 4-level encoder-decoder, 32 channels, bias-free
3x3 convolutions with zero padding, ReLU, 2x2 average pooling, nearest
upsampling with additive skips, a 1-channel FP32 output, mean squared error.

Arrays are images (H, W) = (ny, nx) with channels last.  The parameter vector
holds, in order: W0[tap][co] (1 -> 32), W1..W6[tap][co][ci] (32 -> 32),
W7[tap][ci] (32 -> 1); tap = 3 (dy + 1) + (dx + 1).

``bf16=True`` rounds to BF16 (round to nearest even) at the points where the
GPU stores BF16: the input, the weights, every activation, pooled and
upsampled tensor, and every activation gradient; sums are FP64 here (FP32 on
the GPU), so the two agree to about one BF16 rounding per stored value.
``bf16=False`` is exact FP64 arithmetic (finite-difference checks of the
backward pass).
"""
from __future__ import annotations

import numpy as np

C = 32
W1 = 9 * C
W32 = 9 * C * C
NPARAMS = 2 * W1 + 6 * W32


def layer_slices():
    off = [0, W1] + [W1 + k * W32 for k in range(1, 7)] + [NPARAMS]
    return [slice(off[i], off[i + 1]) for i in range(8)]


def bf16_round(a):
    """Round-to-nearest-even to BF16 (returned as float64)."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    sl = layer_slices()
    w0 = p[sl[0]].reshape(9, C)
    ws = [p[sl[k]].reshape(9, C, C) for k in range(1, 7)]
    w7 = p[sl[7]].reshape(9, C)
    return w0, ws, w7


def _pad(a):
    return np.pad(a, ((1, 1), (1, 1), (0, 0)))


def conv(a, w):
    """out[y,x,co] = sum_tap sum_ci a[y+dy, x+dx, ci] w[tap, co, ci] (zero padding)."""
    H, W, _ = a.shape
    ap = _pad(a)
    out = np.zeros((H, W, w.shape[1]))
    for t in range(9):
        dy, dx = divmod(t, 3)
        out += np.einsum("hwc,oc->hwo", ap[dy:dy + H, dx:dx + W], w[t], optimize=True)
    return out


def conv_dx(g, w):
    """Gradient w.r.t. the input of conv for output gradient g."""
    H, W, _ = g.shape
    dp = np.zeros((H + 2, W + 2, w.shape[2]))
    for t in range(9):
        dy, dx = divmod(t, 3)
        dp[dy:dy + H, dx:dx + W] += np.einsum("hwo,oc->hwc", g, w[t], optimize=True)
    return dp[1:H + 1, 1:W + 1]


def conv_dw(a, g):
    """dw[tap, co, ci] = sum_p g[p, co] a[p + off(tap), ci]."""
    H, W, _ = g.shape
    ap = _pad(a)
    return np.stack([np.einsum("hwo,hwc->oc", g, ap[t // 3:t // 3 + H, t % 3:t % 3 + W], optimize=True)
                     for t in range(9)])


def pool(a):
    return 0.25 * (a[0::2, 0::2] + a[1::2, 0::2] + a[0::2, 1::2] + a[1::2, 1::2])


def up(a):
    return np.repeat(np.repeat(a, 2, axis=0), 2, axis=1)


def up_bwd(g):
    return g[0::2, 0::2] + g[1::2, 0::2] + g[0::2, 1::2] + g[1::2, 1::2]


def forward(params, x, bf16=True):
    """Returns (y, cache) for the input image x (H, W)."""
    R = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    w0, ws, w7 = unpack(params)
    w0, w7 = R(w0), R(w7)
    ws = [R(w) for w in ws]
    x = R(x)[:, :, None]
    relu = lambda v: np.maximum(v, 0.0)
    a = [None] * 7
    p = [None] * 4
    u = [None] * 3
    a[0] = R(relu(conv(x, w0.reshape(9, C, 1))))
    for l in (1, 2, 3):
        p[l] = R(pool(a[l - 1]))
        a[l] = R(relu(conv(p[l], ws[l - 1])))
    for l in (2, 1, 0):
        li = 6 - l
        u[l] = R(up(a[li - 1]) + a[l])
        a[li] = R(relu(conv(u[l], ws[li - 1])))
    y = conv(a[6], w7.reshape(9, 1, C))[:, :, 0]
    return y, dict(x=x, a=a, p=p, u=u, w0=w0, ws=ws, w7=w7)


def loss_grad(params, x, target, bf16=True):
    """Mean squared error of forward(x) against target and its gradient."""
    R = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    y, k = forward(params, x, bf16)
    a, p, u, ws = k["a"], k["p"], k["u"], k["ws"]
    P = y.size
    d = y - np.asarray(target, dtype=np.float64)
    loss = float(np.sum(d * d) / P)
    dy = (2.0 * d / P)[:, :, None]
    g = [None] * 8
    dz = [None] * 7
    du = [None] * 3
    dp = [None] * 4
    g[7] = conv_dw(a[6], dy)[:, 0, :]
    dz[6] = R(conv_dx(dy, k["w7"].reshape(9, 1, C)) * (a[6] > 0))
    for l in (0, 1, 2):
        li = 6 - l
        du[l] = R(conv_dx(dz[li], ws[li - 1]))
        g[li] = conv_dw(u[l], dz[li])
        dz[li - 1] = R(up_bwd(du[l]) * (a[li - 1] > 0))
    for l in (3, 2, 1):
        dp[l] = R(conv_dx(dz[l], ws[l - 1]))
        g[l] = conv_dw(p[l], dz[l])
        dz[l - 1] = R((0.25 * up(dp[l]) + du[l - 1]) * (a[l - 1] > 0))
    g[0] = conv_dw(k["x"], dz[0])[:, :, 0]
    grad = np.concatenate([gi.ravel() for gi in g])
    return loss, grad, y
