"""FP64 numpy oracle of the learned WFF2 surrogate -- TEST INFRASTRUCTURE ONLY.

The surrogate has no counterpart in the reference project (which only has
the plain WFF2, ``WFT/WFT2_CPU.cpp:190-390``); this module restates the
network the CUDA library implements so that its forward pass and every
parameter gradient can be checked:

    a0  = relu(conv(x,  W0, b0, d0))       x = (Re z, Im z), 2 -> 32
    a_l = relu(conv(a_{l-1}, W_l, b_l, d_l))   l = 1..6, 32 -> 32
    y   = x + conv(a6, W7, b7, d7)          32 -> 2
    out = y / |y|
    loss = mean_p  min(s |t|, 1) |out - t/|t||^2   (s = 1 by default)

conv is a 3x3 convolution with dilation d and zero padding.  With
``bf16=True`` the oracle rounds (to nearest even) where the CUDA path stores
BF16: every weight, the activations a0..a6 and the gradients with respect
to the hidden pre-activations; sums stay FP64.  Only the tests use it.
"""
from __future__ import annotations

import numpy as np

LAYERS = 8
SIZES = [(32, 2)] + [(32, 32)] * 6 + [(2, 32)]  # (cout, cin)


def param_count() -> int:
    return sum(co * ci * 9 + co for co, ci in SIZES)


def bf16(a) -> np.ndarray:
    """Round float32 values to BF16 (nearest, ties to even); returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def unpack(params):
    """Flat FP32 vector -> list of (W [co][ci][3][3], b [co]) in FP64."""
    p = np.asarray(params, np.float64)
    out, off = [], 0
    for co, ci in SIZES:
        w = p[off:off + co * ci * 9].reshape(co, ci, 3, 3)
        off += co * ci * 9
        b = p[off:off + co]
        off += co
        out.append((w, b))
    return out


def pack(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in layers]).astype(np.float32)


def init_params(seed: int = 0, scale_last: float = 0.1) -> np.ndarray:
    """He-normal hidden layers, small last layer (the network starts near the identity)."""
    rng = np.random.default_rng(seed)
    layers = []
    for l, (co, ci) in enumerate(SIZES):
        std = np.sqrt(2.0 / (ci * 9))
        if l == LAYERS - 1:
            std *= scale_last
        layers.append((rng.normal(0, std, (co, ci, 3, 3)), np.zeros(co)))
    return pack(layers)


def _shift(x, dy, dx):
    """x [B,H,W,C] -> x[:, y+dy, x+dx] with zeros outside."""
    B, H, W, C = x.shape
    out = np.zeros_like(x)
    ys, yd = max(0, dy), max(0, -dy)
    xs, xd = max(0, dx), max(0, -dx)
    out[:, yd:H - ys, xd:W - xs] = x[:, ys:H - yd, xs:W - xd]
    return out


def conv(x, w, b, d):
    """x [B,H,W,ci], w [co][ci][3][3] -> [B,H,W,co]."""
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for ky in range(3):
        for kx in range(3):
            out += _shift(x, (ky - 1) * d, (kx - 1) * d) @ w[:, :, ky, kx].T
    return out + b


def conv_bwd_data(g, w, d):
    """d/dx of sum(g * conv(x, w)): g [B,H,W,co] -> [B,H,W,ci]."""
    out = np.zeros(g.shape[:3] + (w.shape[1],))
    for ky in range(3):
        for kx in range(3):
            out += _shift(g, -(ky - 1) * d, -(kx - 1) * d) @ w[:, :, ky, kx]
    return out


def conv_bwd_weight(g, x, d):
    """(dW [co][ci][3][3], db [co]) of sum(g * conv(x, w) + b)."""
    co, ci = g.shape[-1], x.shape[-1]
    dw = np.zeros((co, ci, 3, 3))
    g2 = g.reshape(-1, co)
    for ky in range(3):
        for kx in range(3):
            dw[:, :, ky, kx] = g2.T @ _shift(x, (ky - 1) * d, (kx - 1) * d).reshape(-1, ci)
    return dw, g2.sum(0)


def forward(params, z, dil, bf16_emul=True):
    """z complex [B,H,W] -> (out complex [B,H,W], cache)."""
    r = bf16 if bf16_emul else (lambda a: np.asarray(a, np.float64))
    layers = unpack(params)
    x = np.stack([np.real(z), np.imag(z)], -1).astype(np.float64)
    acts = []
    h = x
    for l in range(LAYERS - 1):
        w, b = layers[l]
        h = r(np.maximum(conv(h, r(w), b, dil[l]), 0.0))
        acts.append(h)
    w7, b7 = layers[-1]
    y = x + conv(h, r(w7), b7, dil[-1])
    n = np.sqrt((y ** 2).sum(-1, keepdims=True))
    out = y / np.where(n > 0, n, 1.0)
    return out[..., 0] + 1j * out[..., 1], dict(x=x, acts=acts, y=y, n=n, out=out)


def loss_and_grad(params, z, target, dil, bf16_emul=True, wscale=1.0):
    """(loss, flat gradient FP64) of the training loss (pixel weight
    min(wscale |target|, 1))."""
    r = bf16 if bf16_emul else (lambda a: np.asarray(a, np.float64))
    layers = unpack(params)
    _, c = forward(params, z, dil, bf16_emul)
    t = np.stack([np.real(target), np.imag(target)], -1).astype(np.float64)
    tn = np.sqrt((t ** 2).sum(-1, keepdims=True))
    wgt = np.minimum(wscale * tn, 1.0)
    tt = t / np.where(tn > 0, tn, 1.0)
    out, n = c["out"], c["n"]
    npix = out.shape[0] * out.shape[1] * out.shape[2]
    e = out - tt
    loss = float((wgt * e ** 2).sum() / npix)
    gout = 2.0 * wgt * e / npix
    dot = (out * gout).sum(-1, keepdims=True)
    gy = (gout - out * dot) / np.where(n > 0, n, np.inf)
    grads = [None] * LAYERS
    acts = c["acts"]
    w7 = r(layers[-1][0])
    grads[-1] = conv_bwd_weight(gy, acts[-1], dil[-1])
    g = r(conv_bwd_data(gy, w7, dil[-1]) * (acts[-1] > 0))
    for l in range(LAYERS - 2, 0, -1):
        grads[l] = conv_bwd_weight(g, acts[l - 1], dil[l])
        g = r(conv_bwd_data(g, r(layers[l][0]), dil[l]) * (acts[l - 1] > 0))
    grads[0] = conv_bwd_weight(g, c["x"], dil[0])
    return loss, np.concatenate([np.concatenate([dw.ravel(), db.ravel()]) for dw, db in grads])
